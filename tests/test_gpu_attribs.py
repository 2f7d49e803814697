"""Per-hit surface attributes (GetData, TraverseBVHStack.glsl:422-455) through the C ABI: the
IntersectRay overloads that return Albedo, Normal and Alpha beside TUVW, Mesh and TriangleIdx
(:458-502).  rq_closest_attribs and rq_hit_attribs against the oracle (its GetData is composed of
the restatement's normal, UV and albedo functions, which are pinned to the shader compiled as C++ by
tests/test_oracle_glsl_pin.py), bit for bit: textured and untextured meshes, emissive and
translucent entities under transforms, the IgnoreTransparent form, both BVH2 layouts and BVH8q,
device and host buffers, misses."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import assert_hits_identical, hits_from_device, mesh, rays_to_device

pytestmark = pytest.mark.gpu

ALBEDO = np.float32([[0.7, 0.6, 0.5], [0.2, 0.8, 0.4], [0.9, 0.9, 0.2], [0.3, 0.3, 0.3]])
MESH_TEX = [1, -1, 0]  # mesh 3 has no entry: ModelColor
ORC = {R.STACK: O.ORC_STACK, R.STACKLESS: O.ORC_STACKLESS}


def _textured(m, scale, mesh_mod):
    pos = m.positions().astype(np.float64)
    uv = np.stack([(pos[:, 0] + 1.0) * scale - 0.25, (pos[:, 1] + 1.0) * scale + 0.1], 1)
    mids = (np.arange(m.n_tris) % mesh_mod).astype(np.int32)
    return S.Mesh(S.with_texcoords(m.vertices, uv), m.indices, mids)


@pytest.fixture(scope="module", params=[R.STACK, R.STACKLESS])
def scene(ctx, request):
    layout = request.param
    ri = R.RayIntersector(layout)
    ri.add_object(1, [_textured(mesh("hf32"), 1.5, 3)])
    ri.add_object(2, [_textured(mesh("ico2"), 0.7, 4)])
    M = S.instance_transforms(5, (-2.0, -2.0, 0.2), (2.0, 2.0, 0.8), 0.5, 0.9, seed=9, tilt=0.2)
    ri.push_entity(1, emissive=0.25)
    for i, (em, tr) in enumerate(((0.5, 0.0), (2.0, 0.5), (0.0, 0.0), (1.0, 0.3), (0.0, 0.0))):
        ri.push_entity(2 if i % 2 == 0 else 1, model=M[i].astype(np.float64), emissive=em, translucency=tr)
    ri.buffer_entities()
    sc = ri.buffer_data(ctx)
    textures = [(S.noise_texture(64, 3), 1, 0), (S.noise_texture(17, 4), 0, 1)]
    sc.set_materials(ALBEDO)
    sc.set_textures(textures, MESH_TEX)
    osc = O.OracleScene(ORC[layout], *ri.global_buffers())
    rays = np.concatenate([S.camera_rays(96, 72, eye=(0.0, -5.0, 3.0), target=(0.0, 0.0, 0.3)),
                           S.sphere_rays(30_000, (-2.5, -2.5, -0.2), (2.5, 2.5, 1.5), seed=11)])
    yield layout, sc, osc, rays, textures
    sc.close()


@pytest.mark.parametrize("flags", [0, L.FLAG_IGNORE_TRANSPARENT, L.FLAG_REF_COMPAT])
def test_closest_attribs_bit_exact(scene, flags):
    layout, sc, osc, rays, textures = scene
    want_h = osc.closest(rays, flags=flags)
    want_a = osc.getdata(want_h, ALBEDO, textures, MESH_TEX)
    h, a = sc.closest_attribs(rays_to_device(rays), flags=flags)
    assert_hits_identical(hits_from_device(h), want_h, f"layout {layout} flags {flags}")
    np.testing.assert_array_equal(a.cpu().numpy().view(np.uint32), want_a.view(np.uint32))
    hit = want_h["t"] > 0
    assert 0.2 < hit.mean() < 0.95
    assert len(np.unique(want_a[hit, 7])) >= 3
    if not flags & L.FLAG_IGNORE_TRANSPARENT:
        assert len(np.unique(want_a[hit, 3])) >= 2  # translucent entities hit
    # host buffers: the same records
    hh, ah = sc.closest_attribs(rays, flags=flags)
    assert_hits_identical(hh, want_h, "host buffers")
    np.testing.assert_array_equal(ah.view(np.uint32), want_a.view(np.uint32))


def test_hit_attribs_over_given_hits_and_bvh8(scene):
    layout, sc, osc, rays, textures = scene
    want_h = osc.closest(rays)
    want_a = osc.getdata(want_h, ALBEDO, textures, MESH_TEX)
    got = sc.hit_attribs(rays_to_device(want_h)).cpu().numpy()
    np.testing.assert_array_equal(got.view(np.uint32), want_a.view(np.uint32))
    np.testing.assert_array_equal(sc.hit_attribs(want_h).view(np.uint32), want_a.view(np.uint32))
    if layout == R.STACK:
        sc.build_bvh8()
        h8, a8 = sc.closest_attribs(rays_to_device(rays), layout=L.LAYOUT_BVH8Q, block_size=128, min_blocks=7,
                                    persistent=1)
        h8 = hits_from_device(h8)
        same = np.ones(len(rays), bool)
        for f in ("t", "u", "v", "w", "tri", "mesh", "entity"):
            same &= h8[f].view(np.uint32) == want_h[f].view(np.uint32)
        assert same.mean() > 0.999
        np.testing.assert_array_equal(a8.cpu().numpy()[same].view(np.uint32), want_a[same].view(np.uint32))
    assert sc.ctx.device_status() == 0
