"""Radiance-probe update (UpdateRadianceProbes.glsl, rq_probe_update) against the CPU restatement:
probe rays, hits, shadow rays, shading, the bounce from the previous volume, SH encoding, temporal
blending and packing are bit-exact, so the packed SH volume, the raw radiance and the depth-moment
map are equal bit for bit, frame after frame."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300.engine import probe_params, probe_volumes
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import mesh

pytestmark = pytest.mark.gpu

MODEL = np.float32([[0.7, 0.6, 0.5], [0.3, 0.8, 0.4]])


def _scene(layout):
    ri = R.RayIntersector(layout)
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    M = S.instance_transforms(6, (-1.5, -1.5, 0.1), (1.5, 1.5, 0.6), 0.4, 0.8, seed=12, tilt=0.1)
    ri.push_entity(1)
    for i in range(6):
        ri.push_entity(2, model=M[i].astype(np.float64), emissive=0.3 if i == 2 else 0.0)
    ri.buffer_entities()
    return ri.global_buffers()


def _frames(grid=(16, 8, 12), temporal=(True, True, False), shadow=True, normal_mode=0):
    origins = [(0.0, 0.0, 0.6), (0.13, -0.07, 0.62), (0.3, 0.05, 0.55)]
    prev = origins[0]
    for k, org in enumerate(origins):
        yield probe_params(grid=grid, origin=org, prev_origin=prev, size=(2.0, 1.0, 1.6), seed=5 + k,
                           temporal=temporal[k], shadow_rays=shadow, normal_mode=normal_mode,
                           sky_color=(0.4, 0.55, 0.9))
        prev = org


def _torch_volumes(sh, raw, pmap):
    import torch
    return (torch.from_numpy(sh.view(np.int32).copy()).cuda(), torch.from_numpy(raw.copy()).cuda(),
            torch.from_numpy(pmap.copy()).cuda())


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
@pytest.mark.parametrize("shadow,normal_mode", [(True, 0), (False, 1)])
def test_probe_update_bit_exact(ctx, layout, shadow, normal_mode):
    v, t, n, e = _scene(layout)
    osc = O.OracleScene(O.ORC_STACK if layout == R.STACK else O.ORC_STACKLESS, v, t, n, e)
    sc = ctx.scene(layout, v, t, n, e)
    sc.set_materials(MODEL)
    frames = list(_frames(shadow=shadow, normal_mode=normal_mode))
    sh, raw, pmap = probe_volumes(frames[0])
    d_sh, d_raw, d_map = _torch_volumes(sh, raw, pmap)
    for k, p in enumerate(frames):
        want_sh, want_raw, want_map, rays, hits = osc.probe_update(p, MODEL, sh, raw, pmap)
        got_sh, got_raw = sc.probe_update(p, d_sh, d_raw, d_map)
        np.testing.assert_array_equal(got_sh.cpu().numpy().view(np.uint32), want_sh, err_msg=f"frame {k} sh")
        np.testing.assert_array_equal(got_raw.cpu().numpy().view(np.uint32), want_raw.view(np.uint32),
                                      err_msg=f"frame {k} raw")
        np.testing.assert_array_equal(d_map.cpu().numpy().view(np.uint32), want_map.view(np.uint32),
                                      err_msg=f"frame {k} map")
        sh, raw, pmap = want_sh, want_raw, want_map
        d_sh, d_raw = got_sh, got_raw
        hit = hits["t"] > 0
        assert 0.2 < hit.mean() < 0.95
    assert (sh[:, 7] > 0).mean() > 0.5 and (np.abs(raw[:, :3]).sum(1) > 0).mean() > 0.5


def test_probe_update_host_buffers_and_bvh8(ctx):
    """Host buffers give the device result; the BVH8 layout gives the strict hits, so the same
    volume (single object: no instance whose slab test could lose a hit)."""
    import torch
    bufs = _single()
    osc = O.OracleScene(O.ORC_STACK, *bufs)
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(MODEL)
    sc.build_bvh8()
    p = next(_frames(grid=(24, 8, 24)))
    sh, raw, pmap = probe_volumes(p)
    want_sh, want_raw, want_map, rays, hits = osc.probe_update(p, MODEL, sh, raw, pmap)
    for layout in (R.STACK, L.LAYOUT_BVH8Q):
        hmap = pmap.copy()
        h_sh, h_raw = sc.probe_update(p, sh, raw, hmap, layout=layout)
        np.testing.assert_array_equal(h_sh, want_sh)
        np.testing.assert_array_equal(h_raw.view(np.uint32), want_raw.view(np.uint32))
        np.testing.assert_array_equal(hmap.view(np.uint32), want_map.view(np.uint32))
        d_sh, d_raw, d_map = _torch_volumes(sh, raw, pmap)
        g_sh, g_raw = sc.probe_update(p, d_sh, d_raw, d_map, layout=layout)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(g_sh.cpu().numpy().view(np.uint32), want_sh)
    assert 0.1 < (hits["t"] > 0).mean() < 0.95


def _single():
    from .helpers import single_object
    return single_object("ico2", R.STACK)


def test_probe_update_rejects_bad_arguments(ctx):
    v, t, n, e = _scene(R.STACK)
    sc = ctx.scene(R.STACK, v, t, n, e)
    p = probe_params(grid=(4, 4, 4))
    sh, raw, pmap = probe_volumes(p)
    for bad in ((0, 4, 4), (4, -1, 4), (5000, 1, 1)):
        q = probe_params(grid=bad)
        with pytest.raises(R.RqError):
            sc.probe_update(q, sh, raw, pmap, out_sh=sh.copy(), out_raw=raw.copy())
    d_sh, d_raw, d_map = _torch_volumes(sh, raw, pmap)
    with pytest.raises(R.RqError):                       # output volume aliasing the previous one
        sc.probe_update(p, d_sh, d_raw, d_map, out_sh=d_sh)


@pytest.mark.parametrize("flags", [0, L.FLAG_REF_COMPAT])
def test_probe_update_textures_and_ref_compat(ctx, flags):
    """Textured albedo (a repeat and a clamped sRGB texture over a heightfield with texture
    coordinates) and the reference's conventions (RQ_FLAG_REF_COMPAT: a hit on global triangle 0
    reads as a miss, and the raw radiance is held as the reference's r11f_g11f_b10f images hold it,
    which the next frame's temporal blend reads): the volume equals the oracle's bit for bit."""
    m = S.heightfield(48, seed=8)
    pos = m.positions().astype(np.float64)
    verts = S.with_texcoords(m.vertices, np.stack([pos[:, 0] * 1.5 + 0.2, pos[:, 1] * -1.3], 1))
    mids = (np.arange(m.n_tris) % 3).astype(np.int32)
    b = R.build_bvh(verts, m.indices, mids, 0, layout=R.STACK)
    ents = R.identity_entity(0, b.nodes.shape[0], emissive=0.1)
    osc = O.OracleScene(O.ORC_STACK, verts, b.tris, b.nodes, ents)
    sc = ctx.scene(R.STACK, verts, b.tris, b.nodes, ents)
    albedo = np.float32([[0.6, 0.5, 0.4], [0.3, 0.7, 0.3], [0.8, 0.8, 0.2]])
    tex = [(S.noise_texture(32, 3), 0, 0), (S.noise_texture(16, 4), 1, 1)]
    mesh_tex = [0, -1, 1]
    sc.set_materials(albedo)
    sc.set_textures(tex, mesh_tex)
    sh, raw, pmap = probe_volumes(probe_params(grid=(12, 12, 6)))
    d_sh, d_raw, d_map = _torch_volumes(sh, raw, pmap)
    frames = [probe_params(grid=(12, 12, 6), origin=org, prev_origin=prev, size=(1.0, 1.0, 0.4), seed=3 + k,
                           sky_color=(0.4, 0.55, 0.9))
              for k, (org, prev) in enumerate([((0.0, 0.0, 0.3), (0.0, 0.0, 0.3)),
                                               ((0.05, -0.04, 0.31), (0.0, 0.0, 0.3))])]
    for k, p in enumerate(frames):
        want_sh, want_raw, want_map, rays, hits = osc.probe_update(p, albedo, sh, raw, pmap, flags=flags,
                                                                   textures=tex, mesh_texture=mesh_tex)
        got_sh, got_raw = sc.probe_update(p, d_sh, d_raw, d_map, flags=flags)
        np.testing.assert_array_equal(got_sh.cpu().numpy().view(np.uint32), want_sh, err_msg=f"frame {k} sh")
        np.testing.assert_array_equal(got_raw.cpu().numpy().view(np.uint32), want_raw.view(np.uint32))
        np.testing.assert_array_equal(d_map.cpu().numpy().view(np.uint32), want_map.view(np.uint32))
        r11 = np.vectorize(lambda x, mb: O.small_ufloat(float(x), mb), otypes=[np.float32])
        packed = np.stack([r11(want_raw[:, 0], 6), r11(want_raw[:, 1], 6), r11(want_raw[:, 2], 5)], 1)
        if flags & L.FLAG_REF_COMPAT:  # every value representable in the packed format
            np.testing.assert_array_equal(packed.view(np.uint32), want_raw[:, :3].view(np.uint32))
        else:  # float32 keeps more than the packed format
            assert (packed != want_raw[:, :3]).any()
        sh, raw, pmap = want_sh, want_raw, want_map
        d_sh, d_raw = got_sh, got_raw
        assert 0.2 < (hits["t"] > 0).mean() < 0.95
