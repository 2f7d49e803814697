"""Specular reflection pass (SpecularTrace.glsl world-trace path) against the CPU restatement:
reflection rays, their hits, shadow rays and the lighting are bit-exact, so the output is equal
bit for bit (no transcendental beyond the shared turn-based sine / cosine)."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S
from candela_gb300.engine import specular_params

from .helpers import oracle_scene, rays_to_device, single_object

pytestmark = pytest.mark.gpu


def _oracle_pass(osc, rays, p, albedo, textures=None, mesh_texture=None, flags=0):
    ph = osc.closest(rays, flags=flags)
    sr = osc.spec_raygen(rays, ph, p.seed, p.roughness, p.ray_tmax, p.normal_mode)
    sh = osc.closest(sr, flags=flags)
    lit = None
    if p.shadow_rays:
        lit = 1 - osc.anyhit(osc.shadow_raygen(sr, sh, np.array(p.sun_dir), p.shadow_offset, p.normal_mode))
    return osc.spec_shade(sr, sh, lit, albedo, p.roughness, np.array(p.sun_color), np.array(p.sky_color),
                          np.array(p.ambient), textures=textures, mesh_texture=mesh_texture), sr, sh


@pytest.mark.parametrize("roughness,shadow,normal_mode", [(0.0, False, 0), (0.3, True, 0), (0.8, True, 1),
                                                          (0.011, False, 0)])
def test_specular_frame_bit_exact(ctx, roughness, shadow, normal_mode):
    bufs = single_object("ico2", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    albedo = np.float32([[0.7, 0.6, 0.5], [0.9, 0.3, 0.3], [0.3, 0.9, 0.3], [0.5, 0.5, 0.9]])
    sc.set_materials(albedo)
    rays = S.camera_rays(200, 150, eye=(0.0, -4.0, 2.5), target=(0.0, 0.0, 0.4))
    p = specular_params(seed=11, roughness=roughness, shadow_rays=shadow, normal_mode=normal_mode)
    want, sr, sh = _oracle_pass(osc, rays, p, albedo)
    got = sc.specular_frame(rays_to_device(rays), p).cpu().numpy()
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    active = sr["tmax"] > sr["tmin"]
    assert active.mean() > 0.3 and 0.05 < (sh["t"][active] > 0).mean() < 0.95
    # host buffers: the same output
    np.testing.assert_array_equal(sc.specular_frame(rays, p), got)


def test_specular_mirror_direction_and_textures(ctx):
    """Roughness 0 reflects the incident direction exactly (reflect(I, N)); textured hits take the
    texture's albedo."""
    m = S.heightfield(32, seed=5)
    pos = m.positions().astype(np.float64)
    verts = S.with_texcoords(m.vertices, np.stack([pos[:, 0] * 2.0, pos[:, 1] * 2.0], 1))
    b = R.build_bvh(verts, m.indices, m.mesh_ids, 0, layout=R.STACKLESS)
    bufs = (verts, b.tris, b.nodes, R.identity_entity(0, b.nodes.shape[0]))
    osc = oracle_scene(bufs, R.STACKLESS)
    sc = ctx.scene(R.STACKLESS, *bufs)
    albedo = np.float32([[0.6, 0.6, 0.6]])
    tex = [(S.noise_texture(32, 9), 1, 0)]
    sc.set_materials(albedo)
    sc.set_textures(tex, [0])
    rays = S.camera_rays(160, 120, **S.C1_CAMERA)
    p = specular_params(seed=2, roughness=0.0)
    want, sr, sh = _oracle_pass(osc, rays, p, albedo, tex, [0], flags=L.FLAG_REF_COMPAT)
    got = sc.specular_frame(rays_to_device(rays), p, flags=L.FLAG_REF_COMPAT).cpu().numpy()
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    # mirror: the reflected direction keeps its angle to the normal
    ph = osc.closest(rays)
    hit = (ph["t"] > 0) & (sr["tmax"] > 0)
    assert hit.mean() > 0.1
    d_in = rays["d"][hit] / np.linalg.norm(rays["d"][hit], axis=1, keepdims=True)
    d_out = sr["d"][hit]
    np.testing.assert_allclose(np.linalg.norm(d_out, axis=1), 1.0, atol=1e-5)
    assert (d_out[:, 2] > 0).mean() > 0.7 and (d_in[:, 2] < 0).all()
    # reflect(I, N): the bisector n of -I and the outgoing direction sees both at the same angle
    n = d_out - d_in
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    assert np.abs((d_in * n).sum(1) + (d_out * n).sum(1)).max() < 1e-4
