"""Diffuse-GI / RTAO pass on the GPU against the CPU restatement: ray generation bit-exact,
secondary hits bit-exact, shading within 2e-6 relative (pow is the only non-exact operation)."""
import numpy as np
import pytest

import candela_gb300 as R
from oracle import oracle as O
from candela_gb300 import scenes as S
from candela_gb300.engine import gi_params

from .helpers import (assert_hits_identical, hits_from_device, oracle_scene, rays_to_device,
                      single_object)

pytestmark = pytest.mark.gpu

SHADE_RTOL = 2e-6


def _rays_from_device(t):
    return t.cpu().numpy().view(R.RAY_DTYPE)


@pytest.mark.parametrize("spp,normal_mode", [(1, 0), (4, 0), (2, 1)])
def test_gi_raygen_bit_exact(ctx, spp, normal_mode):
    bufs = single_object("c1", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    rays = S.camera_rays(256, 256, **S.C1_CAMERA)
    hits = osc.closest(rays)
    sc = ctx.scene(R.STACK, *bufs)
    p = gi_params(spp=spp, seed=1234, origin_offset=1e-3, normal_mode=normal_mode)
    d_hits = rays_to_device(hits)
    got = _rays_from_device(sc.gi_raygen(rays_to_device(rays), d_hits, p))
    want = osc.gi_raygen(rays, hits, spp, 1234, 1e-3, 1000000.0, normal_mode)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert (want["tmax"] > 0).sum() == spp * (hits["t"] > 0).sum()


def test_gi_frame_matches_oracle_pipeline(ctx):
    bufs = single_object("hf64", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    rays = S.camera_rays(160, 120, **S.C1_CAMERA)
    albedo = np.array([[0.7, 0.6, 0.5]], dtype=np.float32)
    p = gi_params(spp=4, seed=99, origin_offset=1e-3, shadow_rays=True, shadow_offset=1e-3)
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(albedo)
    # oracle pipeline
    ph = osc.closest(rays)
    sec = osc.gi_raygen(rays, ph, 4, 99, 1e-3)
    sh = osc.closest(sec)
    shadow = osc.shadow_raygen(sec, sh, np.array(p.sun_dir), 1e-3)
    lit = 1 - osc.anyhit(shadow)
    shaded = osc.shade(sec, sh, lit, albedo, np.array(p.sun_dir), np.array(p.sun_color),
                       np.array(p.sky_color))
    want = shaded.reshape(-1, 4, 4).sum(1) * np.float32(0.25)
    # GPU, device buffers
    got_dev, st = sc.gi_frame(rays_to_device(rays), p, stats=True)
    got = got_dev.cpu().numpy()
    np.testing.assert_allclose(got, want, rtol=SHADE_RTOL * 4, atol=1e-6)
    assert st["primary_hits"] == (ph["t"] > 0).sum()
    assert st["secondary_rays"] == (sec["tmax"] > 0).sum()
    assert st["secondary_hits"] == (sh["t"] > 0).sum()
    assert st["shadow_rays"] == (shadow["tmax"] > 0).sum()
    # GPU, host buffers: identical to the device path
    got_host = sc.gi_frame(rays, p)
    np.testing.assert_array_equal(got_host, got)


def test_secondary_hits_and_shading(ctx):
    bufs = single_object("ico2", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    rays = S.camera_rays(200, 150, eye=(0.0, -4.0, 2.0), target=(0.0, 0.0, 0.3))
    ph = osc.closest(rays)
    sec = osc.gi_raygen(rays, ph, 2, 5, 0.05)
    sc = ctx.scene(R.STACK, *bufs)
    albedo = np.random.default_rng(0).uniform(0.2, 0.9, (7, 3)).astype(np.float32)
    sc.set_materials(albedo)
    d_sec = rays_to_device(sec)
    sh_gpu = sc.closest(d_sec)
    assert_hits_identical(hits_from_device(sh_gpu), osc.closest(sec), "secondary")
    p = gi_params(spp=2, seed=5, origin_offset=0.05)
    got = sc.shade(d_sec, sh_gpu, p).cpu().numpy()
    want = osc.shade(sec, osc.closest(sec), None, albedo, np.array(p.sun_dir),
                     np.array(p.sun_color), np.array(p.sky_color))
    np.testing.assert_allclose(got, want, rtol=SHADE_RTOL, atol=1e-7)


def test_rtao_frame(ctx):
    """RTAO: one AO any-hit ray per pixel (tmax 0.25); visibility = fraction unoccluded."""
    bufs = single_object("c1", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    rays = S.camera_rays(256, 256, **S.C1_CAMERA)
    p = gi_params(spp=1, seed=7, origin_offset=1e-3, ray_tmax=0.25, query=1)
    sc = ctx.scene(R.STACK, *bufs)
    got = sc.gi_frame(rays_to_device(rays), p).cpu().numpy()
    ph = osc.closest(rays)
    ao = osc.gi_raygen(rays, ph, 1, 7, 1e-3, 0.25)
    occ = osc.anyhit(ao)
    vis = np.where(ao["tmax"] > 0, 1.0 - occ, 0.0).astype(np.float32)
    np.testing.assert_array_equal(got[:, 3], vis)


@pytest.mark.parametrize("query", [0, 1])
def test_gi_frame_forms_identical(ctx, query):
    """The GI/RTAO frame gives the same pixels bit for bit on every traversal form: strict BVH2,
    BVH8q one thread per ray, BVH8q persistent ray queue, with and without octant binning, with
    per-pixel or per-sample ray generation and shading."""
    from candela_gb300 import _lib as L
    bufs = single_object("hf64", R.STACK)
    rays = rays_to_device(S.camera_rays(192, 160, **S.C1_CAMERA))
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(np.array([[0.7, 0.6, 0.5]], dtype=np.float32))
    sc.build_bvh8()
    kw = dict(spp=3, seed=11, origin_offset=1e-3, shadow_rays=True, shadow_offset=1e-3)
    if query == 1:
        kw = dict(spp=2, seed=11, origin_offset=1e-3, ray_tmax=0.25, query=1)
    want, st = sc.gi_frame(rays, gi_params(**kw), stats=True)
    want = want.cpu().numpy()
    assert st["secondary_rays"] > 1000
    for sort in (False, True):
        for unfused in (False, True):
            p = gi_params(sort_rays=sort, unfused=unfused, **kw)
            for launch in (dict(block_size=128, min_blocks=8), dict(block_size=128, min_blocks=7, persistent=1),
                           dict(block_size=128, min_blocks=1, persistent=1)):
                got, st2 = sc.gi_frame(rays, p, layout=L.LAYOUT_BVH8Q, stats=True, **launch)
                got = got.cpu().numpy()
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (sort, unfused, launch)
                assert st2 == st, (sort, unfused, launch)
    assert ctx.device_status() == 0


@pytest.mark.parametrize("query", [0, 1])
def test_gi_frame_per_pixel_host_buffers_and_ref_compat(ctx, query):
    """The per-pixel ray generation and shading kernels, through host buffers and with
    RQ_FLAG_REF_COMPAT (a hit on triangle 0 shades as a miss), equal the per-sample kernels, and
    the ray counts equal the oracle pipeline's."""
    from candela_gb300 import _lib as L
    bufs = single_object("ico2", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    rays = S.camera_rays(160, 128, eye=(0.0, -4.0, 2.0), target=(0.0, 0.0, 0.3))
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(np.random.default_rng(1).uniform(0.2, 0.9, (7, 3)).astype(np.float32))
    sc.build_bvh8()
    kw = dict(spp=2, seed=3, origin_offset=0.05)
    if query == 1:
        kw.update(ray_tmax=0.5, query=1)
    for flags in (0, L.FLAG_REF_COMPAT):
        want, st = sc.gi_frame(rays_to_device(rays), gi_params(unfused=True, **kw), layout=L.LAYOUT_BVH8Q,
                               flags=flags, stats=True)
        got_host = sc.gi_frame(rays, gi_params(**kw), layout=L.LAYOUT_BVH8Q, flags=flags)
        np.testing.assert_array_equal(got_host.view(np.uint32), want.cpu().numpy().view(np.uint32))
        # pinned host rays: the primary launch reads them over the host link and leaves the device
        # copy the later kernels read; the pixels are the same
        import torch
        pinned = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory().numpy().view(R.RAY_DTYPE)
        pinned_out = torch.empty((len(rays), 4), dtype=torch.float32).pin_memory().numpy()
        sc.gi_frame(pinned, gi_params(**kw), out=pinned_out, layout=L.LAYOUT_BVH8Q, flags=flags)
        np.testing.assert_array_equal(pinned_out.view(np.uint32), want.cpu().numpy().view(np.uint32))
    ph = osc.closest(rays)
    sec = osc.gi_raygen(rays, ph, kw["spp"], kw["seed"], kw["origin_offset"], kw.get("ray_tmax", 1e6))
    _, st = sc.gi_frame(rays_to_device(rays), gi_params(**kw), layout=L.LAYOUT_BVH8Q, stats=True)
    assert st["primary_hits"] == (ph["t"] > 0).sum()
    assert st["secondary_rays"] == (sec["tmax"] > 0).sum()
    want_sec = (osc.anyhit(sec) != 0).sum() if query == 1 else (osc.closest(sec)["t"] > 0).sum()
    assert st["secondary_hits"] == want_sec
    assert ctx.device_status() == 0


@pytest.mark.parametrize("query", [0, 1])
def test_gi_frame_host_chunks_equal_device_pass(ctx, query):
    """A host-buffer frame of several shading chunks (pixels copied out chunk by chunk while the
    next chunk is shaded) gives the pixels and ray counts of the device-buffer pass, bit for bit."""
    from candela_gb300 import _lib as L
    bufs = single_object("hf64", R.STACK)
    rays = S.camera_rays(1280, 1024, **S.C1_CAMERA)
    assert len(rays) > 4 * (1 << 18)
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(np.array([[0.7, 0.6, 0.5]], dtype=np.float32))
    sc.build_bvh8()
    kw = dict(spp=2, seed=21, origin_offset=1e-3)
    if query == 1:
        kw.update(ray_tmax=0.25, query=1)
    p = gi_params(**kw)
    for layout in (R.STACK, L.LAYOUT_BVH8Q):
        want, st = sc.gi_frame(rays_to_device(rays), p, layout=layout, stats=True)
        got, st_h = sc.gi_frame(rays, p, layout=layout, stats=True)
        np.testing.assert_array_equal(got.view(np.uint32), want.cpu().numpy().view(np.uint32))
        assert st_h == st
    assert ctx.device_status() == 0


def _oracle_bounce_pass(osc, rays, p, albedo, bounces, ref_miss, flags=0, textures=None,
                        mesh_texture=None, albedo_of=None):
    """The GI pass with the RT second-bounce loop, composed from the oracle's pieces: rays, hits and
    shading per bounce, then the loop's accumulation (FinalRadiance + Bounced,
    oracle.bounce_accumulate, pinned to the shader's loop) and the per-pixel mean."""
    f = np.float32
    spp, seed = p.spp, p.seed
    sd, sc_, sky = np.array(p.sun_dir), np.array(p.sun_color), np.array(p.sky_color, np.float32)
    ph = osc.closest(rays, flags=flags)
    sec = osc.gi_raygen(rays, ph, spp, seed, p.origin_offset)
    sh = osc.closest(sec, flags=flags)
    lit = 1 - osc.anyhit(osc.shadow_raygen(sec, sh, sd, p.shadow_offset)) if p.shadow_rays else None
    tex = dict(textures=textures, mesh_texture=mesh_texture)
    rad = osc.shade(sec, sh, lit, albedo, sd, sc_, sky, **tex).astype(np.float32)
    alb_of = albedo_of or (lambda hits: osc.hit_albedo(hits, albedo))  # noqa: E731
    emissive = osc.entities["data"][:, 0].view(np.float32)
    alive = sh["t"] > 0
    thr0 = np.where(alive[:, None], alb_of(sh), f(0)).astype(np.float32)
    inputs = np.zeros((len(sec), max(bounces, 1), 12), dtype=np.float32)
    inputs[:, :, 0] = -1.0
    prev_r, prev_h = sec, sh
    sid = np.arange(len(sec), dtype=np.uint32)
    bflags = flags & ~R.engine.L.FLAG_IGNORE_TRANSPARENT
    n_rays = n_hits = 0
    for b in range(bounces):
        br = osc.bounce_raygen(prev_r, prev_h, alive, sid, seed, b, 0.02, p.ray_tmax)
        bh = osc.closest(br, flags=bflags)
        blit = (1 - osc.anyhit(osc.shadow_raygen(br, bh, sd, p.shadow_offset))) if p.shadow_rays \
            else np.ones(len(br), np.uint8)
        hit = alive & (bh["t"] > 0)
        n_rays += int(alive.sum())
        n_hits += int(hit.sum())
        x = inputs[:, b]
        x[hit, 0] = bh["t"][hit]
        x[hit, 1:4] = alb_of(bh[hit])
        x[hit, 4] = emissive[bh["entity"][hit]]
        x[hit, 5:8] = osc.hit_normal(bh[hit], p.normal_mode)
        x[hit, 8:11] = br["d"][hit]
        x[hit, 11] = blit[hit]
        alive = hit
        prev_r, prev_h = br, bh
    if bounces:
        rad[:, :3] = O.bounce_accumulate(rad[:, :3], thr0, inputs[:, :bounces], sd, sc_, sky, ref_miss)
    rad = np.where((sec["tmax"] > sec["tmin"])[:, None], rad, f(0))
    acc = np.zeros((len(rays), 4), np.float32)
    r3 = rad.reshape(len(rays), spp, 4)
    for k in range(spp):
        acc = acc + r3[:, k]
    return acc * (f(1) / f(spp)), n_rays, n_hits


@pytest.mark.parametrize("bounces,shadow,ref", [(1, False, False), (3, True, False), (2, True, True)])
def test_gi_frame_bounces_match_oracle_pipeline(ctx, bounces, shadow, ref):
    """The RT second-bounce loop: bounce rays, hits and shadow rays bit-exact through the oracle's
    pieces; radiance bit for bit (the loop's accumulation is pinned to the shader), AO within the
    shading tolerance (its pow); ray counts equal."""
    from candela_gb300 import _lib as L
    bufs = single_object("ico2", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    rays = S.camera_rays(160, 120, eye=(0.0, -4.0, 2.5), target=(0.0, 0.0, 0.4))
    albedo = np.array([[0.7, 0.6, 0.5], [0.9, 0.3, 0.3], [0.3, 0.9, 0.3], [0.5, 0.5, 0.9]], dtype=np.float32)
    p = gi_params(spp=2, seed=7, origin_offset=1e-3, shadow_rays=shadow, bounces=bounces)
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(albedo)
    flags = L.FLAG_REF_COMPAT if ref else 0
    want, n_rays, n_hits = _oracle_bounce_pass(osc, rays, p, albedo, bounces, ref, flags)
    got_dev, st = sc.gi_frame(rays_to_device(rays), p, flags=flags, stats=True)
    got = got_dev.cpu().numpy()
    np.testing.assert_array_equal(got[:, :3].view(np.uint32), want[:, :3].view(np.uint32))
    np.testing.assert_allclose(got[:, 3], want[:, 3], rtol=SHADE_RTOL * 8, atol=1e-6)
    assert st["bounce_rays"] == n_rays and st["bounce_hits"] == n_hits and n_hits > 0
    # the bounces add light: compared with the same pass without them
    p0 = gi_params(spp=2, seed=7, origin_offset=1e-3, shadow_rays=shadow)
    base = sc.gi_frame(rays_to_device(rays), p0, flags=flags).cpu().numpy()
    assert (got[:, :3] >= base[:, :3] - 1e-6).all() and got[:, :3].sum() > base[:, :3].sum()
    np.testing.assert_array_equal(got[:, 3], base[:, 3])  # AO is the first bounce's
    # host buffers give the same pixels
    np.testing.assert_array_equal(sc.gi_frame(rays, p, flags=flags), got)


@pytest.mark.parametrize("srgb,wrap", [(0, 0), (1, 0), (1, 1)])
def test_textured_shading_matches_oracle(ctx, srgb, wrap):
    """GetData's albedo texture: UV from the half-packed texture coordinates, bilinear level-0
    sample; the shaded colour equals the oracle's bit for bit (AO within the pow tolerance),
    also through the bounce loop's throughput."""
    m = S.heightfield(32, seed=5)
    pos = m.positions().astype(np.float64)
    uv = np.stack([(pos[:, 0] + 1.0) * 1.5 - 0.25, (pos[:, 1] + 1.0) * 1.5 + 0.1], 1)  # outside [0, 1] too
    verts = S.with_texcoords(m.vertices, uv)
    mids = (np.arange(m.n_tris) % 3).astype(np.int32)       # three meshes, two textured
    b = R.build_bvh(verts, m.indices, mids, 0, layout=R.STACK)
    bufs = (verts, b.tris, b.nodes, R.identity_entity(0, b.nodes.shape[0]))
    osc = oracle_scene(bufs, R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    albedo = np.float32([[0.7, 0.6, 0.5], [0.2, 0.8, 0.4], [0.9, 0.9, 0.2]])
    textures = [(S.noise_texture(64, 3), srgb, wrap), (S.noise_texture(17, 4), srgb, wrap)]
    mesh_tex = [1, -1, 0]
    sc.set_materials(albedo)
    sc.set_textures(textures, mesh_tex)
    rays = S.camera_rays(128, 96, **S.C1_CAMERA)
    p = gi_params(spp=2, seed=3, origin_offset=1e-3, shadow_rays=True)
    ph = osc.closest(rays)
    sec = osc.gi_raygen(rays, ph, 2, 3, 1e-3)
    sh = osc.closest(sec)
    lit = 1 - osc.anyhit(osc.shadow_raygen(sec, sh, np.array(p.sun_dir), p.shadow_offset))
    want = osc.shade(sec, sh, lit, albedo, np.array(p.sun_dir), np.array(p.sun_color),
                     np.array(p.sky_color), textures=textures, mesh_texture=mesh_tex)
    d_sec, d_sh = rays_to_device(sec), rays_to_device(sh)
    got = sc.shade(d_sec, d_sh, p, lit=rays_to_device(lit.astype(np.uint8))).cpu().numpy()
    np.testing.assert_array_equal(got[:, :3], want[:, :3])
    np.testing.assert_allclose(got[:, 3], want[:, 3], rtol=SHADE_RTOL)
    textured = (sh["t"] > 0) & np.isin(sh["mesh"], [0, 2])
    assert textured.sum() > 300
    plain = osc.shade(sec, sh, lit, albedo, np.array(p.sun_dir), np.array(p.sun_color), np.array(p.sky_color))
    assert (np.abs(plain[textured, :3] - want[textured, :3]).max(1) > 0).mean() > 0.5
    # the bounce loop multiplies by the textured albedo: compare its pixels with the oracle pipeline
    pb = gi_params(spp=2, seed=3, origin_offset=1e-3, shadow_rays=True, bounces=1)
    alb_fn = lambda hits: osc.hit_albedo(hits, albedo, textures, mesh_tex)  # noqa: E731
    want_px, _, _ = _oracle_bounce_pass(osc, rays, pb, albedo, 1, False, 0, textures=textures,
                                        mesh_texture=mesh_tex, albedo_of=alb_fn)
    got_px = sc.gi_frame(rays_to_device(rays), pb).cpu().numpy()
    np.testing.assert_allclose(got_px, want_px, rtol=SHADE_RTOL * 8, atol=1e-6)


def test_gi_frame_pinned_large_equals_device_pass(ctx):
    """A frame of several host chunks with pinned host rays on the BVH8 layout (the primary launch
    reads them over the host link, the pixels return in chunks while later chunks are shaded; the
    last chunk is short): pixels and ray counts equal the device frame.  Then RTAO on pageable
    host buffers and the RT bounce loop on pinned ones."""
    import torch
    from candela_gb300 import _lib as L
    bufs = single_object("ico2", R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(np.random.default_rng(2).uniform(0.2, 0.9, (7, 3)).astype(np.float32))
    sc.build_bvh8()
    rays = S.camera_rays(1024, 520, eye=(0.0, -4.0, 2.0), target=(0.0, 0.0, 0.3))    # 532,480 pixels
    p = gi_params(spp=2, seed=5, origin_offset=0.05, shadow_rays=True)
    want, st_want = sc.gi_frame(rays_to_device(rays), p, layout=L.LAYOUT_BVH8Q, stats=True)
    pinned = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory().numpy().view(R.RAY_DTYPE)
    out = torch.empty((len(rays), 4), dtype=torch.float32).pin_memory().numpy()
    _, st_got = sc.gi_frame(pinned, p, out=out, layout=L.LAYOUT_BVH8Q, stats=True)
    np.testing.assert_array_equal(out.view(np.uint32), want.cpu().numpy().view(np.uint32))
    assert st_got == st_want
    assert 0.1 < st_want["primary_hits"] / len(rays) < 0.9
    pa = gi_params(spp=3, seed=9, origin_offset=0.05, ray_tmax=0.5, query=1)
    want_a, st_a = sc.gi_frame(rays_to_device(rays), pa, layout=L.LAYOUT_BVH8Q, stats=True)
    got_a, st_ga = sc.gi_frame(rays, pa, layout=L.LAYOUT_BVH8Q, stats=True)
    np.testing.assert_array_equal(got_a.view(np.uint32), want_a.cpu().numpy().view(np.uint32))
    assert st_ga == st_a and 0 < st_a["secondary_hits"] < st_a["secondary_rays"]
    pb = gi_params(spp=1, seed=3, origin_offset=0.05, bounces=1)
    want_b = sc.gi_frame(rays_to_device(rays), pb, layout=L.LAYOUT_BVH8Q)
    np.testing.assert_array_equal(sc.gi_frame(pinned, pb, layout=L.LAYOUT_BVH8Q).view(np.uint32),
                                  want_b.cpu().numpy().view(np.uint32))
    assert sc.ctx.device_status() == 0


@pytest.mark.parametrize("query", [0, 1])
def test_gi_frame_rgba16f_pixels(ctx, query):
    """pixel_format = RGBA16F (the reference's rgba16f output image, DiffuseTrace.glsl:17): every
    pixel is the float pixel rounded to binary16, nearest with ties to even (numpy's conversion),
    bit for bit, on device buffers, pinned and pageable host buffers (several host chunks), the
    BVH8 layout, the bounce loop and the no-alloc entry point; a bad format is rejected."""
    import torch
    from candela_gb300 import _lib as L
    bufs = single_object("ico2", R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(np.random.default_rng(4).uniform(0.2, 0.9, (7, 3)).astype(np.float32))
    sc.build_bvh8()
    rays = S.camera_rays(768, 480, eye=(0.0, -4.0, 2.0), target=(0.0, 0.0, 0.3))  # 368,640 pixels
    kw = dict(spp=2, seed=21, origin_offset=0.05, query=query)
    if query == 1:
        kw["ray_tmax"] = 0.5
    else:
        kw["shadow_rays"] = True
    d = rays_to_device(rays)
    pinned = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory().numpy().view(R.RAY_DTYPE)
    for layout in (0, L.LAYOUT_BVH8Q):
        want = sc.gi_frame(d, gi_params(**kw), layout=layout).cpu().numpy().astype(np.float16)
        p16 = gi_params(**kw, pixel_format=L.PIXELS_RGBA16F)
        got = sc.gi_frame(d, p16, layout=layout)
        assert got.dtype == torch.float16
        np.testing.assert_array_equal(got.cpu().numpy().view(np.uint16), want.view(np.uint16))
        np.testing.assert_array_equal(sc.gi_frame(rays, p16, layout=layout).view(np.uint16), want.view(np.uint16))
        out = torch.empty((len(rays), 4), dtype=torch.float16).pin_memory().numpy()
        sc.gi_frame(pinned, p16, out=out, layout=layout)
        np.testing.assert_array_equal(out.view(np.uint16), want.view(np.uint16))
    assert np.abs(want.astype(np.float32)).sum() > 0
    if query == 0:
        pb = gi_params(spp=1, seed=3, origin_offset=0.05, bounces=2)
        wb = sc.gi_frame(d, pb).cpu().numpy().astype(np.float16)
        gb = sc.gi_frame(d, gi_params(spp=1, seed=3, origin_offset=0.05, bounces=2, pixel_format=L.PIXELS_RGBA16F))
        np.testing.assert_array_equal(gb.cpu().numpy().view(np.uint16), wb.view(np.uint16))
    # the no-alloc entry point (at most NOALLOC_MAX_RAYS secondary rays)
    small = rays_to_device(S.camera_rays(128, 96, eye=(0.0, -4.0, 2.0), target=(0.0, 0.0, 0.3)))
    want_s = sc.gi_frame(small, gi_params(**kw)).cpu().numpy().astype(np.float16)
    out_s = torch.empty((128 * 96, 4), dtype=torch.float16, device="cuda")
    import ctypes as C
    from candela_gb300.engine import _opts
    st = L.lib().rq_gi_frame_noalloc(ctx.handle, sc.handle, L.ptr(small), 128 * 96,
                                     C.byref(gi_params(**kw, pixel_format=L.PIXELS_RGBA16F)), C.byref(_opts()),
                                     L.ptr(out_s), torch.cuda.current_stream().cuda_stream)
    L.check(st, ctx.handle)
    np.testing.assert_array_equal(out_s.cpu().numpy().view(np.uint16), want_s.view(np.uint16))
    with pytest.raises(R.RqError) as e:
        sc.gi_frame(d, gi_params(**kw, pixel_format=2))
    assert e.value.status == L.RQ_EINVAL
    assert sc.ctx.device_status() == 0
