"""Parity at the benchmark scales, against the CPU restatement of the reference traversal.

The GI-pass scene (64 displaced subdivision-5 icospheres + ground, 1,310,722 triangles) and the
precision scene (256 icospheres, 5,242,880 triangles) have deeper BVHs than the small test scenes:
the 1024-iteration and 63-push caps, exact ties and the slab test's NaN paths all scale with tree
depth.  Sampled ray sets (camera rays of the 1920x1080 view, their four cosine GI rays each, rays
with origins uniform in the bounds and directions uniform on the sphere) are traced by every query
form and compared with the oracle: strict stack and stackless closest hits bit for bit (iteration
counts included) and any-hit bits identical; BVH8q records identical except rays that a brute force
over every triangle proves (see helpers.assert_equal_or_proven); fast mode within its stated bar;
the GI pass's pixels within the shading tolerance of the GI tests.
"""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S
from candela_gb300.engine import gi_params
from oracle import oracle as O

from .helpers import (assert_equal_or_proven, assert_hits_identical, assert_occlusion_equal_or_proven,
                      hits_from_device, mesh, oracle_scene, rays_to_device, single_object)

pytestmark = pytest.mark.gpu

SHADE_RTOL = 2e-6  # the GI tests' shading tolerance (the AO pow is the only non-exact operation)
TUNED = dict(block_size=128, min_blocks=7, persistent=1)  # the launch the autotuner picks for BVH8q


def _c2_rays():
    cam = S.camera_rays(1920, 1080, **S.C2_CAMERA)
    cam = np.ascontiguousarray(cam[::31][:65536])
    sph = S.sphere_rays(65536, (-4.5, -4.5, -0.2), (4.5, 4.5, 2.6), seed=71)
    return cam, sph


@pytest.fixture(scope="module")
def c2(ctx):
    out = {}
    for layout in (R.STACK, R.STACKLESS):
        bufs = single_object("c2", layout)
        sc = ctx.scene(layout, *bufs)
        out[layout] = (bufs, sc, oracle_scene(bufs, layout))
    cam, sph = _c2_rays()
    osc = out[R.STACK][2]
    ph = osc.closest(cam)
    gi = osc.gi_raygen(cam, ph, 4, 1, 1e-3, 1000000.0)
    gi = np.ascontiguousarray(gi[gi["tmax"] > 0])
    out["rays"] = {"camera": cam, "gi": gi, "sphere": sph}
    out[R.STACK][1].build_bvh8()
    yield out
    for layout in (R.STACK, R.STACKLESS):
        out[layout][1].close()


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_c2_strict_closest_and_anyhit_bit_exact(c2, layout):
    bufs, sc, osc = c2[layout]
    for name, rays in c2["rays"].items():
        d = rays_to_device(rays)
        want = osc.closest(rays)
        assert_hits_identical(hits_from_device(sc.closest(d)), want, f"c2 {name} layout {layout}")
        # the persistent ray-queue form of the same walk
        assert_hits_identical(hits_from_device(sc.closest(d, block_size=128, min_blocks=1, persistent=1)),
                              want, f"c2 {name} layout {layout} persistent")
        np.testing.assert_array_equal(sc.anyhit(d).cpu().numpy(), osc.anyhit(rays))
        assert (want["t"] > 0).sum() > len(rays) // 10
    assert sc.ctx.device_status() == 0


def test_c2_first_found_ties_and_short_tmax(c2):
    bufs, sc, osc = c2[R.STACK]
    gi = c2["rays"]["gi"].copy()
    d = rays_to_device(gi)
    assert_hits_identical(hits_from_device(sc.closest(d, tie=L.TIE_FIRST_FOUND)),
                          osc.closest(gi, tie=O.ORC_TIE_FIRST_FOUND), "c2 gi first-found")
    gi["tmax"] = np.float32(0.25)  # AO-length rays: the any-hit early exit at a short TMax
    d = rays_to_device(gi)
    want = osc.anyhit(gi)
    np.testing.assert_array_equal(sc.anyhit(d).cpu().numpy(), want)
    assert 100 < want.sum() < len(want) - 100


def test_c2_bvh8q_against_oracle(c2):
    bufs, sc, osc = c2[R.STACK]
    exceptions = 0
    for name, rays in c2["rays"].items():
        d = rays_to_device(rays)
        want = osc.closest(rays)
        for kw in (dict(), TUNED, dict(block_size=128, min_blocks=8, persistent=0)):
            got = hits_from_device(sc.closest(d, layout=L.LAYOUT_BVH8Q, **kw))
            exceptions += assert_equal_or_proven(got, want, osc, rays, what=f"c2 {name} bvh8q {kw}")
        want_occ = osc.anyhit(rays)
        for kw in (dict(), TUNED):
            occ = sc.anyhit(d, layout=L.LAYOUT_BVH8Q, **kw).cpu().numpy()
            exceptions += assert_occlusion_equal_or_proven(occ, want_occ, osc, rays, what=f"c2 {name} any {kw}")
    assert sc.ctx.device_status() == 0


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_c2_fast_mode_against_oracle(c2, layout):
    """Fast mode: identical hit/miss and triangle on >= 99.99 % of rays; |dt| <= 1e-5 t."""
    bufs, sc, osc = c2[layout]
    rays = np.concatenate([c2["rays"]["camera"], c2["rays"]["gi"], c2["rays"]["sphere"]])
    d = rays_to_device(rays)
    want = osc.closest(rays)
    got = hits_from_device(sc.closest(d, mode=L.MODE_FAST))
    same_id = ((want["t"] > 0) == (got["t"] > 0)) & (want["tri"] == got["tri"])
    assert same_id.mean() >= 0.9999, (~same_id).sum()
    both = same_id & (want["t"] > 0)
    rel = np.abs(got["t"][both] - want["t"][both]) / want["t"][both]
    assert (rel <= 1e-5).mean() >= 0.9999 and rel.max() < 1e-3
    occ = sc.anyhit(d, mode=L.MODE_FAST).cpu().numpy()
    assert (occ == osc.anyhit(rays)).mean() >= 0.9999


@pytest.mark.parametrize("layout", [0, L.LAYOUT_BVH8Q])
def test_c2_gi_pass_pixels_against_oracle(c2, layout):
    """The GI pass of the benchmark (4 cosine GI rays per hit, offset 1e-3, Lambert shading with
    per-mesh albedo) on the sampled pixels, against the oracle's pipeline."""
    bufs, sc, osc = c2[R.STACK]
    cam = c2["rays"]["camera"]
    n_mesh = int(mesh("c2").mesh_ids.max()) + 1
    albedo = (0.25 + 0.65 * S.uniform(17, 5, n_mesh * 3)).astype(np.float32).reshape(-1, 3)
    sc.set_materials(albedo)
    p = gi_params(spp=4, seed=1, origin_offset=1e-3, ray_tmax=1000000.0, query=0)
    ph = osc.closest(cam)
    sec = osc.gi_raygen(cam, ph, 4, 1, 1e-3)
    sh = osc.closest(sec)
    shaded = osc.shade(sec, sh, None, albedo, np.array(p.sun_dir), np.array(p.sun_color),
                       np.array(p.sky_color))
    want = shaded.reshape(-1, 4, 4).sum(1) * np.float32(0.25)
    kw = TUNED if layout == L.LAYOUT_BVH8Q else {}
    got, st = sc.gi_frame(rays_to_device(cam), p, layout=layout, stats=True, **kw)
    np.testing.assert_allclose(got.cpu().numpy(), want, rtol=SHADE_RTOL * 4, atol=1e-6)
    assert st["primary_hits"] == (ph["t"] > 0).sum()
    assert st["secondary_hits"] == (sh["t"] > 0).sum()
    assert sc.ctx.device_status() == 0


@pytest.fixture(scope="module")
def c4(ctx):
    bufs = single_object("c4", R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    sc.build_bvh8()
    rays = S.sphere_rays(65536, *S.C4_BOUNDS, seed=44)
    yield bufs, sc, oracle_scene(bufs, R.STACK), rays
    sc.close()


def test_c4_strict_and_bvh8q_against_oracle(c4):
    """Precision scene (5,242,880 triangles), incoherent rays: strict closest hits and any-hit bits
    bit for bit, BVH8q records identical or proven, fast mode within its bar."""
    bufs, sc, osc, rays = c4
    d = rays_to_device(rays)
    want = osc.closest(rays)
    assert_hits_identical(hits_from_device(sc.closest(d)), want, "c4 strict")
    want_occ = osc.anyhit(rays)
    np.testing.assert_array_equal(sc.anyhit(d).cpu().numpy(), want_occ)
    n_exc = 0
    for kw in (dict(), TUNED):
        got = hits_from_device(sc.closest(d, layout=L.LAYOUT_BVH8Q, **kw))
        n_exc += assert_equal_or_proven(got, want, osc, rays, what=f"c4 bvh8q {kw}")
        occ = sc.anyhit(d, layout=L.LAYOUT_BVH8Q, **kw).cpu().numpy()
        n_exc += assert_occlusion_equal_or_proven(occ, want_occ, osc, rays, what=f"c4 any {kw}")
    fast = hits_from_device(sc.closest(d, mode=L.MODE_FAST))
    same_id = ((want["t"] > 0) == (fast["t"] > 0)) & (want["tri"] == fast["tri"])
    assert same_id.mean() >= 0.9999
    assert 0.1 < (want["t"] > 0).mean() < 0.95
    assert sc.ctx.device_status() == 0
