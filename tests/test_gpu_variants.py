"""Every compiled launch variant (block size x occupancy target x persistent x BVH8 group-stack
depth) gives bit-identical results, the autotuners (traversal launches, the batch plan, the GI
pass's compaction threshold) record valid choices that later queries use, and every choice they can
make gives the same hits and pixels."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S

from .helpers import hits_from_device, rays_to_device, single_object

pytestmark = pytest.mark.gpu

VARIANTS = [(128, 1, 0, 0), (128, 4, 0, 0), (128, 6, 0, 0), (128, 8, 0, 0), (256, 3, 0, 0), (64, 12, 0, 0),
            (128, 1, 1, 0), (128, 7, 1, 0), (128, 7, 1, 32), (128, 7, 1, 24)]


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS, L.LAYOUT_BVH8Q])
def test_all_variants_identical(ctx, layout):
    base = R.STACK if layout == L.LAYOUT_BVH8Q else layout
    sc = ctx.scene(base, *single_object("ico2", base))
    if layout == L.LAYOUT_BVH8Q:
        sc.build_bvh8()
    rays = rays_to_device(S.sphere_rays(150_000, (-2, -2, -0.2), (2, 2, 1.2), seed=5))
    ref_h = sc.closest(rays, layout=layout, block_size=128, min_blocks=1).cpu().numpy()
    ref_o = sc.anyhit(rays, layout=layout, block_size=128, min_blocks=1).cpu().numpy()
    for b, m, p, dep in VARIANTS:
        kw = dict(layout=layout, block_size=b, min_blocks=m, persistent=p, stack_depth=dep)
        h = sc.closest(rays, **kw).cpu().numpy()
        assert np.array_equal(h.view(np.uint32), ref_h.view(np.uint32)), kw
        o = sc.anyhit(rays, **kw).cpu().numpy()
        assert np.array_equal(o, ref_o), kw
    assert ctx.device_status() == 0  # no stack overflow at any depth
    with pytest.raises(R.RqError):
        sc.closest(rays, layout=layout, block_size=96, min_blocks=1)
    with pytest.raises(R.RqError):
        sc.closest(rays, layout=layout, block_size=128, min_blocks=7, persistent=1, stack_depth=40)


def test_autotune_records_choice(ctx):
    sc = ctx.scene(R.STACK, *single_object("c1", R.STACK))
    sc.build_bvh8()
    rays = rays_to_device(S.camera_rays(512, 512, **S.C1_CAMERA))
    before = sc.closest(rays, layout=L.LAYOUT_BVH8Q).cpu().numpy()
    res = sc.autotune(rays, query=0, layout=L.LAYOUT_BVH8Q)
    assert 0 <= res["variant"] < len(VARIANTS)
    timed = [v["ms"] for v in res["variants"] if v["ms"] >= 0]
    assert len(timed) == len(VARIANTS) and min(timed) > 0
    assert res["stack_depth"] in (48, 32, 24)
    assert [v["stack_depth"] for v in res["variants"]][-3:] == [48, 32, 24]
    after = sc.closest(rays, layout=L.LAYOUT_BVH8Q).cpu().numpy()   # uses the tuned variant
    assert np.array_equal(before.view(np.uint32), after.view(np.uint32))
    res2 = sc.autotune(rays, query=1, layout=R.STACK)
    assert res2["variants"][6]["ms"] > 0 and res2["variants"][7]["ms"] > 0  # persistent forms timed
    assert res2["variants"][8]["ms"] == -1 and res2["variants"][9]["ms"] == -1  # depth: BVH8 only
    assert ctx.device_status() == 0


def test_gi_compaction_threshold_and_tuner(ctx):
    """The GI pass with its secondary rays compacted or in place (forced by the threshold, or picked
    by rq_gi_autotune) gives the same pixels bit for bit and the same ray counts, for GI with shadow
    rays and for RTAO, on BVH8q and strict BVH2, one thread per ray and persistent launches."""
    from candela_gb300.engine import gi_params
    sc = ctx.scene(R.STACK, *single_object("hf64", R.STACK))
    sc.set_materials(np.array([[0.7, 0.6, 0.5]], dtype=np.float32))
    sc.build_bvh8()
    rays = rays_to_device(S.camera_rays(192, 160, eye=(0.0, -1.8, 1.2), target=(0.0, 0.3, 0.0)))
    for kw in (dict(spp=3, seed=11, origin_offset=1e-3, shadow_rays=True, shadow_offset=1e-3),
               dict(spp=2, seed=11, origin_offset=1e-3, ray_tmax=0.25, query=1)):
        want, st_w = sc.gi_frame(rays, gi_params(**kw, compact_below=2.0), stats=True)
        want = want.cpu().numpy()
        assert 0.2 < st_w["primary_hits"] / st_w["primary_rays"] < 0.999
        for launch in (dict(), dict(layout=L.LAYOUT_BVH8Q, block_size=128, min_blocks=7, persistent=1),
                       dict(layout=L.LAYOUT_BVH8Q, block_size=128, min_blocks=7, persistent=1, stack_depth=24)):
            for cb in (2.0, 1e-30, 0.5, 0.99):
                got, st = sc.gi_frame(rays, gi_params(**kw, compact_below=cb), stats=True, **launch)
                np.testing.assert_array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32))
                assert st == st_w, (launch, cb)
        tune = sc.gi_autotune(rays, gi_params(**kw), layout=L.LAYOUT_BVH8Q)
        assert tune["ms_compact"] > 0 and tune["ms_in_place"] > 0
        assert abs(tune["live_fraction"] - st_w["primary_hits"] / st_w["primary_rays"]) < 1e-6
        assert tune["compact_below"] == 2.0 or tune["compact_below"] == pytest.approx(tune["live_fraction"])
        got = sc.gi_frame(rays, gi_params(**kw), layout=L.LAYOUT_BVH8Q).cpu().numpy()  # the tuned threshold
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert ctx.device_status() == 0
