"""Every compiled launch variant (block size x occupancy target x persistent) gives bit-identical
results, and the autotuner records a valid choice that later queries use."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S

from .helpers import hits_from_device, rays_to_device, single_object

pytestmark = pytest.mark.gpu

VARIANTS = [(128, 1, 0), (128, 4, 0), (128, 6, 0), (128, 8, 0), (256, 3, 0), (64, 12, 0), (128, 1, 1),
            (128, 8, 1)]


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS, L.LAYOUT_BVH8Q])
def test_all_variants_identical(ctx, layout):
    base = R.STACK if layout == L.LAYOUT_BVH8Q else layout
    sc = ctx.scene(base, *single_object("ico2", base))
    if layout == L.LAYOUT_BVH8Q:
        sc.build_bvh8()
    rays = rays_to_device(S.sphere_rays(150_000, (-2, -2, -0.2), (2, 2, 1.2), seed=5))
    ref_h = sc.closest(rays, layout=layout, block_size=128, min_blocks=1).cpu().numpy()
    ref_o = sc.anyhit(rays, layout=layout, block_size=128, min_blocks=1).cpu().numpy()
    for b, m, p in VARIANTS:
        h = sc.closest(rays, layout=layout, block_size=b, min_blocks=m, persistent=p).cpu().numpy()
        assert np.array_equal(h.view(np.uint32), ref_h.view(np.uint32)), (b, m, p)
        o = sc.anyhit(rays, layout=layout, block_size=b, min_blocks=m, persistent=p).cpu().numpy()
        assert np.array_equal(o, ref_o), (b, m, p)
    with pytest.raises(R.RqError):
        sc.closest(rays, layout=layout, block_size=96, min_blocks=1)


def test_autotune_records_choice(ctx):
    sc = ctx.scene(R.STACK, *single_object("c1", R.STACK))
    sc.build_bvh8()
    rays = rays_to_device(S.camera_rays(512, 512, **S.C1_CAMERA))
    before = sc.closest(rays, layout=L.LAYOUT_BVH8Q).cpu().numpy()
    res = sc.autotune(rays, query=0, layout=L.LAYOUT_BVH8Q)
    assert 0 <= res["variant"] < len(VARIANTS)
    timed = [v["ms"] for v in res["variants"] if v["ms"] >= 0]
    assert len(timed) == len(VARIANTS) and min(timed) > 0
    after = sc.closest(rays, layout=L.LAYOUT_BVH8Q).cpu().numpy()   # uses the tuned variant
    assert np.array_equal(before.view(np.uint32), after.view(np.uint32))
    res2 = sc.autotune(rays, query=1, layout=R.STACK)
    assert res2["variants"][6]["ms"] > 0 and res2["variants"][7]["ms"] > 0  # persistent forms timed
    assert ctx.device_status() == 0
