"""Fast mode against the oracle's strict hits, and batched queries against per-query calls."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S

from .helpers import hits_from_device, oracle_scene, rays_to_device, single_object

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,layout", [("c1", R.STACK), ("c1", R.STACKLESS), ("ico2", R.STACK)])
def test_fast_mode_agrees_with_oracle(ctx, name, layout):
    """Fast mode: identical hit/miss and triangle IDs against the oracle's strict hits on >= 99.99 %
    of rays, |dt| <= 1e-5 t on >= 99.99 % of the shared hits; occlusion bits likewise."""
    bufs = single_object(name, layout)
    sc = ctx.scene(layout, *bufs)
    osc = oracle_scene(bufs, layout)
    rays = np.concatenate([S.camera_rays(384, 256, **S.C1_CAMERA),
                           S.sphere_rays(200_000, (-1.5, -1.5, -0.3), (1.5, 1.5, 1.2), seed=7)])
    d = rays_to_device(rays)
    st = osc.closest(rays)
    fa = hits_from_device(sc.closest(d, mode=L.MODE_FAST))
    same_hit = (st["t"] > 0) == (fa["t"] > 0)
    same_id = same_hit & (st["tri"] == fa["tri"])
    assert same_id.mean() >= 0.9999, (~same_id).sum()
    both = same_id & (st["t"] > 0)
    rel = np.abs(fa["t"][both] - st["t"][both]) / st["t"][both]
    assert (rel <= 1e-5).mean() >= 0.9999 and rel.max() < 1e-3
    oc_s = osc.anyhit(rays)
    oc_f = sc.anyhit(d, mode=L.MODE_FAST).cpu().numpy()
    assert (oc_s == oc_f).mean() >= 0.9999


def _scenes(ctx):
    out = []
    for name, layout in (("hf32", R.STACK), ("ico2", R.STACK), ("hf64", R.STACKLESS)):
        sc = ctx.scene(layout, *single_object(name, layout))
        sc.build_bvh8()
        out.append(sc)
    return out


def _queries(scenes):
    import torch
    rng = np.random.default_rng(2)
    qs = []
    sizes = [1000, 0, 1, 37, 25_000, 3_000, 70_000, 513]
    for k, n in enumerate(sizes):
        sc = scenes[k % len(scenes)]
        rays = S.sphere_rays(max(n, 1), (-1.5, -1.5, -0.3), (1.5, 1.5, 1.0), seed=100 + k)[:n]
        d = rays_to_device(rays) if n else torch.zeros(0, dtype=torch.uint8, device="cuda")
        kind = int(rng.integers(0, 2))
        out = (torch.empty((n, 8), dtype=torch.float32, device="cuda") if kind == 0
               else torch.empty(n, dtype=torch.uint8, device="cuda"))
        qs.append((sc, d, kind, out))
    return qs


def _per_query(qs, **kw):
    res = []
    for sc, d, kind, out in qs:
        if d.numel() == 0:
            res.append(None)
            continue
        r = sc.closest(d, **kw) if kind == 0 else sc.anyhit(d, **kw)
        res.append(r.cpu().numpy().copy())
    return res


def _check(qs, want):
    for (sc, d, kind, out), w in zip(qs, want):
        if w is None:
            continue
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint8), w.view(np.uint8))


@pytest.mark.parametrize("layout,mode", [(0, L.MODE_STRICT), (L.LAYOUT_BVH8Q, L.MODE_STRICT),
                                         (0, L.MODE_FAST)])
def test_batch_equals_per_query(ctx, layout, mode):
    scenes = _scenes(ctx)
    qs = _queries(scenes)
    want = _per_query(qs, layout=layout, mode=mode)
    R.engine.batch(ctx, qs, layout=layout, mode=mode)
    _check(qs, want)
    for sc, d, kind, out in qs:
        out.zero_()
    R.engine.batch(ctx, qs, layout=layout, mode=mode, block_size=128, min_blocks=7)
    _check(qs, want)
    assert ctx.device_status() == 0


@pytest.mark.parametrize("kinds", ["closest", "any", "alternating"])
def test_batch_bvh8_lane_refill_kinds(ctx, kinds):
    """The BVH8q batch on scenes without a top level runs the closest-hit queries' rays, then the
    any-hit queries' rays, each from its own ray queue: batches of one kind (one phase empty) and
    alternating kinds give the per-query records, in every launch shape and group-stack depth."""
    import torch
    scenes = _scenes(ctx)
    qs = []
    for k, n in enumerate([4000, 1, 0, 30_000, 777, 12_000]):
        kind = {"closest": 0, "any": 1}.get(kinds, k % 2)
        rays = S.sphere_rays(max(n, 1), (-1.5, -1.5, -0.3), (1.5, 1.5, 1.0), seed=300 + k)[:n]
        d = rays_to_device(rays) if n else torch.zeros(0, dtype=torch.uint8, device="cuda")
        out = (torch.empty((n, 8), dtype=torch.float32, device="cuda") if kind == 0
               else torch.empty(n, dtype=torch.uint8, device="cuda"))
        qs.append((scenes[k % len(scenes)], d, kind, out))
    want = _per_query(qs, layout=L.LAYOUT_BVH8Q)
    for kw in (dict(), dict(block_size=128, min_blocks=1), dict(block_size=64, min_blocks=12),
               dict(block_size=256, min_blocks=3, stack_depth=24), dict(block_size=128, min_blocks=7, stack_depth=32)):
        for sc, d, kind, out in qs:
            out.zero_()
        R.engine.batch(ctx, qs, layout=L.LAYOUT_BVH8Q, **kw)
        _check(qs, want)
    assert ctx.device_status() == 0


def test_batch_plan_graph_and_autotune(ctx):
    scenes = _scenes(ctx)
    qs = _queries(scenes)
    want = _per_query(qs, layout=L.LAYOUT_BVH8Q)
    plan = R.engine.BatchPlan(ctx, qs, layout=L.LAYOUT_BVH8Q)
    for _ in range(2):
        for sc, d, kind, out in qs:
            out.zero_()
        plan.launch()
        _check(qs, want)
    res = plan.autotune(allow_bvh8=True)
    # BVH8q: 4 launch shapes x group-stack depths 48 / 32 / 24; BVH2 strict: 4 launch shapes
    assert res["family"] in (0, 1) and len(res["combos"]) == 16
    assert sum(c["ms"] > 0 for c in res["combos"]) == 16
    assert sorted({c["stack_depth"] for c in res["combos"] if c["family"] == 0}) == [24, 32, 48]
    # every combination the tuner can pick gives the per-query results
    for depth in (48, 32, 24):
        for sc, d, kind, out in qs:
            out.zero_()
        R.engine.batch(ctx, qs, layout=L.LAYOUT_BVH8Q, block_size=128, min_blocks=7, stack_depth=depth)
        _check(qs, want)
    for sc, d, kind, out in qs:
        out.zero_()
    plan.launch()
    if res["family"] == 0:
        _check(qs, want)
    else:
        _check(qs, _per_query(qs))
    plan.close()
