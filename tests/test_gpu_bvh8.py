"""BVH8 with quantised boxes on the GPU: hit records equal the oracle's strict BVH2 records (t,
barycentrics, triangle, mesh, entity; `iters` counts different nodes) and any-hit bits are equal,
except rays where a brute force over every triangle proves the BVH8 answer (the reference's slab
test can round a node with the closest hit away; the conservative BVH8 boxes keep it).  No status
bits."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S

from .helpers import (assert_equal_or_proven, assert_occlusion_equal_or_proven, hits_from_device, mesh,
                      oracle_scene, rays_to_device, single_object)

pytestmark = pytest.mark.gpu

FIELDS = ["t", "u", "v", "w", "tri", "mesh", "entity"]


def _same(a, b):
    ua = np.ascontiguousarray(a).view(np.uint32).reshape(len(a), 8)[:, :7]
    ub = np.ascontiguousarray(b).view(np.uint32).reshape(len(b), 8)[:, :7]
    return (ua == ub).all(1)


@pytest.mark.parametrize("name,layout,leaf", [("c1", R.STACK, 2), ("c1", R.STACKLESS, 2),
                                              ("ico2", R.STACK, 4), ("hf64", R.STACK, 2)])
def test_bvh8_equals_strict(ctx, name, layout, leaf):
    bufs = single_object(name, layout, leaf)
    sc = ctx.scene(layout, *bufs)
    info = sc.build_bvh8()
    assert info["nodes"] > 0 and info["triangles"] == bufs[1].shape[0]
    rays = np.concatenate([S.camera_rays(384, 256, **S.C1_CAMERA),
                           S.sphere_rays(100_000, (-1.5, -1.5, -0.3), (1.5, 1.5, 1.2), seed=41)])
    d = rays_to_device(rays)
    osc = oracle_scene(bufs, layout)
    want = osc.closest(rays)
    strict = hits_from_device(sc.closest(d))
    assert _same(strict, want).all()
    for kw in (dict(), dict(block_size=128, min_blocks=7, persistent=1)):
        b8 = hits_from_device(sc.closest(d, layout=L.LAYOUT_BVH8Q, **kw))
        assert_equal_or_proven(b8, want, osc, rays, what=f"{name} layout {layout} {kw}")
        occ_8 = sc.anyhit(d, layout=L.LAYOUT_BVH8Q, **kw).cpu().numpy()
        assert_occlusion_equal_or_proven(occ_8, osc.anyhit(rays), osc, rays, what=f"{name} any {kw}")
    assert ctx.device_status() == 0


def test_bvh8_multi_entity_and_oracle(ctx):
    ri = R.RayIntersector(R.STACK)
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    T = np.eye(4)
    T[:3, 3] = [0.25, -0.5, 0.125]
    ri.push_entity(1)
    ri.push_entity(2, model=T)
    ri.push_entity(2)
    ri.buffer_entities()
    sc = ri.buffer_data(ctx)
    sc.build_bvh8()
    rays = S.sphere_rays(100_000, (-1.5, -1.5, -0.5), (1.5, 1.5, 1.5), seed=22)
    from oracle import oracle as O
    osc = O.OracleScene(O.ORC_STACK, *ri.global_buffers())
    want = osc.closest(rays)
    got = hits_from_device(sc.closest(rays_to_device(rays), layout=L.LAYOUT_BVH8Q))
    assert_equal_or_proven(got, want, osc, rays, what="multi-entity")
    # entities changed after the build: the BVH8 follows
    ri.push_entity(1, model=T)
    ri.buffer_entities()
    osc2 = O.OracleScene(O.ORC_STACK, *ri.global_buffers())
    want2 = osc2.closest(rays)
    got2 = hits_from_device(sc.closest(rays_to_device(rays), layout=L.LAYOUT_BVH8Q))
    assert_equal_or_proven(got2, want2, osc2, rays, what="multi-entity after set_entities")
    assert ctx.device_status() == 0


def test_bvh8_requires_build_and_strict(ctx):
    bufs = single_object("hf32", R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    rays = rays_to_device(S.camera_rays(16, 16, **S.C1_CAMERA))
    with pytest.raises(R.RqError) as e:
        sc.closest(rays, layout=L.LAYOUT_BVH8Q)
    assert e.value.status == L.RQ_ENOTSUP


def test_fp64_verification_kernel(ctx):
    """rq_verify_hits: FP64 recomputation of each winning hit agrees with a numpy FP64 evaluation and
    bounds the FP32 error."""
    bufs = single_object("ico2", R.STACK)
    v, t, n, e = bufs
    sc = ctx.scene(R.STACK, *bufs)
    rays = S.sphere_rays(50_000, (-1.5, -1.5, -0.2), (1.5, 1.5, 1.0), seed=9)
    d = rays_to_device(rays)
    h = sc.closest(d)
    err = sc.verify(d, h).cpu().numpy()
    hh = hits_from_device(h)
    hit = hh["t"] > 0
    assert np.isnan(err[~hit]).all()
    ok = np.isfinite(err[:, 0])
    assert ok.sum() >= 0.99 * hit.sum()
    assert np.median(err[ok, 0]) < 1e-6 and err[ok, 0].max() < 1e-3
    # numpy FP64 reference on a few hits
    P = v["pos"][:, :3].astype(np.float64)
    for i in np.nonzero(ok)[0][:50]:
        a, b, c = P[t[hh["tri"][i], :3]]
        o, dd = rays["o"][i].astype(np.float64), rays["d"][i].astype(np.float64)
        e1, e2 = b - a, c - a
        p_ = np.cross(dd, e2)
        det = e1 @ p_
        tv = o - a
        q = np.cross(tv, e1)
        t64 = (e2 @ q) / det
        assert abs(abs(hh["t"][i] - t64) / t64 - err[i, 0]) <= 1e-6 * max(1.0, err[i, 0])
