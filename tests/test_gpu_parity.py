"""Strict-mode parity: the CUDA kernels (through the C ABI) against the CPU restatement of the
reference traversal, bit for bit, on the same BVH buffers and rays."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import (assert_hits_identical, hits_from_device, oracle_scene, rays_to_device,
                      single_object)

pytestmark = pytest.mark.gpu

TIES = [(R.engine.L.TIE_LOWER_INDEX, O.ORC_TIE_LOWER_INDEX),
        (R.engine.L.TIE_FIRST_FOUND, O.ORC_TIE_FIRST_FOUND)]


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
@pytest.mark.parametrize("tie", TIES, ids=["lower_index", "first_found"])
def test_c1_primary_closest_bit_exact(ctx, layout, tie):
    """Heightfield 256x256 (131,072 tris), 512x512 camera rays: closest hit bit-exact."""
    bufs = single_object("c1", layout)
    rays = S.camera_rays(512, 512, **S.C1_CAMERA)
    want = oracle_scene(bufs, layout).closest(rays, tie=tie[1])
    sc = ctx.scene(layout, *bufs)
    got = hits_from_device(sc.closest(rays_to_device(rays), tie=tie[0]))
    assert_hits_identical(got, want, f"layout {layout}")
    assert (want["t"] > 0).sum() > 50000


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_c1_ao_anyhit_bit_exact(ctx, layout):
    """One cosine-weighted AO ray per primary hit (tmax 0.25): occlusion bits identical."""
    bufs = single_object("c1", layout)
    osc = oracle_scene(bufs, layout)
    rays = S.camera_rays(512, 512, **S.C1_CAMERA)
    hits = osc.closest(rays)
    ao = osc.gi_raygen(rays, hits, 1, 7, 1e-3, 0.25)
    want = osc.anyhit(ao)
    sc = ctx.scene(layout, *bufs)
    got = sc.anyhit(rays_to_device(ao)).cpu().numpy()
    np.testing.assert_array_equal(got, want)
    assert 0 < want.sum() < (ao["tmax"] > 0).sum()


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_host_buffer_path_matches_device_path(ctx, layout):
    bufs = single_object("hf64", layout)
    rays = S.sphere_rays(300_000, (-1.2, -1.2, -0.3), (1.2, 1.2, 0.6), seed=3)
    sc = ctx.scene(layout, *bufs)
    host = sc.closest(rays)                       # numpy in/out: copies inside the call
    dev = hits_from_device(sc.closest(rays_to_device(rays)))
    assert_hits_identical(host, dev, "host vs device buffers")
    want = oracle_scene(bufs, layout).closest(rays)
    assert_hits_identical(host, want, "host path vs oracle")
    occ_h = sc.anyhit(rays)
    np.testing.assert_array_equal(occ_h, oracle_scene(bufs, layout).anyhit(rays))


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_incoherent_rays_icospheres(ctx, layout):
    bufs = single_object("ico2", layout)
    rays = S.sphere_rays(200_000, (-2, -2, -0.2), (2, 2, 1.2), seed=8)
    osc = oracle_scene(bufs, layout)
    sc = ctx.scene(layout, *bufs)
    for tie in TIES:
        assert_hits_identical(hits_from_device(sc.closest(rays_to_device(rays), tie=tie[0])),
                              osc.closest(rays, tie=tie[1]), "icospheres")
    np.testing.assert_array_equal(sc.anyhit(rays_to_device(rays)).cpu().numpy(), osc.anyhit(rays))


def test_ref_compat_triangle_zero_quirk(ctx):
    """RQ_FLAG_REF_COMPAT reproduces IntersectScene's `TriangleIdx > 0` test."""
    layout = R.STACK
    bufs = single_object("hf32", layout)
    v, t, n, e = bufs
    tri0 = t[0, :3]
    p = v["pos"][tri0, :3].astype(np.float64).mean(0)
    rays = np.zeros(2, dtype=R.RAY_DTYPE)
    rays["o"] = p + [0.0, 0.0, 1.0]
    rays["d"] = [0.0, 0.0, -1.0]
    rays["tmax"] = 1e6
    rays[1]["o"] = p + [0.001, 0.002, 1.0]
    osc = oracle_scene(bufs, layout)
    sc = ctx.scene(layout, *bufs)
    for flags in (0, R.engine.L.FLAG_REF_COMPAT):
        want = osc.closest(rays, flags=flags)
        got = hits_from_device(sc.closest(rays_to_device(rays), flags=flags))
        assert_hits_identical(got, want, f"flags {flags}")
    w = osc.closest(rays, flags=O.ORC_FLAG_REF_COMPAT)
    if w["tri"][0] == 0:
        assert w["t"][0] == -1.0


def test_multi_entity_transforms_and_transparency(ctx):
    """Two objects, three entities (one translated, one translucent), ignore-transparent flag."""
    layout = R.STACK
    ri = R.RayIntersector(layout)
    from .helpers import mesh
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    T = np.eye(4)
    T[:3, 3] = [0.25, -0.5, 0.125]
    ri.push_entity(1)
    ri.push_entity(2, model=T)
    ri.push_entity(1, model=np.diag([1.0, 1.0, 1.0, 1.0]) @ np.array(
        [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0.3], [0, 0, 0, 1]]), translucency=0.5)
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    rays = S.sphere_rays(100_000, (-1.5, -1.5, -0.5), (1.5, 1.5, 1.5), seed=21)
    osc = O.OracleScene(O.ORC_STACK, v, t, n, e)
    sc = ri.buffer_data(ctx)
    for flags in (0, R.engine.L.FLAG_IGNORE_TRANSPARENT):
        want = osc.closest(rays, flags=flags)
        got = hits_from_device(sc.closest(rays_to_device(rays), flags=flags))
        assert_hits_identical(got, want, f"multi-entity flags {flags}")
        assert len(np.unique(want["entity"][want["t"] > 0])) >= 2
    np.testing.assert_array_equal(sc.anyhit(rays_to_device(rays)).cpu().numpy(), osc.anyhit(rays))


def test_edge_rays(ctx):
    """Empty batch, inactive rays (tmax <= tmin), NaN/inf/zero directions, axis-aligned rays."""
    layout = R.STACK
    bufs = single_object("hf32", layout)
    osc = oracle_scene(bufs, layout)
    sc = ctx.scene(layout, *bufs)
    empty = np.zeros(0, dtype=R.RAY_DTYPE)
    assert sc.closest(empty).shape == (0,)
    r = np.zeros(12, dtype=R.RAY_DTYPE)
    r["o"] = [0.1, 0.2, 1.0]
    r["d"] = [0.0, 0.0, -1.0]
    r["tmax"] = 1e6
    r[1]["tmax"] = 0.0                       # inactive
    r[2]["tmax"] = -1.0                      # inactive
    r[3]["d"] = [np.nan, 0.0, -1.0]
    r[4]["d"] = [0.0, 0.0, 0.0]
    r[5]["d"] = [np.inf, 0.0, -1.0]
    r[6]["o"] = [0.0, 0.0, 1.0]              # origin on box planes, zero x/y direction
    r[7]["o"] = [-1.0, -1.0, 0.5]            # on the scene AABB corner
    r[8]["d"] = [1.0, 0.0, 0.0]              # parallel to the ground plane
    r[8]["o"] = [-2.0, 0.0, 0.0]
    r[9]["o"] = [0.1, 0.2, 1.0]
    r[9]["d"] = [-0.0, -0.0, -1.0]           # negative zeros
    r[10]["tmin"] = 5.0                      # hit before tmin
    r[11]["tmax"] = 1e-6                     # hit beyond tmax
    want = osc.closest(r)
    got = hits_from_device(sc.closest(rays_to_device(r)))
    assert_hits_identical(got, want, "edge rays")
    np.testing.assert_array_equal(sc.anyhit(rays_to_device(r)).cpu().numpy(), osc.anyhit(r))


def test_leaf4_bvh(ctx):
    layout = R.STACK
    bufs = single_object("c1", layout, leaf=4)
    rays = S.camera_rays(256, 256, **S.C1_CAMERA)
    sc = ctx.scene(layout, *bufs)
    assert_hits_identical(hits_from_device(sc.closest(rays_to_device(rays))),
                          oracle_scene(bufs, layout).closest(rays), "leaf 4")


@pytest.mark.parametrize("depth", [40, 70])
def test_push_cap_on_gpu(ctx, depth):
    """The reference's 63-push cap (TraverseBVHStack.glsl:293-295) on a hand-made chain BVH."""
    from .test_oracle import _chain_bvh
    v, t, n, e = _chain_bvh(depth)
    rays = np.zeros(3, dtype=R.RAY_DTYPE)
    rays["o"] = [[0, 0, 0.5], [0.1, -0.2, 0.7], [0.0, 0.3, -0.5]]
    rays["d"] = [[0, 0, -1], [0, 0, -1], [0, 0, 1]]
    rays["tmax"] = 1e6
    osc = O.OracleScene(O.ORC_STACK, v, t, n, e)
    sc = ctx.scene(R.STACK, v, t, n, e)
    assert_hits_identical(hits_from_device(sc.closest(rays_to_device(rays))), osc.closest(rays),
                          f"chain depth {depth}")
    np.testing.assert_array_equal(sc.anyhit(rays_to_device(rays)).cpu().numpy(), osc.anyhit(rays))
