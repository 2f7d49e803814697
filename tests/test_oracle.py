"""The CPU restatement of the reference traversal (oracle/), checked on its own: known-answer tests
for the primitives, an independent FP64 brute-force intersector, the committed golden results, and
the reference's traversal caps."""
from pathlib import Path

import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import hits_u32, oracle_scene, single_object

F = np.float32
INF = np.float32(np.inf)


# ---- RayTriangle (TraverseBVHStack.glsl:87-105) ---------------------------------------------

def test_ray_triangle_center_hit():
    t, u, v = O.ray_triangle([0.25, 0.25, 1.0], [0, 0, -1], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert t == F(1.0) and u == F(0.25) and v == F(0.25)


def test_ray_triangle_back_face_and_behind():
    # IQ's test is two-sided: a hit from below reports the same t
    t, u, v = O.ray_triangle([0.25, 0.25, -2.0], [0, 0, 1], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert t == F(2.0)
    # triangle behind the origin: negative t (rejected by the caller's t > 0)
    t, _, _ = O.ray_triangle([0.25, 0.25, 1.0], [0, 0, 1], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert t == F(-1.0)


def test_ray_triangle_outside_and_edges():
    # outside: u < 0 -> t = -1
    t, u, v = O.ray_triangle([-0.1, 0.5, 1.0], [0, 0, -1], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert t == F(-1.0) and u < 0
    # exactly on the u+v = 1 edge: accepted (the test is u + v > 1)
    t, u, v = O.ray_triangle([0.5, 0.5, 1.0], [0, 0, -1], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert t == F(1.0) and u + v == F(1.0)
    # on a vertex
    t, u, v = O.ray_triangle([0.0, 0.0, 1.0], [0, 0, -1], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert t == F(1.0) and u == 0 and v == 0


def test_ray_triangle_parallel_and_degenerate():
    # ray parallel to the plane: 1/dot = inf, u, v, t become inf/nan; NaN comparisons are false
    # so the GLSL test does not reject it and t stays non-finite (the caller's t < TMax rejects)
    t, u, v = O.ray_triangle([0.25, 0.25, 1.0], [1, 0, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert not np.isfinite(t) or t == -1.0
    # zero-area triangle: n = 0, d = 1/0 = inf, t = inf*0 = nan -> never accepted
    t, u, v = O.ray_triangle([0.25, 0.25, 1.0], [0, 0, -1], [0, 0, 0], [1, 0, 0], [2, 0, 0])
    assert not (t > 0 and t < 1e6)


# ---- RayBounds: GLSL min/max semantics --------------------------------------------------------

def test_ray_bounds_stack_basic():
    t = O.ray_bounds_stack([0, 0, -5], [INF, INF, 1.0], [-1, -1, -1], [1, 1, 1], 1e6)
    assert t == F(4.0)
    # origin inside: t0 = 0 -> returns t1 (the exit distance)
    t = O.ray_bounds_stack([0, 0, 0], [INF, INF, 1.0], [-1, -1, -1], [1, 1, 1], 1e6)
    assert t == F(1.0)
    # miss
    assert O.ray_bounds_stack([5, 0, -5], [INF, INF, 1.0], [-1, -1, -1], [1, 1, 1], 1e6) == -1.0
    # beyond maxt
    assert O.ray_bounds_stack([0, 0, -5], [INF, INF, 1.0], [-1, -1, -1], [1, 1, 1], 3.0) == -1.0


def test_ray_bounds_nan_semantics():
    """Origin exactly on a slab plane with a zero direction component: (b - o) * inf = 0*inf = NaN.
    GLSL min(x, y) = y < x ? y : x keeps x when y is NaN and returns NaN when x is NaN; the
    restatement must follow that rather than IEEE minNum."""
    # f.x = (1 - 1) * inf = NaN, n.x = (-1 - 1) * inf = -inf
    t = O.ray_bounds_stack([1.0, 0, -5], [INF, INF, 1.0], [-1, -1, -1], [1, 1, 1], 1e6)
    # tmax.x = max(NaN, -inf) = NaN (x < y false -> x); tmin.x = min(NaN, -inf) = -inf
    # t1 = min(min(NaN, min(inf, 6)), 1e6): min(inf,6)=6; min(NaN,6) = 6 (6 < NaN false -> NaN?)
    # GLSL: min(x=NaN, y=6) = (6 < NaN) ? 6 : NaN = NaN; then min(NaN, 1e6) = NaN
    # t1 >= t0 is false for NaN -> miss
    assert t == -1.0
    t2 = O.ray_bounds_stackless([-1, -1, -1], [1, 1, 1], [1.0, 0, -5], [INF, INF, 1.0], 1e-4, 1e6)
    # stackless: a = min(t0, t1) with t0.x = -inf, t1.x = NaN -> min(-inf, NaN) = -inf (NaN < -inf
    # false -> x); b.x = max(-inf, NaN) = -inf; tmax = min(-inf, ...) -> miss
    assert t2 == -1.0


def test_barycentrics_kat():
    u, v, w = O.barycentrics([0.25, 0.25, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert (u, v, w) == (F(0.5), F(0.25), F(0.25))
    u, v, w = O.barycentrics([1, 0, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0])
    assert (u, v, w) == (F(0.0), F(1.0), F(0.0))


def test_pcg_hash_and_sincos():
    # pcg_hash(0) from the published constants: state = 2891336453
    s = 2891336453
    word = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
    assert O.pcg_hash(0) == ((word >> 22) ^ word)
    for x in np.linspace(0, 0.999, 1000):
        s, c = O.sincos_turns(float(x))
        assert abs(s - np.sin(2 * np.pi * x)) < 4e-7 and abs(c - np.cos(2 * np.pi * x)) < 4e-7


# ---- whole traversal ----------------------------------------------------------------------

def _fp64_brute_force(vertices, tris, rays):
    """Closest t > 0 over ALL triangles in FP64 (Moller-Trumbore), independent of any BVH."""
    P = vertices["pos"][:, :3].astype(np.float64)
    A, B, C = P[tris[:, 0]], P[tris[:, 1]], P[tris[:, 2]]
    e1, e2 = B - A, C - A
    o = rays["o"].astype(np.float64)
    d = rays["d"].astype(np.float64)
    best_t = np.full(len(rays), np.inf)
    best_i = np.full(len(rays), -1)
    second = np.full(len(rays), np.inf)
    for i0 in range(0, len(rays), 256):
        oo, dd = o[i0:i0 + 256, None, :], d[i0:i0 + 256, None, :]
        p = np.cross(dd, e2[None])
        det = (e1[None] * p).sum(-1)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / det
            s = oo - A[None]
            u = (s * p).sum(-1) * inv
            q = np.cross(s, e1[None])
            v = (dd * q).sum(-1) * inv
            t = (e2[None] * q).sum(-1) * inv
        ok = (u >= 0) & (v >= 0) & (u + v <= 1) & (t > 0) & np.isfinite(t)
        t = np.where(ok, t, np.inf)
        order = np.argsort(t, axis=1)[:, :2]
        rows = np.arange(t.shape[0])
        best_t[i0:i0 + 256] = t[rows, order[:, 0]]
        best_i[i0:i0 + 256] = np.where(np.isfinite(t[rows, order[:, 0]]), order[:, 0], -1)
        second[i0:i0 + 256] = t[rows, order[:, 1]]
    return best_t, best_i, second


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_oracle_against_fp64_brute_force(layout):
    bufs = single_object("hf32", layout)
    v, t, n, e = bufs
    rays = np.concatenate([S.camera_rays(48, 48, **S.C1_CAMERA),
                           S.sphere_rays(2000, (-1.2, -1.2, -0.4), (1.2, 1.2, 0.8), seed=17)])
    h = oracle_scene(bufs, layout).closest(rays)
    bt, bi, second = _fp64_brute_force(v, t, rays)
    hit = h["t"] > 0
    # same hit / miss except grazing cases within float32 rounding of an edge or the near plane
    agree = hit == np.isfinite(bt)
    assert agree.mean() > 0.999, f"hit/miss agreement {agree.mean()}"
    both = hit & np.isfinite(bt)
    rel = np.abs(h["t"][both] - bt[both]) / bt[both]
    assert rel.max() < 2e-5
    # same triangle unless the two nearest FP64 hits are within float32 rounding of each other
    same = h["tri"][both] == bi[both]
    near_tie = (second[both] - bt[both]) <= 2e-5 * bt[both]
    assert (same | near_tie).all()
    assert both.sum() > 1000


def test_oracle_golden_results():
    """The oracle's results on a small seeded scene are pinned (tests/golden/oracle_hits_hf32.npz)."""
    g = np.load(Path(__file__).parent / "golden" / "oracle_hits_hf32.npz")
    bufs = single_object("hf32", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    rays = g["rays"].view(O.RAY_DTYPE)
    hits = osc.closest(rays, nthreads=2)
    assert np.array_equal(hits_u32(hits), hits_u32(g["hits"].view(O.HIT_DTYPE)))
    ao = osc.gi_raygen(rays, hits, 1, 3, 1e-3, 0.25)
    assert np.array_equal(ao.view(np.uint32), g["ao_rays"].view(np.uint32))
    assert np.array_equal(osc.anyhit(ao), g["occluded"])


def test_stack_and_stackless_agree():
    rays = S.sphere_rays(20000, (-1.1, -1.1, -0.3), (1.1, 1.1, 0.6), seed=23)
    hs = oracle_scene(single_object("hf64", R.STACK), R.STACK).closest(rays)
    hl = oracle_scene(single_object("hf64", R.STACKLESS), R.STACKLESS).closest(rays)
    assert (hs["t"] == hl["t"]).mean() > 0.9999
    assert (hs["tri"] == hl["tri"]).mean() > 0.999
    os_ = oracle_scene(single_object("hf64", R.STACK), R.STACK).anyhit(rays)
    ol = oracle_scene(single_object("hf64", R.STACKLESS), R.STACKLESS).anyhit(rays)
    assert (os_ == ol).mean() > 0.9999


def test_tie_rules_on_shared_edge():
    """Rays through the shared diagonal of heightfield quads hit two triangles at the same t.
    First-found keeps traversal order; lower-index keeps the smaller triangle index."""
    bufs = single_object("hf32", R.STACK)
    v, t, n, e = bufs
    osc = oracle_scene(bufs, R.STACK)
    # points on the v00-v11 diagonal of every quad, rays straight down
    P = v["pos"][:, :3]
    i00, i11 = t[:, 0], t[:, 2]
    mid = ((P[i00].astype(np.float64) + P[i11]) * 0.5).astype(np.float32)
    rays = np.zeros(len(mid), dtype=O.RAY_DTYPE)
    rays["o"] = mid + np.float32([0, 0, 2])
    rays["d"] = [0, 0, -1]
    rays["tmax"] = 1e6
    lo = osc.closest(rays, tie=O.ORC_TIE_LOWER_INDEX)
    ff = osc.closest(rays, tie=O.ORC_TIE_FIRST_FOUND)
    assert (lo["t"] == ff["t"]).all()
    assert (lo["tri"] <= ff["tri"]).all()
    assert (lo["tri"] < ff["tri"]).any(), "no tie exercised"


def _chain_bvh(depth: int):
    """A hand-made stack BVH whose every node has two hit internal children: node i -> (i+1, T),
    T a terminal node with two empty leaves; the last chain node points at a leaf triangle.
    Traversal pushes one node per level, so depth > 63 reaches the reference's push cap."""
    tri_v = np.zeros(3, dtype=R.VERTEX_DTYPE)
    tri_v["pos"] = [[-1, -1, 0, 1], [1, -1, 0, 1], [0, 1, 0, 1]]
    tris = np.array([[0, 1, 2, 0]], dtype=np.int32)
    N = depth + 2
    T = depth + 1
    nodes = np.zeros((N, 16), dtype=np.float32)
    w = nodes.view(np.int32)
    box = [-2, -2, -1, 0, 2, 2, 1, 0]
    for i in range(depth + 1):
        nodes[i, 0:8] = box
        nodes[i, 8:16] = box
        w[i, 3] = -1
        w[i, 7] = i + 1 if i < depth else T
        w[i, 11] = -1
        w[i, 15] = T
    # the last chain node: left child = leaf with the triangle
    w[depth, 3] = (0 << 4) | 1
    w[depth, 7] = 0
    nodes[T, 0:8] = box
    nodes[T, 8:16] = box
    w[T, 3] = 0        # empty leaves (start 0, count 0)
    w[T, 11] = 0
    ent = R.identity_entity(0, N)
    return tri_v, tris, nodes, ent


@pytest.mark.parametrize("depth,expect_hit", [(40, True), (70, False)])
def test_push_cap_reproduced(depth, expect_hit):
    v, t, n, e = _chain_bvh(depth)
    ok, msg = R.validate_scene(R.STACK, v, t, n, e)
    assert ok, msg
    osc = O.OracleScene(O.ORC_STACK, v, t, n, e)
    rays = np.zeros(1, dtype=O.RAY_DTYPE)
    rays["o"] = [0, 0, 0.5]
    rays["d"] = [0, 0, -1]
    rays["tmax"] = 1e6
    h = osc.closest(rays)
    assert (h["t"][0] > 0) == expect_hit
    if not expect_hit:
        assert h["iters"][0] == 64  # 63 pushes, then the 64th node's push is refused


# ---- GetData's albedo texture (TraverseBVHStack.glsl:436-447) --------------------------------

def _textured_hit(u, v, w, uvs):
    """A one-triangle scene whose vertices carry texture coordinates `uvs`, and a hit record with
    barycentrics (u, v, w) on it."""
    pos = np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0], [5, 5, 5], [6, 5, 5], [5, 6, 5]])
    vert = S.with_texcoords(S.make_vertices(pos, np.tile([0.0, 0.0, 1.0], (6, 1))),
                            np.concatenate([uvs, np.zeros((3, 2))]).astype(np.float32))
    b = R.build_bvh(vert, np.arange(6, dtype=np.uint32), np.array([0, 1], np.int32), 0, layout=R.STACKLESS)
    osc = O.OracleScene(O.ORC_STACKLESS, vert, b.tris, b.nodes, R.identity_entity(0, b.nodes.shape[0]))
    k = int(np.nonzero(b.tris[:, 3] == 0)[0][0])
    h = np.zeros(1, dtype=R.HIT_DTYPE)
    h["t"], h["u"], h["v"], h["w"], h["tri"], h["mesh"], h["entity"] = 1.0, u, v, w, k, 0, 0
    return osc, h


def test_texture_bilinear_known_answers():
    img = np.zeros((2, 2, 4), np.uint8)
    img[0, 0, :3], img[0, 1, :3], img[1, 0, :3], img[1, 1, :3] = 0, 255, 51, 102   # (row v, column u)
    alb = np.float32([[0.1, 0.2, 0.3]])
    uvs = np.float32([[0.25, 0.25], [0.75, 0.25], [0.25, 0.75]])
    # barycentric weight 1 on vertex A: uv = (0.25, 0.25), the centre of texel (0, 0)
    osc, h = _textured_hit(1.0, 0.0, 0.0, uvs)
    a = osc.hit_albedo(h, alb, [(img, 0, 0)], [0])
    np.testing.assert_array_equal(a, [[0.0, 0.0, 0.0]])
    osc, h = _textured_hit(0.0, 1.0, 0.0, uvs)                       # texel (1, 0): 255
    np.testing.assert_array_equal(osc.hit_albedo(h, alb, [(img, 0, 0)], [0]), [[1.0, 1.0, 1.0]])
    # halfway between the four texel centres: the mean (0 + 255 + 51 + 102) / 4 / 255
    osc, h = _textured_hit(0.0, 0.5, 0.5, uvs)                       # uv = (0.5, 0.5)
    got = osc.hit_albedo(h, alb, [(img, 0, 0)], [0])
    np.testing.assert_allclose(got, np.full((1, 3), (0 + 255 + 51 + 102) / 4 / 255), rtol=1e-6)
    # GL_REPEAT: u = 1.25 samples the same texel as u = 0.25; clamp keeps the edge texel
    uvs2 = np.float32([[1.25, 0.25], [0.75, 0.25], [0.25, 0.75]])
    osc, h = _textured_hit(1.0, 0.0, 0.0, uvs2)
    np.testing.assert_array_equal(osc.hit_albedo(h, alb, [(img, 0, 0)], [0]), [[0.0, 0.0, 0.0]])
    np.testing.assert_array_equal(osc.hit_albedo(h, alb, [(img, 0, 1)], [0]), [[1.0, 1.0, 1.0]])
    # sRGB: 255 -> 1, 0 -> 0, 51 -> 0.0331048 (IEC 61966-2-1)
    osc, h = _textured_hit(0.0, 0.0, 1.0, uvs)                       # texel (0, 1): 51
    np.testing.assert_allclose(osc.hit_albedo(h, alb, [(img, 1, 0)], [0]), [[0.0331048] * 3], rtol=1e-5)
    # a mesh without a texture, and a miss, keep the ModelColor
    np.testing.assert_array_equal(osc.hit_albedo(h, alb, [(img, 1, 0)], [-1]), alb)
    h2 = h.copy()
    h2["t"] = -1.0
    np.testing.assert_array_equal(osc.hit_albedo(h2, alb, [(img, 1, 0)], [0]), alb)
