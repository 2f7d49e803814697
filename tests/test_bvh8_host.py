"""BVH8 derivation on the host: structure and conservative quantisation (every decoded child box
contains every triangle below it), every triangle exactly once, records bit-equal to the strict
arithmetic's edges and normal."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300.engine import build_bvh8_host

from .helpers import single_object


def _decode(node):
    p = node[:3].view(np.float32).astype(np.float64)
    e = np.array([(node[3] >> (8 * a)) & 0xFF for a in range(3)], dtype=np.int64)
    step = np.ldexp(1.0, (e - 127).astype(np.int32))
    q = node[8:20].view(np.uint8).reshape(6, 8).astype(np.float64)
    lo = p[:, None] + q[0:3] * step[:, None]
    hi = p[:, None] + q[3:6] * step[:, None]
    return lo, hi  # (3, 8)


def _walk(nodes8, recs, verts):
    """Yields (slot box lo, hi, triangle vertex array) for every non-empty slot."""
    P = verts["pos"][:, :3].astype(np.float64)
    below = {}

    def tris_under(i):
        if i in below:
            return below[i]
        nd = nodes8[i]
        imask = nd[3] >> 24
        meta = nd[6:8].view(np.uint8)
        out = []
        k = 0
        for s in range(8):
            if (imask >> s) & 1:
                out.extend(tris_under(int(nd[4]) + k))
                k += 1
            elif meta[s]:
                cnt = int(meta[s] >> 5)
                off = int(meta[s] & 31)
                out.extend(range(int(nd[5]) + off, int(nd[5]) + off + cnt))
        below[i] = out
        return out

    import sys
    sys.setrecursionlimit(10000)
    for i in range(nodes8.shape[0]):
        nd = nodes8[i]
        lo, hi = _decode(nd)
        imask = nd[3] >> 24
        meta = nd[6:8].view(np.uint8)
        k = 0
        for s in range(8):
            if (imask >> s) & 1:
                ts = tris_under(int(nd[4]) + k)
                k += 1
            elif meta[s]:
                cnt = int(meta[s] >> 5)
                off = int(meta[s] & 31)
                ts = list(range(int(nd[5]) + off, int(nd[5]) + off + cnt))
            else:
                continue
            yield lo[:, s], hi[:, s], ts


@pytest.mark.parametrize("name,layout,leaf", [("hf32", R.STACK, 2), ("hf64", R.STACKLESS, 2),
                                              ("ico2", R.STACK, 4), ("ico2", R.STACKLESS, 2)])
def test_bvh8_conservative_and_complete(name, layout, leaf):
    v, t, n, e = single_object(name, layout, leaf)
    nodes8, recs = build_bvh8_host(layout, n, t, v)
    assert recs.shape[0] == t.shape[0]
    ids = recs[:, 3].view(np.int32)
    assert np.array_equal(np.sort(ids), np.arange(t.shape[0]))  # every triangle exactly once
    # records: e1, e2, n equal the float32 arithmetic of RayTriangle
    P = v["pos"][:, :3]
    tr = t[ids]
    v0, v1, v2 = P[tr[:, 0]], P[tr[:, 1]], P[tr[:, 2]]
    e1 = (v1 - v0).astype(np.float32)
    e2 = (v2 - v0).astype(np.float32)
    nn = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1], e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                   e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], 1).astype(np.float32)
    assert np.array_equal(recs[:, 0:3], v0) and np.array_equal(recs[:, 4:7], e1)
    assert np.array_equal(recs[:, 8:11], e2) and np.array_equal(recs[:, 12:15], nn)
    assert np.array_equal(recs[:, 7].view(np.int32), tr[:, 3])
    # conservative boxes
    rec_tri_verts = np.stack([v0, v1, v2], 1).astype(np.float64)  # (M, 3, 3)
    checked = 0
    reachable = set()
    for lo, hi, ts in _walk(nodes8, recs, v):
        reachable.update(ts)
        pts = rec_tri_verts[ts].reshape(-1, 3)
        assert (pts >= lo[None, :]).all() and (pts <= hi[None, :]).all()
        checked += 1
    assert checked >= nodes8.shape[0]
    assert reachable == set(range(recs.shape[0])), "a triangle record is not reachable via any slot"


def test_bvh8_rejects_big_leaves():
    v, t, n, e = single_object("hf32", R.STACK)
    b = R.build_bvh(v, t[:, :3].ravel().astype(np.uint32) if False else
                    np.asarray(__import__("candela_gb300").scenes.heightfield(32, seed=5).indices),
                    None, 0, layout=R.STACK, leaf_size=6)
    with pytest.raises(R.RqError):
        build_bvh8_host(R.STACK, b.nodes, b.tris, v)
