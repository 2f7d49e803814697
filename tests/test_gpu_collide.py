"""rq_collide (AABB collision queries) against the CPU restatement: bit-exact records for both BVH2
layouts, with and without RQ_FLAG_REF_COMPAT, multi-entity scenes with transforms, host buffers,
degenerate / NaN / inverted boxes, and a million boxes on the 1.3M-triangle icosphere scene."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import mesh, oracle_scene, single_object

pytestmark = pytest.mark.gpu


def _boxes(name, n, seed, half_hi=0.08):
    p = mesh(name).positions()
    pick = (S.uniform(seed, 7, n) * p.shape[0]).astype(np.int64)
    b = S.query_boxes(n, (-0.12,) * 3, (0.12,) * 3, 0.002, half_hi, seed=seed)
    b[:, 0:3] += p[pick]
    b[:, 4:7] += p[pick]
    return b


def _edge_boxes():
    nan, inf = np.float32(np.nan), np.float32(np.inf)
    return np.array([
        [0.1, 0.1, 0.0, 1, 0.1, 0.1, 0.0, 1],          # a point
        [0.5, 0.5, 0.5, 1, -0.5, -0.5, -0.5, 1],       # inverted
        [nan, 0.0, 0.0, 1, 0.1, 0.1, 0.1, 1],          # NaN corner
        [-inf, -inf, -inf, 1, inf, inf, inf, 1],       # everything
        [-10, -10, -10, 1, 10, 10, 10, 1],             # encloses the scene
        [50, 50, 50, 1, 51, 51, 51, 1],                # far away
        [0.0, 0.0, -5.0, 1, 0.0, 0.0, 5.0, 1],         # a vertical segment
    ], dtype=np.float32)


def _to_dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", ["hf32", "ico2", "c1"])
@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
@pytest.mark.parametrize("ref", [False, True])
def test_collide_bit_exact(ctx, name, layout, ref):
    bufs = single_object(name, layout, leaf=4 if name == "hf32" else 2)
    osc = oracle_scene(bufs, layout)
    sc = ctx.scene(layout, *bufs)
    boxes = np.concatenate([_boxes(name, 60_000, seed=11), _edge_boxes()])
    flags = L.FLAG_REF_COMPAT if ref else 0
    want = osc.collide(boxes, flags=O.ORC_FLAG_REF_COMPAT if ref else 0)
    got = sc.collide(_to_dev(boxes), flags=flags).cpu().numpy()
    bad = np.nonzero((got != want).any(1))[0]
    assert bad.size == 0, (bad.size, bad[:5], got[bad[:5]], want[bad[:5]])
    assert 0.05 * len(boxes) < want[:, 0].sum() < 0.98 * len(boxes)
    # host buffers: the same records
    np.testing.assert_array_equal(sc.collide(boxes, flags=flags), want)
    assert ctx.device_status() == 0


def test_collide_multi_entity(ctx):
    """Three entities over two objects (one translated, one scaled): entities are tried in order
    and the box corners are moved by each entity's inverse matrix."""
    for layout in (R.STACK, R.STACKLESS):
        ri = R.RayIntersector(layout)
        ri.add_object(1, [mesh("hf32")])
        ri.add_object(2, [mesh("ico2")])
        T = np.eye(4)
        T[:3, 3] = [0.25, -0.5, 0.125]
        M = np.diag([1.5, 0.75, 1.0, 1.0])
        M[:3, 3] = [0.0, 0.0, 0.3]
        ri.push_entity(1)
        ri.push_entity(2, model=T)
        ri.push_entity(1, model=M)
        ri.buffer_entities()
        v, t, n, e = ri.global_buffers()
        osc = O.OracleScene({R.STACK: O.ORC_STACK, R.STACKLESS: O.ORC_STACKLESS}[layout], v, t, n, e)
        sc = ri.buffer_data(ctx)
        boxes = np.concatenate([_boxes("hf32", 30_000, seed=5), _boxes("ico2", 30_000, seed=6)])
        for flags in (0, L.FLAG_REF_COMPAT):
            want = osc.collide(boxes, flags=O.ORC_FLAG_REF_COMPAT if flags else 0)
            got = sc.collide(_to_dev(boxes), flags=flags).cpu().numpy()
            np.testing.assert_array_equal(got, want)
            assert len(np.unique(want[want[:, 0] == 1, 1])) >= 2


def test_collide_points_and_box_helpers(ctx):
    """Physics::CollidePoint (box = point -/+ 0.01) and CollideBox through the engine."""
    layout = R.STACKLESS
    bufs = single_object("hf32", layout)
    sc = ctx.scene(layout, *bufs)
    osc = oracle_scene(bufs, layout)
    p = mesh("hf32").positions()[::7]
    got = sc.collide_points(p)
    b = np.zeros((p.shape[0], 8), np.float32)
    b[:, 0:3] = p - np.float32(0.01)
    b[:, 4:7] = p + np.float32(0.01)
    np.testing.assert_array_equal(got, osc.collide(b))
    assert got[:, 0].all()          # every vertex lies on the surface
    assert sc.collide_box((-2, -2, -2), (2, 2, 2))
    assert not sc.collide_box((40, 40, 40), (41, 41, 41))


def test_collide_empty_and_unsupported(ctx):
    layout = R.STACK
    bufs = single_object("hf32", layout)
    sc = ctx.scene(layout, *bufs)
    assert sc.collide(np.zeros((0, 8), np.float32)).shape == (0, 4)
    sc.build_bvh8()
    o = R.engine._opts(layout=L.LAYOUT_BVH8Q)
    out = np.zeros((1, 4), np.int32)
    b = np.zeros((1, 8), np.float32)
    o.flags = L.FLAG_HOST_BUFFERS
    import ctypes as C
    st = L.lib().rq_collide(ctx.handle, sc.handle, b.ctypes.data, 1, out.ctypes.data, C.byref(o), None)
    assert st == L.RQ_ENOTSUP


def test_collide_large_scene(ctx):
    """One million boxes on the 1.3M-triangle icosphere scene: bit-exact on a seeded sample of
    100k boxes, and every record well-formed."""
    layout = R.STACK
    m = S.c2_icosphere_scene()
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=layout, leaf_size=2)
    bufs = (m.vertices, b.tris, b.nodes, R.identity_entity(0, b.nodes.shape[0]))
    sc = ctx.scene(layout, *bufs)
    p = m.positions()
    n = 1 << 20
    pick = (S.uniform(3, 7, n) * p.shape[0]).astype(np.int64)
    boxes = S.query_boxes(n, (-0.05,) * 3, (0.05,) * 3, 0.002, 0.03, seed=4)
    boxes[:, 0:3] += p[pick]
    boxes[:, 4:7] += p[pick]
    got = sc.collide(_to_dev(boxes)).cpu().numpy()
    hit = got[:, 0] == 1
    assert 0.05 < hit.mean() < 0.99
    assert np.all(got[~hit] == [0, -1, -1, -1])
    assert got[hit, 3].min() >= 0 and got[hit, 3].max() < m.n_tris and np.all(got[hit, 1] == 0)
    osc = oracle_scene(bufs, layout)
    sample = np.sort((S.uniform(8, 1, 100_000) * n).astype(np.int64))
    np.testing.assert_array_equal(got[sample], osc.collide(boxes[sample]))
