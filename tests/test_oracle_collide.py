"""The CPU restatement of the reference's AABB collision queries (Collide.comp with
Intersectors/Include/CollideBVHStack.glsl and CollideBVHStackless.glsl), checked on its own:
known answers for the separating-axis test (including the reference's repeated axis), the
no-collision record, and exact-geometry properties on whole scenes against an independent FP64
brute force."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import ORC_LAYOUT, mesh, oracle_scene, single_object

# A triangle and a box that the nine distinct edge axes separate (cross(u1, f2) is the separating
# axis) but the reference's axis set, which repeats cross(u2, f2) in slot 5, does not.  All values
# are dyadic, so float32 holds them exactly.
AXIS_TRI = np.array([[1.0, 0.75, 0.625], [-0.5, -1.0, 0.75], [-0.125, 0.75, -0.375]])
AXIS_BOX = np.array([0.875, 0.625, 0.0625, 1.0, 1.125, 0.875, 0.1875, 1.0], dtype=np.float32)


def _one_triangle_scene(layout, tri=AXIS_TRI, mesh_id=7):
    """The triangle plus a far-away second one (mesh 99; the stack layout needs two leaves).
    Returns the oracle scene and the triangle's index in the BVH's triangle order."""
    pos = np.concatenate([np.asarray(tri, dtype=np.float32),
                          np.float32([[100, 100, 100], [101, 100, 100], [100, 101, 100]])])
    v = S.make_vertices(pos, np.tile([0.0, 0.0, 1.0], (6, 1)))
    b = R.build_bvh(v, np.arange(6, dtype=np.uint32), np.array([mesh_id, 99], dtype=np.int32), 0,
                    layout=layout, leaf_size=1)
    k = int(np.nonzero(b.tris[:, 3] == mesh_id)[0][0])
    return O.OracleScene(ORC_LAYOUT[layout], v, b.tris, b.nodes,
                         R.identity_entity(0, b.nodes.shape[0])), k


def _edge_axes(f, ref):
    u = np.eye(3)
    c = lambda a, b: np.cross(np.broadcast_to(a, b.shape), b)  # noqa: E731
    return [c(u[0], f[0]), c(u[0], f[1]), c(u[0], f[2]), c(u[1], f[0]), c(u[1], f[1]),
            c(u[2], f[2]) if ref else c(u[1], f[2]), c(u[2], f[0]), c(u[2], f[1]), c(u[2], f[2])]


def _margin(tri, bmin, bmax, kind):
    """Largest separation over the axes, FP64, triangles (T, 3, 3) against one box.  kind 'ref'
    / 'fixed': the reference's form (nine edge axes with the full box extent as the radius, axis
    set with or without the repeated slot); 'exact': the true 13-axis test (box faces, triangle
    normal, nine edge axes, half extents).  > 0 means separated."""
    c = (bmin + bmax) / 2.0
    v = tri - c
    f = [v[:, 1] - v[:, 0], v[:, 2] - v[:, 1], v[:, 0] - v[:, 2]]
    if kind == "exact":
        e = (bmax - bmin) / 2.0
        axes = _edge_axes(f, False) + [np.broadcast_to(a, f[0].shape) for a in np.eye(3)]
        axes.append(np.cross(f[0], f[1]))
    else:
        e = bmax - bmin
        axes = _edge_axes(f, kind == "ref")
    best = np.full(tri.shape[0], -np.inf)
    for a in axes:
        p = np.einsum("tkj,tj->tk", v, a)
        r = (e[None, :] * np.abs(a)).sum(1)
        best = np.maximum(best, np.maximum(-p.max(1), p.min(1)) - r)
    return best


def test_box_triangle_axis_known_answer():
    for layout in (R.STACK, R.STACKLESS):
        osc, k = _one_triangle_scene(layout)
        # the reference's axis set finds no separating axis: collision with mesh 7 (one-triangle
        # leaves: index 0 within the leaf on the stack layout, the global index otherwise)
        got = osc.collide(AXIS_BOX[None], flags=O.ORC_FLAG_REF_COMPAT)
        np.testing.assert_array_equal(got, [[1, 0, 7, 0 if layout == R.STACK else k]])
        # the nine distinct axes separate them: no collision, the {0, -1, -1, -1} record
        got = osc.collide(AXIS_BOX[None])
        np.testing.assert_array_equal(got, [[0, -1, -1, -1]])
    # the FP64 forms agree on which axis set separates
    tri = AXIS_TRI[None]
    assert _margin(tri, AXIS_BOX[:3].astype(np.float64), AXIS_BOX[4:7].astype(np.float64), "ref")[0] < 0
    assert _margin(tri, AXIS_BOX[:3].astype(np.float64), AXIS_BOX[4:7].astype(np.float64), "fixed")[0] > 0


def test_collide_containing_far_and_degenerate_boxes():
    tri = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    for layout in (R.STACK, R.STACKLESS):
        osc, k = _one_triangle_scene(layout, tri, mesh_id=3)
        boxes = np.array([
            [-0.5, -0.5, -0.5, 1, 1.5, 1.5, 0.5, 1],     # contains the triangle
            [0.2, 0.2, -0.01, 1, 0.3, 0.3, 0.01, 1],     # inside the face
            [5.0, 5.0, 5.0, 1, 6.0, 6.0, 6.0, 1],        # far away
            [0.2, 0.2, 0.5, 1, 0.3, 0.3, 0.6, 1],        # above the face
            [0.25, 0.25, 0.0, 1, 0.25, 0.25, 0.0, 1],    # a point on the face
        ], dtype=np.float32)
        got = osc.collide(boxes)
        np.testing.assert_array_equal(got[:, 0], [1, 1, 0, 0, 1])
        np.testing.assert_array_equal(got[got[:, 0] == 1], [[1, 0, 3, k]] * 3)
        np.testing.assert_array_equal(got[got[:, 0] == 0], [[0, -1, -1, -1]] * 2)
        assert osc.collide(np.zeros((0, 8), np.float32)).shape == (0, 4)


def _scene_boxes(name, n, seed):
    """Boxes around the surface: each centred within 0.12 of a random vertex."""
    p = mesh(name).positions()
    pick = (S.uniform(seed, 7, n) * p.shape[0]).astype(np.int64)
    b = S.query_boxes(n, (-0.12,) * 3, (0.12,) * 3, 0.004, 0.08, seed=seed)
    b[:, 0:3] += p[pick]
    b[:, 4:7] += p[pick]
    return b


@pytest.mark.parametrize("name", ["hf32", "ico2"])
@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_collide_exact_geometry_properties(name, layout):
    """Against an FP64 brute force over every triangle: a reported triangle passes the
    reference's own (conservative) test; a box that truly cuts a triangle always collides; a box
    reported free truly cuts no triangle."""
    bufs = single_object(name, layout)
    osc = oracle_scene(bufs, layout)
    boxes = _scene_boxes(name, 2000, seed=17)
    got = osc.collide(boxes)
    v = bufs[0]["pos"][:, :3].astype(np.float64)
    tri = v[bufs[1][:, :3].astype(np.int64)]
    n_true = 0
    for i, b in enumerate(boxes.astype(np.float64)):
        bmin, bmax = b[:3], b[4:7]
        exact = _margin(tri, bmin, bmax, "exact")
        if got[i, 0]:
            k = got[i, 3]
            assert 0 <= k < tri.shape[0]
            assert _margin(tri[k:k + 1], bmin, bmax, "fixed")[0] <= 1e-5, i
            assert got[i, 2] == bufs[1][k, 3]
        else:
            assert np.all(got[i, 1:] == -1)
            assert exact.min() > -1e-5, (i, exact.min())
        if exact.min() < -1e-5:
            n_true += 1
            assert got[i, 0] == 1, i
    # the workload exercises both outcomes
    assert 0.1 * len(boxes) < n_true < 0.9 * len(boxes)
    assert 0.1 * len(boxes) < got[:, 0].sum() < 0.95 * len(boxes)


def test_collide_ref_compat_leaf_index_and_entities():
    """RQ_FLAG_REF_COMPAT on the stack layout reports the index within the leaf; the stackless
    walk reports the global index either way.  Entities are tried in order and a translated
    entity moves the query box by its inverse matrix."""
    for layout in (R.STACK, R.STACKLESS):
        bufs = single_object("hf32", layout, leaf=4)
        osc = oracle_scene(bufs, layout)
        boxes = _scene_boxes("hf32", 2000, seed=3)
        ref = osc.collide(boxes, flags=O.ORC_FLAG_REF_COMPAT)
        hit = ref[:, 0] == 1
        assert hit.sum() > 100
        if layout == R.STACK:
            assert ref[hit, 3].max() < 4 and ref[hit, 3].min() >= 0
        else:
            assert ref[hit, 3].max() >= 4
    ri = R.RayIntersector(R.STACK)
    ri.add_object(1, [mesh("hf32")])
    T = np.eye(4)
    T[:3, 3] = [4.0, 0.0, 0.0]
    ri.push_entity(1)
    ri.push_entity(1, model=T)
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    osc = O.OracleScene(O.ORC_STACK, v, t, n, e)
    boxes = _scene_boxes("hf32", 500, seed=9)
    a = osc.collide(boxes)
    shifted = boxes.copy()
    shifted[:, [0, 4]] += np.float32(4.0)
    b = osc.collide(shifted)
    back = shifted.copy()
    back[:, [0, 4]] -= np.float32(4.0)   # what entity 1's inverse matrix does to the corners
    c = osc.collide(back)
    assert a[:, 0].sum() > 50
    assert np.all(a[a[:, 0] == 1, 1] == 0) and np.all(b[b[:, 0] == 1, 1] == 1)
    np.testing.assert_array_equal(b[:, 0], c[:, 0])
    np.testing.assert_array_equal(b[:, 2:], c[:, 2:])


@pytest.mark.skipif(not O.ref_physics_available(), reason="reference source tree not mounted")
@pytest.mark.parametrize("name", ["hf32", "ico2"])
def test_collide_pinned_to_reference_physics(name):
    """The stackless restatement with the reference's axis set (RQ_FLAG_REF_COMPAT) against the
    reference's own host walk, Physics::CollideBox (Physics.cpp), compiled from its source: the
    same collided flag for every box, with an identity entity and two translated ones (translations
    are exact, so glm's pairwise matrix sum and the GLSL left-to-right sum agree)."""
    ri = R.RayIntersector(R.STACKLESS)
    ri.add_object(1, [mesh(name)])
    ri.push_entity(1)
    for dx in (3.0, -5.0):
        T = np.eye(4)
        T[:3, 3] = [dx, 0.5, 0.25]
        ri.push_entity(1, model=T)
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    osc = O.OracleScene(O.ORC_STACKLESS, v, t, n, e)
    boxes = _scene_boxes(name, 4000, seed=21)
    shifted = boxes.copy()
    shifted[:, [0, 4]] += np.float32(3.0)
    shifted[:, [1, 5]] += np.float32(0.5)
    shifted[:, [2, 6]] += np.float32(0.25)
    for bx in (boxes, shifted):
        ref = O.ref_collide_boxes(v, t, n, e, bx)
        ours = osc.collide(bx, flags=O.ORC_FLAG_REF_COMPAT)[:, 0]
        np.testing.assert_array_equal(ours, ref)
        assert 0.1 < ref.mean() < 0.95
