"""Host-side fault injection: malformed scene buffers are rejected before anything reaches a device
(rq_scene_validate runs the checks of rq_scene_create without a GPU)."""
import numpy as np
import pytest

import candela_gb300 as R

from .helpers import single_object


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_valid_scene_passes(layout):
    ok, msg = R.validate_scene(layout, *single_object("hf32", layout))
    assert ok, msg


def _corrupt(layout, fn):
    v, t, n, e = (x.copy() for x in single_object("hf32", layout))
    fn(v, t, n, e)
    return R.validate_scene(layout, v, t, n, e)


def test_vertex_index_out_of_range():
    ok, msg = _corrupt(R.STACK, lambda v, t, n, e: t.__setitem__((7, 1), v.shape[0]))
    assert not ok and "vertex index" in msg
    ok, msg = _corrupt(R.STACK, lambda v, t, n, e: t.__setitem__((7, 2), -3))
    assert not ok


def test_stack_child_link_out_of_range():
    def f(v, t, n, e):
        w = n.view(np.int32)
        i = np.nonzero(w[:, 3] == -1)[0][3]
        w[i, 7] = n.shape[0] + 5
    ok, msg = _corrupt(R.STACK, f)
    assert not ok and "child link" in msg


def test_stack_leaf_range_out_of_bounds():
    def f(v, t, n, e):
        w = n.view(np.int32)
        i = np.nonzero(w[:, 11] != -1)[0][0]
        w[i, 11] = ((t.shape[0] - 1) << 4) | 3
    ok, msg = _corrupt(R.STACK, f)
    assert not ok and "leaf" in msg


def test_stackless_escape_and_successor():
    def esc(v, t, n, e):
        n.view(np.int32)[4, 7] = 10 ** 6
    ok, msg = _corrupt(R.STACKLESS, esc)
    assert not ok and "escape" in msg

    def last_internal(v, t, n, e):
        n.view(np.int32)[-1, 3] = -1
    ok, msg = _corrupt(R.STACKLESS, last_internal)
    assert not ok and "successor" in msg


def test_entity_range_outside_nodes():
    ok, msg = _corrupt(R.STACK, lambda v, t, n, e: e.__setitem__("node_count", n.shape[0] + 1))
    assert not ok and "entity" in msg
    ok, msg = _corrupt(R.STACK, lambda v, t, n, e: e.__setitem__("node_offset", -1))
    assert not ok


def test_wrong_layout_rejected():
    v, t, n, e = single_object("hf32", R.STACK)
    ok, msg = R.validate_scene(7, v, t, n, e)
    assert not ok


def test_intersector_mirror_rejects_unknown_object():
    ri = R.RayIntersector(R.STACK)
    with pytest.raises(KeyError):
        ri.push_entity(42)
