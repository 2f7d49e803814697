"""GPU BVH build (rq_build_bvh_gpu) against the host builder, which is byte-identical to the
reference constructor: every buffer byte, the used-node count, the leaf count and the midpoint
fallback count must be equal."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import scenes as S

from .helpers import mesh

pytestmark = pytest.mark.gpu


def _same(ctx, v, idx, mid, **kw):
    h = R.build_bvh(v, idx, mid, **kw)
    g = R.build_bvh(v, idx, mid, ctx=ctx, **kw)
    assert g.nodes.shape == h.nodes.shape
    assert np.array_equal(g.nodes.view(np.uint32), h.nodes.view(np.uint32)), kw
    assert np.array_equal(g.tris, h.tris), kw
    assert (g.n_nodes_used, g.leaf_count, g.split_fails) == (h.n_nodes_used, h.leaf_count, h.split_fails), kw
    return h


@pytest.mark.parametrize("name", ["hf32", "hf64", "ico2", "c1"])
@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_gpu_build_equals_host(ctx, name, layout):
    m = mesh(name)
    for leaf in (1, 2, 4):
        _same(ctx, m.vertices, m.indices, m.mesh_ids, layout=layout, leaf_size=leaf, tri_offset=7 * leaf)
    if layout == R.STACKLESS:
        for seed in (0, 12345):
            _same(ctx, m.vertices, m.indices, m.mesh_ids, layout=layout, swap_children=True, swap_seed=seed)


def test_gpu_build_small_degenerate_and_signed_zeros(ctx):
    # small scenes: one subtree (<= 256 triangles) and a single stackless leaf
    m = S.heightfield(8, seed=3)
    _same(ctx, m.vertices, m.indices, m.mesh_ids, layout=R.STACK)
    _same(ctx, m.vertices, m.indices[:6], m.mesh_ids[:2], layout=R.STACKLESS)
    # every triangle at the same place: every split falls back to the midpoint
    v = S.heightfield(4, seed=1).vertices.copy()
    idx = np.tile(np.array([0, 1, 2], dtype=np.uint32), 3000)
    h = _same(ctx, v, idx, None, layout=R.STACK)
    assert h.split_fails > 0
    _same(ctx, v, idx, None, layout=R.STACKLESS, swap_children=True, swap_seed=5)
    # signed zeros: flat ground at z = +-0 and x = +-0 columns (order decides which zero survives)
    m = S.heightfield(48, seed=7)
    v = m.vertices.copy()
    pos = v["pos"]
    pos[:, 2] = np.where(np.arange(len(v)) % 3 == 0, -0.0, 0.0).astype(np.float32)
    pos[::5, 0] = np.float32(-0.0)
    pos[1::5, 0] = np.float32(0.0)
    for layout in (R.STACK, R.STACKLESS):
        _same(ctx, v, m.indices, m.mesh_ids, layout=layout)


def test_gpu_build_large_scene(ctx):
    m = mesh("c2")
    h = _same(ctx, m.vertices, m.indices, m.mesh_ids, layout=R.STACK)
    assert h.tris.shape[0] == 1310722
