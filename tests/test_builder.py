"""Our SAH builder against the reference constructor: byte-identical node and triangle buffers."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import scenes as S
from oracle import oracle as O

from .golden.make_golden import BUILDER_CASES, scene_hash, sha

GOLDEN = json.loads((Path(__file__).parent / "golden" / "builder.json").read_text())


@pytest.mark.parametrize("case", BUILDER_CASES, ids=[c[0] for c in BUILDER_CASES])
def test_builder_matches_reference_golden_hashes(case):
    """Hashes of the reference constructor's output (tests/golden/builder.json) — runs anywhere."""
    name, fn, stackless, leaf4, seed, off = case
    m = fn()
    g = GOLDEN[name]
    assert scene_hash(m) == g["scene_sha256"], "scene generator is not deterministic"
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, off,
                    layout=R.STACKLESS if stackless else R.STACK, leaf_size=4 if leaf4 else 2,
                    swap_children=seed is not None, swap_seed=seed or 0)
    assert b.nodes.shape[0] == g["n_nodes"]
    assert b.leaf_count == g["leaf_count"]
    assert b.split_fails == g["split_fails"]
    assert sha(b.tris) == g["tris_sha256"]
    assert sha(b.nodes) == g["nodes_sha256"]


@pytest.mark.parametrize("case", BUILDER_CASES, ids=[c[0] for c in BUILDER_CASES])
def test_oracle_builder_matches_reference_golden_hashes(case):
    """The oracle's restatement of the reference constructor (oracle/orc_build.cpp, which the CPU
    reference arm of the benchmark builds with) reproduces the reference's output hashes."""
    name, fn, stackless, leaf4, seed, off = case
    m = fn()
    g = GOLDEN[name]
    nodes, tris, info = O.build_bvh(m.vertices, m.indices, m.mesh_ids, off, stackless=stackless,
                                    leaf_size=4 if leaf4 else 2, swap_children=seed is not None,
                                    swap_seed=seed or 0)
    assert nodes.shape[0] == g["n_nodes"]
    assert info["leaf_count"] == g["leaf_count"] and info["split_fails"] == g["split_fails"]
    assert sha(tris) == g["tris_sha256"]
    assert sha(nodes) == g["nodes_sha256"]


needs_ref = pytest.mark.skipif(not O.ref_available(leaf4=True),
                               reason="reference tree not mounted (builder golden hashes still run)")


@needs_ref
@pytest.mark.parametrize("layout,leaf,seed", [(R.STACK, 2, None), (R.STACKLESS, 2, None),
                                              (R.STACKLESS, 2, 99), (R.STACK, 4, None),
                                              (R.STACKLESS, 4, 5)])
def test_builder_byte_identical_live_reference(layout, leaf, seed):
    m = S.icosphere_set(n_spheres=12, subdiv=3, seed=31, lo=(-2, -2, 0), hi=(2, 2, 1), ground=3.0)
    nodes, tris, info = O.ref_build_bvh(m.vertices, m.indices, m.mesh_ids, 123,
                                        stackless=layout == R.STACKLESS,
                                        swap_mode=0 if seed is None else 1, swap_seed=seed or 0,
                                        leaf4=leaf == 4)
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 123, layout=layout, leaf_size=leaf,
                    swap_children=seed is not None, swap_seed=seed or 0, n_threads=4)
    assert np.array_equal(b.nodes.view(np.uint32), nodes.view(np.uint32))
    assert np.array_equal(b.tris, tris)
    assert b.leaf_count == info["leaf_count"] and b.split_fails == info["split_fails"]
    o_nodes, o_tris, o_info = O.build_bvh(m.vertices, m.indices, m.mesh_ids, 123,
                                          stackless=layout == R.STACKLESS, leaf_size=leaf,
                                          swap_children=seed is not None, swap_seed=seed or 0)
    assert np.array_equal(o_nodes.view(np.uint32), nodes.view(np.uint32))
    assert np.array_equal(o_tris, tris) and o_info["split_fails"] == info["split_fails"]


@needs_ref
def test_builder_signed_zero_and_degenerate_geometry():
    """-0.0 coordinates, duplicate vertices and zero-area triangles: glm min/max argument order
    decides which zero survives; the midpoint fallback handles unsplittable nodes."""
    rng = np.random.default_rng(4)
    pos = rng.integers(-3, 4, size=(400, 3)).astype(np.float32) * 0.5
    pos[rng.random((400, 3)) < 0.2] = -0.0
    v = np.zeros(400, dtype=R.VERTEX_DTYPE)
    v["pos"][:, :3] = pos
    v["pos"][:, 3] = 1.0
    idx = rng.integers(0, 400, size=(300, 3)).astype(np.uint32)
    idx[:20, 1] = idx[:20, 0]  # degenerate triangles
    for layout in (R.STACK, R.STACKLESS):
        nodes, tris, info = O.ref_build_bvh(v, idx, None, 0, stackless=layout == R.STACKLESS)
        b = R.build_bvh(v, idx, None, 0, layout=layout)
        assert np.array_equal(b.nodes.view(np.uint32), nodes.view(np.uint32))
        assert np.array_equal(b.tris, tris)
        assert b.split_fails == info["split_fails"]
        o_nodes, o_tris, o_info = O.build_bvh(v, idx, None, 0, stackless=layout == R.STACKLESS)
        assert np.array_equal(o_nodes.view(np.uint32), nodes.view(np.uint32))
        assert np.array_equal(o_tris, tris) and o_info["split_fails"] == info["split_fails"]


def test_builder_multithreaded_equals_single_threaded():
    m = S.c1_heightfield_scene()
    a = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=R.STACK, n_threads=1)
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=R.STACK, n_threads=8)
    assert np.array_equal(a.nodes.view(np.uint32), b.nodes.view(np.uint32))
    assert np.array_equal(a.tris, b.tris)


def test_builder_rejects_bad_input():
    m = S.heightfield(16, seed=2)
    with pytest.raises(R.RqError):
        R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, leaf_size=16)
    with pytest.raises(R.RqError):
        R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, leaf_size=0 - 1)
    bad = m.indices.copy()
    bad[5] = m.vertices.shape[0]
    with pytest.raises(R.RqError):
        R.build_bvh(m.vertices, bad, m.mesh_ids, 0)
    with pytest.raises(R.RqError):  # a stack BVH needs a split root (the reference dereferences null)
        R.build_bvh(m.vertices, m.indices[:6], m.mesh_ids[:2], 0, layout=R.STACK)
    one = R.build_bvh(m.vertices, m.indices[:6], m.mesh_ids[:2], 0, layout=R.STACKLESS)
    assert one.nodes.shape[0] == 1 and one.leaf_count == 1


def test_stack_layout_structure():
    """Every internal child link points inside the used prefix; the tail is zero; every triangle
    appears in exactly one leaf."""
    m = S.heightfield(48, seed=8)
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=R.STACK, leaf_size=3)
    n = b.nodes
    used = b.n_nodes_used
    assert not n[used:].any()
    w = n[:used].view(np.int32)
    seen = np.zeros(b.tris.shape[0], dtype=np.int32)
    for side in (0, 8):
        kind = w[:, side + 3]
        link = w[:, side + 7]
        interior = kind == -1
        assert ((link[interior] > 0) & (link[interior] < used)).all()
        for p in kind[~interior]:
            seen[(p >> 4):(p >> 4) + (p & 15)] += 1
            assert 1 <= (p & 15) <= 3
    assert (seen == 1).all()
