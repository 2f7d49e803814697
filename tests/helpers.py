"""Shared scene set-up for the tests: seeded scenes, their BVHs, oracle views and device scenes."""
from __future__ import annotations

import functools

import numpy as np

import candela_gb300 as R
from candela_gb300 import scenes as S
from oracle import oracle as O

ORC_LAYOUT = {R.STACK: O.ORC_STACK, R.STACKLESS: O.ORC_STACKLESS}


@functools.lru_cache(maxsize=None)
def mesh(name: str) -> S.Mesh:
    if name == "c1":
        return S.c1_heightfield_scene()
    if name == "hf32":
        return S.heightfield(32, seed=5)
    if name == "hf64":
        return S.heightfield(64, seed=11)
    if name == "ico2":
        return S.icosphere_set(n_spheres=6, subdiv=2, seed=9, lo=(-1.5, -1.5, 0.0),
                               hi=(1.5, 1.5, 1.0), ground=3.0)
    if name == "c2":
        return S.c2_icosphere_scene()
    if name == "c4":
        return S.c4_icosphere_scene()
    raise KeyError(name)


@functools.lru_cache(maxsize=None)
def bvh(name: str, layout: int, leaf: int = 2) -> R.BVH:
    m = mesh(name)
    return R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=layout, leaf_size=leaf)


def single_object(name: str, layout: int, leaf: int = 2):
    """(vertices, tris, nodes, entities) of a one-object, one-identity-entity scene."""
    m = mesh(name)
    b = bvh(name, layout, leaf)
    return m.vertices, b.tris, b.nodes, R.identity_entity(0, b.nodes.shape[0])


def oracle_scene(bufs, layout):
    v, t, n, e = bufs
    return O.OracleScene(ORC_LAYOUT[layout], v, t, n, e)


def hits_u32(h: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(h).view(np.uint32).reshape(len(h), 8)


def assert_hits_identical(got, want, what=""):
    g = hits_u32(np.asarray(got))
    w = hits_u32(np.asarray(want))
    bad = np.nonzero((g != w).any(1))[0]
    if bad.size:
        i = bad[0]
        raise AssertionError(f"{what}: {bad.size} of {len(w)} hits differ; first at {i}: "
                             f"got {np.asarray(got)[i]} want {np.asarray(want)[i]}")


def hits_from_device(t) -> np.ndarray:
    """(n, 8) float32 torch tensor -> HIT_DTYPE numpy array."""
    a = t.detach().cpu().numpy()
    return np.ascontiguousarray(a).view(R.HIT_DTYPE).reshape(-1)


def rays_to_device(rays: np.ndarray):
    import torch
    return torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1)).cuda()


HIT_FIELDS = ("t", "u", "v", "w", "tri", "mesh", "entity")


def same_records(a, b) -> np.ndarray:
    """Per ray: t, u, v, w, triangle, mesh and entity bit-identical (iters not compared)."""
    a, b = np.asarray(a), np.asarray(b)
    same = np.ones(len(a), bool)
    for f in HIT_FIELDS:
        same &= a[f].view(np.uint32) == b[f].view(np.uint32)
    return same


def assert_equal_or_proven(got, want, osc, rays, flags=0, what="", max_frac=1e-3):
    """`got` (a BVH8q walk) equals `want` (the oracle's BVH2 walk) record for record, except on rays
    where a brute force over every triangle (the strict triangle test, no box tests) finds exactly
    `got`'s hit and `want` is a miss or a farther hit: there the reference's slab test rounded a node
    with the hit away, and the conservative BVH8 boxes kept it.  Returns the number of such rays."""
    same = same_records(got, want)
    bad = np.nonzero(~same)[0]
    if bad.size == 0:
        return 0
    assert bad.size <= max(1, max_frac * len(rays)), f"{what}: {bad.size} of {len(rays)} rays differ"
    brute, _ = osc.brute_closest(np.asarray(rays)[bad], flags=flags)
    g = np.asarray(got)[bad]
    w = np.asarray(want)[bad]
    proven = same_records(g, brute)
    assert proven.all(), (f"{what}: ray {bad[~proven][0]} differs from the brute force: got {g[~proven][0]} "
                          f"oracle {w[~proven][0]} brute {brute[~proven][0]}")
    assert np.all((w["t"] < 0) | (g["t"] <= w["t"])), what
    return int(bad.size)


def assert_occlusion_equal_or_proven(got, want, osc, rays, what="", max_frac=1e-3):
    """Occlusion bits equal, except rays that the BVH8q finds occluded where the oracle's walk does
    not, and for which a brute force over every triangle finds an occluder."""
    got, want = np.asarray(got), np.asarray(want)
    bad = np.nonzero(got != want)[0]
    if bad.size == 0:
        return 0
    assert bad.size <= max(1, max_frac * len(rays)), f"{what}: {bad.size} of {len(rays)} rays differ"
    assert np.all(got[bad] == 1), f"{what}: an occluder the oracle found was missed"
    _, occ = osc.brute_closest(np.asarray(rays)[bad])
    assert occ.all(), f"{what}: occlusion without an occluder"
    return int(bad.size)
