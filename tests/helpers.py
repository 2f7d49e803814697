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
