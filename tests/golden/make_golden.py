"""Regenerates the committed golden fixtures in tests/golden/.

    python tests/golden/make_golden.py

* builder.json — SHA-256 of the buffers the REFERENCE BVH constructor (compiled unmodified from
  the mounted reference tree by oracle/Makefile) produces for seeded scenes, plus the SHA-256 of
  the scene bytes themselves.  Needs the reference tree; the tests then check our builder against
  these hashes on any machine.
* oracle_hits_hf32.npz — closest-hit / any-hit results of the CPU restatement (oracle/) on a small
  seeded scene, so a change in the oracle's arithmetic on any platform is caught.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from candela_gb300 import scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

# (name, scene factory, stackless, leaf4, swap seed or None, tri offset)
BUILDER_CASES = [
    ("hf32_stack", lambda: S.heightfield(32, seed=5), False, False, None, 0),
    ("hf64_stackless", lambda: S.heightfield(64, seed=11), True, False, None, 0),
    ("hf64_stackless_swap1234", lambda: S.heightfield(64, seed=11), True, False, 1234, 0),
    ("hf64_stack_offset777", lambda: S.heightfield(64, seed=11), False, False, None, 777),
    ("ico2_stack_leaf4", lambda: S.icosphere_set(n_spheres=6, subdiv=2, seed=9, lo=(-1.5, -1.5, 0.0),
                                                  hi=(1.5, 1.5, 1.0), ground=3.0), False, True, None, 0),
    ("ico2_stackless", lambda: S.icosphere_set(n_spheres=6, subdiv=2, seed=9, lo=(-1.5, -1.5, 0.0),
                                                hi=(1.5, 1.5, 1.0), ground=3.0), True, False, None, 0),
    ("c1_stack", S.c1_heightfield_scene, False, False, None, 0),
]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def scene_hash(m) -> str:
    return hashlib.sha256(m.vertices.tobytes() + m.indices.tobytes() + m.mesh_ids.tobytes()).hexdigest()


def make_builder():
    if not O.ref_available(leaf4=True):
        raise SystemExit("the reference tree is needed to regenerate builder.json")
    out = {}
    for name, fn, stackless, leaf4, seed, off in BUILDER_CASES:
        m = fn()
        nodes, tris, info = O.ref_build_bvh(m.vertices, m.indices, m.mesh_ids, off,
                                            stackless=stackless, swap_mode=0 if seed is None else 1,
                                            swap_seed=seed or 0, leaf4=leaf4)
        out[name] = dict(scene_sha256=scene_hash(m), nodes_sha256=sha(nodes), tris_sha256=sha(tris),
                         n_nodes=int(nodes.shape[0]), n_tris=int(tris.shape[0]), **info)
    (HERE / "builder.json").write_text(json.dumps(out, indent=1) + "\n")


def make_oracle_hits():
    import candela_gb300 as R
    m = S.heightfield(32, seed=5)
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=R.STACK)
    ent = R.identity_entity(0, b.nodes.shape[0])
    osc = O.OracleScene(O.ORC_STACK, m.vertices, b.tris, b.nodes, ent)
    rays = np.concatenate([S.camera_rays(32, 32, **S.C1_CAMERA),
                           S.sphere_rays(1024, (-1.1, -1.1, -0.3), (1.1, 1.1, 0.6), seed=13)])
    hits = osc.closest(rays)
    ao = osc.gi_raygen(rays, hits, 1, 3, 1e-3, 0.25)
    occ = osc.anyhit(ao)
    np.savez_compressed(HERE / "oracle_hits_hf32.npz", rays=rays.view(np.uint8),
                        hits=hits.view(np.uint8), ao_rays=ao.view(np.uint8), occluded=occ)


if __name__ == "__main__":
    O.build()
    make_builder()
    make_oracle_hits()
    print("golden fixtures written to", HERE)
