"""Regenerates the committed golden fixtures in tests/golden/.

    python tests/golden/make_golden.py

* builder.json — SHA-256 of the buffers the REFERENCE BVH constructor (compiled unmodified from
  the mounted reference tree by oracle/Makefile) produces for seeded scenes, plus the SHA-256 of
  the scene bytes themselves.  Needs the reference tree; the tests then check our builder against
  these hashes on any machine.
* oracle_hits_hf32.npz — closest-hit / any-hit results of the CPU restatement (oracle/) on a small
  seeded scene, so a change in the oracle's arithmetic on any platform is caught.
* glsl_pins.json — SHA-256 of the outputs of the reference's own shaders compiled as C++
  (oracle/_ref/librefglsl.so, built by oracle/Makefile from the mounted reference tree) on seeded
  inputs: closest hits and occlusion on both layouts, closest hits over transformed and
  translucent entities, collision records, GetData's surface values, the diffuse and specular
  shading sums, the RT second-bounce loop and three frames of the probe update.  Needs the reference tree; tests/test_golden_glsl.py then checks that the
  restatement reproduces every one of them, on any machine.
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


def _canon_hits(h):
    """Closest-hit records in a form both implementations share: triangle, mesh and entity only
    where there is a hit (the shader leaves them unwritten otherwise)."""
    hit = h["t"] > 0
    return np.stack([h["t"].view(np.int32), h["u"].view(np.int32), h["v"].view(np.int32),
                     h["w"].view(np.int32), np.where(hit, h["tri"], -1), np.where(hit, h["mesh"], -1),
                     np.where(hit, h["entity"], -1)], 1).astype(np.int32)


def glsl_case_outputs(reference: bool) -> dict:
    """Outputs of the reference shaders compiled as C++ (reference=True) or of the restatement
    with the reference's conventions (first-found ties, the tri-0 test), on the same seeded inputs."""
    import candela_gb300 as R
    from candela_gb300.engine import probe_params, probe_volumes
    sys.path.insert(0, str(ROOT))
    from tests.helpers import mesh, single_object  # noqa: E402

    out = {}
    layouts = (("stack", R.STACK, O.ORC_STACK), ("stackless", R.STACKLESS, O.ORC_STACKLESS))
    edge = np.zeros(4, dtype=R.RAY_DTYPE)
    edge["o"] = [[0, 0, 5], [0, 0, 5], [0.1, 0.2, 3], [-3, 0.1, 0.05]]
    edge["d"] = [[np.nan, 0, -1], [0, 0, 0], [0, 0, -1], [1, 0, 0]]
    edge["tmax"] = 1e6
    for name in ("hf32", "ico2"):
        rays = np.concatenate([S.sphere_rays(4000, (-1.5, -1.5, -0.3), (1.5, 1.5, 1.2), seed=21),
                               S.camera_rays(48, 36, **S.C1_CAMERA), edge])
        for lname, lay, olay in layouts:
            bufs = single_object(name, lay)
            if reference:
                h = O.ref_glsl_closest(olay, *bufs, rays)
                occ = O.ref_glsl_occluded(olay, *bufs, rays)
            else:
                osc = O.OracleScene(olay, *bufs)
                h = osc.closest(rays, tie=O.ORC_TIE_FIRST_FOUND, flags=O.ORC_FLAG_REF_COMPAT)
                occ = osc.anyhit(rays)
            out[f"closest_{name}_{lname}"] = np.concatenate([_canon_hits(h), h["iters"][:, None]], 1)
            out[f"occluded_{name}_{lname}"] = occ.astype(np.uint8)
    # transformed, scaled and translucent entities (the shader's iteration output is the last
    # entity's, so iterations are left out here)
    ri = R.RayIntersector(R.STACK)
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    M = S.instance_transforms(8, (-3.0, -3.0, 0.0), (3.0, 3.0, 1.0), 0.4, 1.2, seed=5, anisotropic=0.3, tilt=0.1)
    for i in range(8):
        ri.push_entity(1 + (i % 2), model=M[i].astype(np.float64), translucency=0.5 if i % 4 == 1 else 0.0)
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    rays = np.concatenate([S.sphere_rays(4000, (-4.0, -4.0, -0.5), (4.0, 4.0, 2.0), seed=22), edge])
    for ignore in (False, True):
        if reference:
            h = O.ref_glsl_closest(O.ORC_STACK, v, t, n, e, rays, ignore_transparent=ignore)
        else:
            flags = O.ORC_FLAG_REF_COMPAT | (O.ORC_FLAG_IGNORE_TRANSPARENT if ignore else 0)
            h = O.OracleScene(O.ORC_STACK, v, t, n, e).closest(rays, tie=O.ORC_TIE_FIRST_FOUND, flags=flags)
        out[f"closest_entities_ignore{int(ignore)}"] = _canon_hits(h)
    # collision records on both layouts
    rng = np.random.default_rng(31)
    for lname, lay, olay in layouts:
        bufs = single_object("ico2", lay)
        pts = bufs[0]["pos"][:, :3][rng.integers(0, bufs[0].shape[0], 3000)]
        c = (pts + rng.uniform(-0.05, 0.05, size=pts.shape)).astype(np.float32)  # IEEE-exact draws
        hsz = rng.uniform(0.002, 0.04, size=(pts.shape[0], 1)).astype(np.float32)
        boxes = np.zeros((pts.shape[0], 8), dtype=np.float32)
        boxes[:, 0:3], boxes[:, 4:7] = c - hsz, c + hsz
        if reference:
            rec = O.ref_glsl_collide(olay, *bufs, boxes)
        else:
            rec = O.OracleScene(olay, *bufs).collide(boxes, flags=O.ORC_FLAG_REF_COMPAT)
        rec = np.where(rec[:, :1] == 1, rec, np.int32([[0, -1, -1, -1]])).astype(np.int32)
        out[f"collide_ico2_{lname}"] = rec
    # GetData: interpolated normal, the UV a textured mesh samples at (the harness texture() reports
    # (u, v, texture index)), the ModelColor of untextured meshes, emissive and alpha
    m = S.heightfield(32, seed=5)
    pos = m.positions().astype(np.float64)
    verts = S.with_texcoords(m.vertices, np.stack([pos[:, 0] * 1.7 + 0.3, pos[:, 1] * -2.1], 1))
    mids = (np.arange(m.n_tris) % 3).astype(np.int32)
    b = R.build_bvh(verts, m.indices, mids, 0, layout=R.STACK)
    ents = R.identity_entity(0, b.nodes.shape[0], emissive=0.25, alpha=0.75)
    gsc = O.OracleScene(O.ORC_STACK, verts, b.tris, b.nodes, ents)
    ghits = gsc.closest(S.camera_rays(64, 48, **S.C1_CAMERA))
    ghits = ghits[ghits["t"] > 0]
    gmodel = np.float32([[0.7, 0.6, 0.5], [0.2, 0.8, 0.4], [0.9, 0.9, 0.2]])
    textured = np.isin(ghits["mesh"], [0, 2])
    if reference:
        g = O.ref_glsl_getdata(verts, b.tris, ents, gmodel, [5, -1, 9], ghits)
    else:
        g = np.zeros((ghits.shape[0], 8), dtype=np.float32)
        g[:, :3] = gsc.hit_normal(ghits, 0)
        g[textured, 3:5] = gsc.hit_uv(ghits[textured])
        g[textured, 5] = np.where(ghits["mesh"][textured] == 0, 5.0, 9.0)
        g[~textured, 3:6] = gsc.hit_albedo(ghits[~textured], gmodel)
        g[:, 6], g[:, 7] = np.float32(0.25), np.float32(0.75)
    out["getdata_hf32"] = g
    # shading sums and the probe update, fed the restatement's traversal and surface data (their
    # own parity with the shader is the closest-hit / GetData pins)
    bufs = single_object("hf32", R.STACK)
    osc = O.OracleScene(O.ORC_STACK, *bufs)
    model = np.float32([[0.7, 0.6, 0.5], [0.2, 0.8, 0.4]])
    rays = S.sphere_rays(3000, (-1.2, -1.2, -0.2), (1.2, 1.2, 1.0), seed=23)
    hits = osc.closest(rays)
    hit = hits["t"] > 0
    alb = np.zeros((rays.shape[0], 4), dtype=np.float32)
    alb[hit, :3] = osc.hit_albedo(hits[hit], model)
    nrm = np.full((rays.shape[0], 3), -1.0, dtype=np.float32)
    nrm[hit] = osc.hit_normal(hits[hit], 0)
    lit = (np.arange(rays.shape[0]) % 3 != 0).astype(np.uint8)
    sun_dir, sun, sky, amb = (np.float32([0.3, 0.4, -0.866]), np.float32([4.0, 3.8, 3.5]),
                              np.float32([0.45, 0.6, 0.95]), np.float32([0.1, 0.1, 0.12]))
    if reference:
        out["shade_diffuse"] = O.ref_glsl_shade(0, rays, hits, alb, nrm, lit, sun_dir, sun, sky)
        out["shade_specular"] = O.ref_glsl_shade(1, rays, hits, alb, nrm, lit, sun_dir, sun, sky, amb, 0.35)
    else:
        out["shade_diffuse"] = osc.shade(rays, hits, lit, model, sun_dir, sun, sky * np.float32(2.0))
        out["shade_specular"] = osc.spec_shade(rays, hits, lit, model, 0.35, sun, sky, amb)
    # the RT second-bounce loop: GI rays from the hits above, three bounces, the reference's silent
    # misses; the bounce ray origins and FinalRadiance + Bounced
    emissive = bufs[3]["data"][:, 0].view(np.float32)
    sec = osc.gi_raygen(rays, hits, 1, 13, 0.05)
    gh = osc.closest(sec)
    glit = 1 - osc.anyhit(osc.shadow_raygen(sec, gh, sun_dir, 1e-3))
    fr = osc.shade(sec, gh, glit, model, sun_dir, sun, sky)[:, :3]
    live = gh["t"] > 0
    nb, ns = 3, len(sec)
    thr0 = np.zeros((ns, 3), dtype=np.float32)
    thr0[live] = osc.hit_albedo(gh[live], model)
    slot = np.zeros((ns, 20), dtype=np.float32)
    slot[:, 0:3], slot[:, 3:6] = sec["o"], sec["d"]
    slot[:, 6], slot[:, 7], slot[:, 8], slot[:, 9] = gh["t"], gh["u"], gh["v"], gh["w"]
    gn = np.full((ns, 3), -1.0, dtype=np.float32)
    gn[live] = osc.hit_normal(gh[live], 0)
    pr = (gn * sec["d"]).astype(np.float32)
    gn[(pr[:, 0] + pr[:, 1]) + pr[:, 2] > np.float32(0.0001)] *= np.float32(-1.0)
    slot[live, 10:13], slot[live, 13] = thr0[live], emissive[gh["entity"][live]]
    slot[:, 14:17], slot[:, 17:20] = gn, fr
    per = np.zeros((ns, nb, 15), dtype=np.float32)
    per[:, :, 3:7], per[:, :, 11:14] = -1.0, -1.0
    acc_in = np.zeros((ns, nb, 12), dtype=np.float32)
    acc_in[:, :, 0] = -1.0
    org = np.zeros((ns, nb, 3), dtype=np.float32)
    prev_r, prev_h = sec, gh
    for b in range(nb):
        br = osc.bounce_raygen(prev_r, prev_h, live, np.arange(ns, dtype=np.uint32), 13, b, 0.02, 1e6)
        bh = osc.closest(br)
        blit = 1 - osc.anyhit(osc.shadow_raygen(br, bh, sun_dir, 1e-3))
        hit = live & (bh["t"] > 0)
        org[live, b] = br["o"][live]
        per[live, b, 0:3] = br["d"][live]
        per[hit, b, 3], per[hit, b, 4], per[hit, b, 5], per[hit, b, 6] = (bh["t"][hit], bh["u"][hit],
                                                                          bh["v"][hit], bh["w"][hit])
        balb, bn = osc.hit_albedo(bh[hit], model), osc.hit_normal(bh[hit], 0)
        per[hit, b, 7:10], per[hit, b, 10], per[hit, b, 11:14] = balb, emissive[bh["entity"][hit]], bn
        per[:, b, 14] = blit
        acc_in[hit, b, 0], acc_in[hit, b, 1:4], acc_in[hit, b, 4] = bh["t"][hit], balb, emissive[bh["entity"][hit]]
        acc_in[hit, b, 5:8], acc_in[hit, b, 8:11], acc_in[hit, b, 11] = bn, br["d"][hit], blit[hit]
        prev_r, prev_h, live_next = br, bh, hit
        live = live_next
    traced = per[:, :, 0:3].any(2)
    if reference:
        bfr, borg = O.ref_glsl_bounce(slot, per, sun_dir, sun, sky)
    else:
        bfr, borg = O.bounce_accumulate(fr, thr0, acc_in, sun_dir, sun, sky, True), org
    out["bounce_loop"] = np.concatenate([bfr.view(np.int32),
                                         np.where(traced[:, :, None], borg, np.float32(0)).reshape(ns, -1).view(np.int32)], 1)
    origins = [(0.0, 0.0, 0.4), (0.07, -0.05, 0.42), (0.15, 0.02, 0.38)]
    sh, raw, pmap = probe_volumes(probe_params(grid=(8, 8, 4)))
    prev = origins[0]
    for k, org in enumerate(origins):
        p = probe_params(grid=(8, 8, 4), origin=org, prev_origin=prev, size=(1.2, 1.2, 0.6), seed=7 + k,
                         temporal=k < 2, sky_color=(0.4, 0.55, 0.9))
        prays = O.probe_raygen(p)
        ph = osc.closest(prays)
        phit = ph["t"] > 0
        palb = np.zeros((prays.shape[0], 4), dtype=np.float32)
        palb[phit, :3] = osc.hit_albedo(ph[phit], model)
        pn = np.full((prays.shape[0], 3), -1.0, dtype=np.float32)
        pn[phit] = osc.hit_normal(ph[phit], 0)
        plit = 1 - osc.anyhit(osc.shadow_raygen(prays, ph, np.array(p.sun_dir, dtype=np.float32), p.shadow_offset, 0))
        if reference:
            sh, raw, pmap = O.ref_glsl_probe(p, prays, ph, palb, pn, plit, sh, raw, pmap)
        else:
            sh, raw, pmap = osc.probe_shade(p, prays, ph, plit, model, sh, raw, pmap)
        out[f"probe_frame{k}"] = np.concatenate([sh.view(np.int32), raw.view(np.int32), pmap.view(np.int32)], 1)
        prev = org
    return out


def make_glsl_pins():
    if not O.ref_glsl_available():
        raise SystemExit("the reference tree is needed to regenerate glsl_pins.json")
    ref = glsl_case_outputs(reference=True)
    ours = glsl_case_outputs(reference=False)
    for k in ref:
        if sha(ref[k]) != sha(ours[k]):
            raise SystemExit(f"the restatement differs from the reference shader on {k}")
    (HERE / "glsl_pins.json").write_text(json.dumps({k: sha(v) for k, v in ref.items()}, indent=1) + "\n")


if __name__ == "__main__":
    O.build()
    make_builder()
    make_oracle_hits()
    make_glsl_pins()
    print("golden fixtures written to", HERE)
