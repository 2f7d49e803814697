"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes wrappers of the checkers built by oracle/Makefile:
  * liboracle.so  — CPU restatement of the reference traversal (rq_oracle.cpp);
  * librefbvh.so  — the reference BVH constructor compiled unmodified (only where the reference
                    source tree is mounted; absent on the GPU hosts).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "liboracle.so"
REF_SO = HERE / "_ref" / "librefbvh.so"
REF_LEAF4_SO = HERE / "_ref" / "librefbvh_leaf4.so"
REF_PHYSICS_SO = HERE / "_ref" / "librefphysics.so"
REF_GLSL_SO = HERE / "_ref" / "librefglsl.so"
# Where the reference source tree is: RQ_REFERENCE_ROOT, else the location the last reference build
# recorded (oracle/_ref/REFERENCE_ROOT); None where it is not mounted (the GPU hosts).
_ROOT_NOTE = HERE / "_ref" / "REFERENCE_ROOT"


def reference_root() -> Path | None:
    env = os.environ.get("RQ_REFERENCE_ROOT")
    if env:
        return Path(env)
    if _ROOT_NOTE.exists():
        return Path(_ROOT_NOTE.read_text().strip())
    return None

RAY_DTYPE = np.dtype([("o", "<f4", (3,)), ("tmin", "<f4"), ("d", "<f4", (3,)), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("w", "<f4"),
                      ("tri", "<i4"), ("mesh", "<i4"), ("entity", "<i4"), ("iters", "<i4")])

ORC_STACK, ORC_STACKLESS = 0, 1
ORC_TIE_FIRST_FOUND, ORC_TIE_LOWER_INDEX = 0, 1
ORC_FLAG_REF_COMPAT, ORC_FLAG_IGNORE_TRANSPARENT = 1, 2


def build(reference: bool | None = None, reference_root: str | os.PathLike | None = None) -> None:
    """Builds liboracle.so; also the reference checkers (oracle/_ref) when the reference source tree
    is given (reference_root, RQ_REFERENCE_ROOT or the location recorded by an earlier build) and
    present.  The location is recorded in oracle/_ref/REFERENCE_ROOT for later sessions."""
    root = Path(reference_root) if reference_root else reference_root_or_none()
    have = root is not None and (root / "Source" / "Core" / "BVH" / "BVHConstructor.cpp").exists()
    if reference is None:
        reference = have
    if reference and not have:
        raise FileNotFoundError("the reference source tree is not available: set RQ_REFERENCE_ROOT")
    targets = ["oracle"] + (["ref"] if reference else [])
    args = ["make", "-s", "-C", str(HERE), *targets] + ([f"REF={root}"] if reference else [])
    subprocess.run(args, check=True)
    if reference:
        _ROOT_NOTE.parent.mkdir(parents=True, exist_ok=True)
        _ROOT_NOTE.write_text(str(root))


def reference_root_or_none() -> Path | None:
    return reference_root()


class OrcScene(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("n_nodes", C.c_int64), ("tris", C.c_void_p),
                ("verts", C.c_void_p), ("ents", C.c_void_p), ("n_ents", C.c_int32),
                ("layout", C.c_int32)]


class OrcMaterials(C.Structure):
    _fields_ = [("albedo", C.c_void_p), ("n_albedo", C.c_int32), ("n_mesh_tex", C.c_int32),
                ("mesh_tex", C.c_void_p), ("tex", C.c_void_p), ("texels", C.c_void_p)]


def materials(albedo, textures=None, mesh_texture=None):
    """orc_materials for ModelColors (n, 3) and optional textures (list of (rgba8 (H, W, 4), srgb,
    wrap)) with a texture index per mesh.  Returns (struct, arrays to keep alive)."""
    alb = np.ascontiguousarray(albedo, dtype=np.float32).reshape(-1, 3)
    keep = [alb]
    m = OrcMaterials(alb.ctypes.data, alb.shape[0], 0, None, None, None)
    if textures:
        desc, texels, off = [], [], 0
        for img, srgb, wrap in textures:
            img = np.ascontiguousarray(img, dtype=np.uint8)
            h, w = img.shape[:2]
            desc.append([off, w, h, int(srgb) | (int(wrap) << 1)])
            texels.append(img.reshape(-1, 4).copy().view(np.uint32).ravel())
            off += w * h
        d = np.ascontiguousarray(desc, dtype=np.int32)
        tx = np.ascontiguousarray(np.concatenate(texels), dtype=np.uint32)
        mt = np.ascontiguousarray(mesh_texture, dtype=np.int32)
        keep += [d, tx, mt]
        m.n_mesh_tex, m.mesh_tex, m.tex, m.texels = mt.size, mt.ctypes.data, d.ctypes.data, tx.ctypes.data
    return m, keep


class OrcProbeParams(C.Structure):
    """orc_probe_params (the layout of rq_probe_params)."""
    _fields_ = [("grid", C.c_int32 * 3), ("origin", C.c_float * 3), ("prev_origin", C.c_float * 3),
                ("size", C.c_float * 3), ("seed", C.c_uint32), ("temporal", C.c_int32), ("normal_mode", C.c_int32),
                ("shadow_rays", C.c_int32), ("shadow_offset", C.c_float), ("ray_tmax", C.c_float),
                ("sun_dir", C.c_float * 3), ("sun_color", C.c_float * 3), ("sky_color", C.c_float * 3)]


def probe_params(p) -> OrcProbeParams:
    """OrcProbeParams holding the bytes of a structure with rq_probe_params' layout."""
    b = bytes(p)
    assert len(b) == C.sizeof(OrcProbeParams)
    return OrcProbeParams.from_buffer_copy(b)


def probe_count(p) -> int:
    return int(p.grid[0]) * int(p.grid[1]) * int(p.grid[2])


def probe_raygen(p, nthreads=None):
    """One ray per probe (UpdateRadianceProbes.glsl:410-427): RAY_DTYPE records, probe-major."""
    q = probe_params(p)
    out = np.empty(probe_count(q), dtype=RAY_DTYPE)
    orc().orc_probe_raygen(C.byref(q), nthreads or os.cpu_count() or 1, _p(out))
    return out


def probe_direction(seed, ids):
    """The probe ray direction of each probe index (normalised LambertBRDF of the hash samples)."""
    ii = np.ascontiguousarray(ids, dtype=np.uint32)
    out = np.empty((ii.shape[0], 3), dtype=np.float32)
    orc().orc_probe_direction(seed & 0xFFFFFFFF, _p(ii), ii.shape[0], _p(out))
    return out


_orc = None


def orc() -> C.CDLL:
    global _orc
    if _orc is None:
        if not ORACLE_SO.exists():
            build(reference=False)
        L = C.CDLL(str(ORACLE_SO))
        P, I64, I32 = C.c_void_p, C.c_int64, C.c_int32
        sp = C.POINTER(OrcScene)
        L.orc_closest.argtypes = [sp, P, I64, P, C.c_int, C.c_int, C.c_int, P]
        L.orc_anyhit.argtypes = [sp, P, I64, P, C.c_int, P, P]
        L.orc_ray_triangle.argtypes = [P] * 6
        L.orc_ray_bounds_stack.argtypes = [P, P, P, P, C.c_float]
        L.orc_ray_bounds_stack.restype = C.c_float
        L.orc_ray_bounds_stackless.argtypes = [P, P, P, P, C.c_float, C.c_float]
        L.orc_ray_bounds_stackless.restype = C.c_float
        L.orc_barycentrics.argtypes = [P] * 5
        L.orc_gi_raygen.argtypes = [sp, P, P, I64, I32, C.c_uint32, C.c_float, C.c_float, I32,
                                    C.c_int, P]
        L.orc_shade.argtypes = [sp, P, P, I64, P, C.POINTER(OrcMaterials), P, P, P, I32, C.c_int, P]
        L.orc_hit_albedo.argtypes = [sp, P, I64, C.POINTER(OrcMaterials), C.c_int, P]
        L.orc_hit_normal.argtypes = [sp, P, I64, I32, P]
        L.orc_hit_uv.argtypes = [sp, P, I64, P]
        L.orc_spec_raygen.argtypes = [sp, P, P, I64, C.c_uint32, C.c_float, C.c_float, I32, C.c_int, P]
        L.orc_spec_direction.argtypes = [P, P, I64, C.c_float, C.c_uint32, P, P]
        L.orc_spec_shade.argtypes = [sp, P, P, I64, P, C.POINTER(OrcMaterials), C.c_float, P, P, P, C.c_int, P]
        L.orc_shadow_raygen.argtypes = [sp, P, P, I64, P, C.c_float, I32, C.c_int, P]
        L.orc_bounce_raygen.argtypes = [sp, P, P, P, P, I64, C.c_uint32, I32, C.c_float, C.c_float, I32,
                                        C.c_int, P]
        L.orc_collide.argtypes = [sp, P, I64, P, C.c_int, C.c_int]
        pp = C.POINTER(OrcProbeParams)
        L.orc_probe_raygen.argtypes = [pp, C.c_int, P]
        L.orc_probe_direction.argtypes = [C.c_uint32, P, I64, P]
        L.orc_probe_shade.argtypes = [sp, pp, P, P, P, C.POINTER(OrcMaterials), P, P, P, P, P, C.c_int, C.c_int]
        L.orc_small_ufloat.argtypes = [C.c_float, C.c_int]
        L.orc_small_ufloat.restype = C.c_float
        L.orc_bounce_accumulate.argtypes = [P, P, P, I64, I32, P, P, P, C.c_int, P]
        L.orc_pcg_hash.argtypes = [C.c_uint32]
        L.orc_pcg_hash.restype = C.c_uint32
        L.orc_sincos_turns.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_cos_hemisphere.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        L.orc_brute_closest.argtypes = [sp, P, I64, P, P, C.c_int, C.c_int]
        L.orc_build_bvh.restype = C.c_void_p
        L.orc_build_bvh.argtypes = [P, I64, P, I64, P, I32, I32, I32, I32, C.c_uint32]
        L.orc_bvh_info.argtypes = [P] + [C.POINTER(C.c_int64)] * 3
        L.orc_bvh_copy.argtypes = [P, P, P]
        L.orc_bvh_free.argtypes = [P]
        _orc = L
    return _orc


def _p(a):
    return None if a is None else a.ctypes.data


def build_bvh(vertices, indices, mesh_ids=None, tri_offset=0, stackless=False, leaf_size=2,
              swap_children=False, swap_seed=0):
    """The restatement of the reference SAH constructor (orc_build.cpp): (nodes float32 (n, 16) or
    (n, 8), triangles int32 (n_tris, 4), {"leaf_count", "split_fails"})."""
    v = np.ascontiguousarray(vertices)
    idx = np.ascontiguousarray(indices, dtype=np.uint32).ravel()
    mid = None if mesh_ids is None else np.ascontiguousarray(mesh_ids, dtype=np.int32)
    L = orc()
    h = L.orc_build_bvh(_p(v), v.shape[0], _p(idx), idx.size, _p(mid), tri_offset, 1 if stackless else 0,
                        leaf_size, 1 if swap_children else 0, swap_seed & 0xFFFFFFFF)
    if not h:
        raise ValueError("oracle BVH build rejected its input")
    try:
        vals = [C.c_int64() for _ in range(3)]
        L.orc_bvh_info(h, *[C.byref(x) for x in vals])
        n_nodes, leaves, fails = (x.value for x in vals)
        nodes = np.empty((n_nodes, 8 if stackless else 16), dtype=np.float32)
        tris = np.empty((idx.size // 3, 4), dtype=np.int32)
        L.orc_bvh_copy(h, _p(nodes), _p(tris))
    finally:
        L.orc_bvh_free(h)
    return nodes, tris, {"leaf_count": leaves, "split_fails": fails}


class OracleScene:
    """Keeps the numpy buffers alive for the C struct that points into them."""

    def __init__(self, layout: int, vertices, tris, nodes, entities):
        self.vertices = np.ascontiguousarray(vertices)
        self.tris = np.ascontiguousarray(tris, dtype=np.int32)
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float32)
        self.entities = np.ascontiguousarray(entities)
        self.layout = layout  # ORC_STACK / ORC_STACKLESS
        self.s = OrcScene(_p(self.nodes), self.nodes.shape[0], _p(self.tris), _p(self.vertices),
                          _p(self.entities), self.entities.shape[0], layout)

    def closest(self, rays, tie=ORC_TIE_LOWER_INDEX, flags=0, nthreads=None, tri_tests=False):
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.empty(rays.shape[0], dtype=HIT_DTYPE)
        tt = np.empty(rays.shape[0], dtype=np.int32) if tri_tests else None
        orc().orc_closest(C.byref(self.s), _p(rays), rays.shape[0], _p(hits), tie, flags,
                          nthreads or os.cpu_count() or 1, _p(tt))
        return (hits, tt) if tri_tests else hits

    def anyhit(self, rays, nthreads=None, counters=False):
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        occ = np.empty(rays.shape[0], dtype=np.uint8)
        it = np.empty(rays.shape[0], dtype=np.int32) if counters else None
        tt = np.empty(rays.shape[0], dtype=np.int32) if counters else None
        orc().orc_anyhit(C.byref(self.s), _p(rays), rays.shape[0], _p(occ),
                         nthreads or os.cpu_count() or 1, _p(it), _p(tt))
        return (occ, it, tt) if counters else occ

    def brute_closest(self, rays, flags=0, nthreads=None):
        """Every triangle of every entity tested (no box tests): (hits, occluded), the hit being the
        lexicographic minimum of (t, triangle, entity).  Decides between two walks that disagree."""
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.empty(rays.shape[0], dtype=HIT_DTYPE)
        occ = np.empty(rays.shape[0], dtype=np.uint8)
        orc().orc_brute_closest(C.byref(self.s), _p(rays), rays.shape[0], _p(hits), _p(occ), flags,
                                nthreads or os.cpu_count() or 1)
        return hits, occ

    def gi_raygen(self, primary, hits, spp, seed, origin_offset, ray_tmax=1000000.0,
                  normal_mode=0, nthreads=None):
        primary = np.ascontiguousarray(primary, dtype=RAY_DTYPE)
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        out = np.empty(primary.shape[0] * spp, dtype=RAY_DTYPE)
        orc().orc_gi_raygen(C.byref(self.s), _p(primary), _p(hits), primary.shape[0], spp,
                            seed & 0xFFFFFFFF, origin_offset, ray_tmax, normal_mode,
                            nthreads or os.cpu_count() or 1, _p(out))
        return out

    def collide(self, boxes, flags=0, nthreads=None):
        """Collide.comp for n query boxes ((n, 8) float32: min xyzw, max xyzw): (n, 4) int32
        {collided, entity, mesh, tri}."""
        boxes = np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 8)
        out = np.empty((boxes.shape[0], 4), dtype=np.int32)
        orc().orc_collide(C.byref(self.s), _p(boxes), boxes.shape[0], _p(out), flags,
                          nthreads or os.cpu_count() or 1)
        return out

    def shadow_raygen(self, rays, hits, sun_dir, origin_offset, normal_mode=0, nthreads=None):
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        out = np.empty(rays.shape[0], dtype=RAY_DTYPE)
        sd = np.asarray(sun_dir, dtype=np.float32)
        orc().orc_shadow_raygen(C.byref(self.s), _p(rays), _p(hits), rays.shape[0], _p(sd),
                                origin_offset, normal_mode, nthreads or os.cpu_count() or 1,
                                _p(out))
        return out

    def bounce_raygen(self, rays, hits, alive, sample_id, seed, bounce, offset=0.02,
                      ray_tmax=1000000.0, normal_mode=0, nthreads=None):
        """Rays of one RT second bounce from the hits of `rays` (DiffuseTrace.glsl:502-536)."""
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        alive = np.ascontiguousarray(alive, dtype=np.uint8)
        sid = np.ascontiguousarray(sample_id, dtype=np.uint32)
        out = np.empty(rays.shape[0], dtype=RAY_DTYPE)
        orc().orc_bounce_raygen(C.byref(self.s), _p(rays), _p(hits), _p(alive), _p(sid), rays.shape[0],
                                seed & 0xFFFFFFFF, bounce, offset, ray_tmax, normal_mode,
                                nthreads or os.cpu_count() or 1, _p(out))
        return out

    def shade(self, rays, hits, shadow_lit, albedo, sun_dir, sun_color, sky_color,
              normal_mode=0, nthreads=None, textures=None, mesh_texture=None):
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        mat, keep = materials(albedo, textures, mesh_texture)
        lit = None if shadow_lit is None else np.ascontiguousarray(shadow_lit, dtype=np.uint8)
        out = np.empty((rays.shape[0], 4), dtype=np.float32)
        f3 = lambda x: np.asarray(x, dtype=np.float32)  # noqa: E731
        sd, sc, sk = f3(sun_dir), f3(sun_color), f3(sky_color)
        orc().orc_shade(C.byref(self.s), _p(rays), _p(hits), rays.shape[0], _p(lit), C.byref(mat),
                        _p(sd), _p(sc), _p(sk), normal_mode, nthreads or os.cpu_count() or 1, _p(out))
        return out

    def spec_raygen(self, primary, hits, seed, roughness, ray_tmax=1000000.0, normal_mode=0, nthreads=None):
        """Reflection rays of the specular pass (SpecularTrace.glsl:505-513)."""
        primary = np.ascontiguousarray(primary, dtype=RAY_DTYPE)
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        out = np.empty(primary.shape[0], dtype=RAY_DTYPE)
        orc().orc_spec_raygen(C.byref(self.s), _p(primary), _p(hits), primary.shape[0], seed & 0xFFFFFFFF,
                              roughness, ray_tmax, normal_mode, nthreads or os.cpu_count() or 1, _p(out))
        return out

    def spec_shade(self, rays, hits, lit, albedo, roughness, sun_color, sky_color, ambient,
                   textures=None, mesh_texture=None, nthreads=None):
        """(radiance, t / 48) of the specular pass (SpecularTrace.glsl:420-437, 588-596)."""
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        mat, keep = materials(albedo, textures, mesh_texture)
        lit = None if lit is None else np.ascontiguousarray(lit, dtype=np.uint8)
        f3 = lambda x: np.asarray(x, dtype=np.float32)  # noqa: E731
        sc_, sk, am = f3(sun_color), f3(sky_color), f3(ambient)
        out = np.empty((rays.shape[0], 4), dtype=np.float32)
        orc().orc_spec_shade(C.byref(self.s), _p(rays), _p(hits), rays.shape[0], _p(lit), C.byref(mat), roughness,
                             _p(sc_), _p(sk), _p(am), nthreads or os.cpu_count() or 1, _p(out))
        return out

    def probe_shade(self, p, rays, hits, lit, albedo, prev_sh, prev_raw, probe_map, textures=None,
                    mesh_texture=None, nthreads=None, raw_r11=False):
        """Shading, bounce, SH encoding, temporal blend and packing of the probe rays
        (UpdateRadianceProbes.glsl:438-519).  Returns (out_sh (n, 8) uint32, out_raw (n, 4),
        the updated probe map (n, 128)).  raw_r11: the raw radiance rounded to what the reference's
        r11f_g11f_b10f images hold."""
        q = probe_params(p)
        n = probe_count(q)
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        assert rays.shape[0] == n and hits.shape[0] == n
        mat, keep = materials(albedo, textures, mesh_texture)
        lit = None if lit is None else np.ascontiguousarray(lit, dtype=np.uint8)
        psh = np.ascontiguousarray(prev_sh, dtype=np.uint32).reshape(n, 8)
        praw = np.ascontiguousarray(prev_raw, dtype=np.float32).reshape(n, 4)
        pmap = np.array(probe_map, dtype=np.float32, copy=True).reshape(n, 128)
        osh = np.empty((n, 8), dtype=np.uint32)
        oraw = np.empty((n, 4), dtype=np.float32)
        orc().orc_probe_shade(C.byref(self.s), C.byref(q), _p(rays), _p(hits), _p(lit), C.byref(mat), _p(psh),
                              _p(praw), _p(pmap), _p(osh), _p(oraw), 1 if raw_r11 else 0,
                              nthreads or os.cpu_count() or 1)
        return osh, oraw, pmap

    def probe_update(self, p, albedo, prev_sh, prev_raw, probe_map, flags=0, textures=None, mesh_texture=None):
        """The whole probe-update frame as the engine composes it: probe rays, closest hits,
        shadow rays toward the sun (any hit) when p.shadow_rays, then probe_shade.  Returns
        (out_sh, out_raw, probe map, rays, hits)."""
        rays = probe_raygen(p)
        hits = self.closest(rays, flags=flags)
        lit = None
        if p.shadow_rays:
            sr = self.shadow_raygen(rays, hits, np.array(p.sun_dir, dtype=np.float32), p.shadow_offset,
                                    p.normal_mode)
            lit = 1 - self.anyhit(sr)
        osh, oraw, pmap = self.probe_shade(p, rays, hits, lit, albedo, prev_sh, prev_raw, probe_map,
                                           textures, mesh_texture, raw_r11=bool(flags & ORC_FLAG_REF_COMPAT))
        return osh, oraw, pmap, rays, hits

    def hit_normal(self, hits, normal_mode=0):
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        out = np.empty((hits.shape[0], 3), dtype=np.float32)
        orc().orc_hit_normal(C.byref(self.s), _p(hits), hits.shape[0], normal_mode, _p(out))
        return out

    def hit_uv(self, hits):
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        out = np.empty((hits.shape[0], 2), dtype=np.float32)
        orc().orc_hit_uv(C.byref(self.s), _p(hits), hits.shape[0], _p(out))
        return out

    def hit_albedo(self, hits, albedo, textures=None, mesh_texture=None, nthreads=None):
        """GetData's albedo per hit ((n, 3) float32): texture at the hit's UV or ModelColor."""
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        mat, keep = materials(albedo, textures, mesh_texture)
        out = np.empty((hits.shape[0], 3), dtype=np.float32)
        orc().orc_hit_albedo(C.byref(self.s), _p(hits), hits.shape[0], C.byref(mat),
                             nthreads or os.cpu_count() or 1, _p(out))
        return out

    def getdata(self, hits, albedo, textures=None, mesh_texture=None):
        """GetData (TraverseBVHStack.glsl:422-455) per hit record: (n, 8) float32 = Normal xyz,
        Alpha, Albedo rgb, Emissivity; a miss (t < 0 or mesh < 0) gives Normal -1, Albedo 0,
        Emissivity 0 and Alpha 0 (the shader returns before writing Alpha)."""
        hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
        out = np.zeros((hits.shape[0], 8), dtype=np.float32)
        out[:, 0:3] = -1.0
        hit = (hits["t"] >= 0) & (hits["mesh"] >= 0)
        h = np.ascontiguousarray(hits[hit])
        if len(h):
            out[hit, 0:3] = self.hit_normal(h, 0)
            out[hit, 4:7] = self.hit_albedo(h, albedo, textures, mesh_texture)
            data = self.entities["data"][h["entity"]]
            out[hit, 7] = data[:, 0].view(np.float32)
            out[hit, 3] = data[:, 1].view(np.float32)
        return out


def ray_triangle(ro, rd, v0, v1, v2):
    f = lambda x: np.ascontiguousarray(x, dtype=np.float32)  # noqa: E731
    a = [f(x) for x in (ro, rd, v0, v1, v2)]
    out = np.zeros(3, dtype=np.float32)
    orc().orc_ray_triangle(*[_p(x) for x in a], _p(out))
    return out


def ray_bounds_stack(ro, invdir, bmin, bmax, maxt):
    f = lambda x: np.ascontiguousarray(x, dtype=np.float32)  # noqa: E731
    a = [f(x) for x in (ro, invdir, bmin, bmax)]
    return orc().orc_ray_bounds_stack(*[_p(x) for x in a], maxt)


def ray_bounds_stackless(bmin, bmax, ro, invdir, t_min, t_max):
    f = lambda x: np.ascontiguousarray(x, dtype=np.float32)  # noqa: E731
    a = [f(x) for x in (bmin, bmax, ro, invdir)]
    return orc().orc_ray_bounds_stackless(*[_p(x) for x in a], t_min, t_max)


def barycentrics(p, a, b, c):
    f = lambda x: np.ascontiguousarray(x, dtype=np.float32)  # noqa: E731
    x = [f(v) for v in (p, a, b, c)]
    out = np.zeros(3, dtype=np.float32)
    orc().orc_barycentrics(*[_p(v) for v in x], _p(out))
    return out


def small_ufloat(x: float, mbits: int) -> float:
    """The value a GL_R11F_G11F_B10F channel with mbits mantissa bits holds for x (restatement)."""
    return orc().orc_small_ufloat(x, mbits)


def pcg_hash(x: int) -> int:
    return orc().orc_pcg_hash(x & 0xFFFFFFFF)


def bounce_accumulate(fr, thr0, inputs, sun_dir, sun_color, sky, ref_miss):
    """FinalRadiance + Bounced of the RT second-bounce loop (DiffuseTrace.glsl:499-535) per GI slot:
    fr, thr0 (n, 3); inputs (n, bounces, 12) {t, albedo rgb, emissive, normal xyz, direction xyz,
    sun visibility}."""
    fr = np.ascontiguousarray(fr, dtype=np.float32)
    th = np.ascontiguousarray(thr0, dtype=np.float32)
    x = np.ascontiguousarray(inputs, dtype=np.float32)
    f3 = lambda v: np.ascontiguousarray(v, dtype=np.float32)  # noqa: E731
    sd, sc, sk = f3(sun_dir), f3(sun_color), f3(sky)
    out = np.empty((fr.shape[0], 3), dtype=np.float32)
    orc().orc_bounce_accumulate(_p(fr), _p(th), _p(x), fr.shape[0], x.shape[1], _p(sd), _p(sc), _p(sk),
                                int(bool(ref_miss)), _p(out))
    return out


def pcg_hash_np(x):
    """pcg_hash over a uint32 array (numpy arithmetic wraps like the C one)."""
    x = np.asarray(x, dtype=np.uint32)
    state = x * np.uint32(747796405) + np.uint32(2891336453)
    word = ((state >> ((state >> np.uint32(28)) + np.uint32(4))) ^ state) * np.uint32(277803737)
    return (word >> np.uint32(22)) ^ word


def sample_u01(seed, ids, dim):
    """The GI / probe samplers' uniform value in [0, 1) for (seed, ray or probe id, dimension)."""
    with np.errstate(over="ignore"):
        h = pcg_hash_np(pcg_hash_np(pcg_hash_np(np.uint32(seed & 0xFFFFFFFF)) + np.asarray(ids, dtype=np.uint32))
                        + np.uint32(dim))
    return (h >> np.uint32(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def sincos_turns(x: float):
    s, c = C.c_float(), C.c_float()
    orc().orc_sincos_turns(x, C.byref(s), C.byref(c))
    return s.value, c.value


# ---- reference BVH constructor (compiled from the mounted reference tree) -----------------

_ref = {}


def ref_glsl_available() -> bool:
    return REF_GLSL_SO.exists()


def _ref_glsl():
    L = C.CDLL(str(REF_GLSL_SO))
    P = C.c_void_p
    L.ref_glsl_closest.restype = None
    L.ref_glsl_closest.argtypes = [C.c_int, C.c_int, P, C.c_int64, P, C.c_int64, P, C.c_int64, P, C.c_int32, P,
                                   C.c_int64, P]
    L.ref_glsl_occluded.restype = None
    L.ref_glsl_occluded.argtypes = [C.c_int, P, C.c_int64, P, C.c_int64, P, C.c_int64, P, C.c_int32, P, C.c_int64, P]
    return L


def ref_glsl_closest(layout, vertices, tris, nodes, entities, rays, ignore_transparent=False):
    """The reference's IntersectScene[IgnoreTransparent] (TraverseBVHStack[less].glsl compiled as
    C++ by oracle/Makefile) per ray: HIT_DTYPE records (t, u, v, w from TUVW; tri, mesh, entity,
    iters from its outputs, -1 where it leaves them unwritten)."""
    v, t = np.ascontiguousarray(vertices), np.ascontiguousarray(tris, dtype=np.int32)
    n, e = np.ascontiguousarray(nodes, dtype=np.float32), np.ascontiguousarray(entities)
    r = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
    out = np.empty(r.shape[0], dtype=HIT_DTYPE)
    _ref_glsl().ref_glsl_closest(int(layout == ORC_STACKLESS), int(ignore_transparent), _p(n), n.shape[0], _p(t),
                                 t.shape[0], _p(v), v.shape[0], _p(e), e.shape[0], _p(r), r.shape[0], _p(out))
    return out


def ref_glsl_occluded(layout, vertices, tris, nodes, entities, rays):
    """The reference's float IntersectRay(o, d) > 0 per ray (compiled from its shader source)."""
    v, t = np.ascontiguousarray(vertices), np.ascontiguousarray(tris, dtype=np.int32)
    n, e = np.ascontiguousarray(nodes, dtype=np.float32), np.ascontiguousarray(entities)
    r = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
    out = np.empty(r.shape[0], dtype=np.uint8)
    _ref_glsl().ref_glsl_occluded(int(layout == ORC_STACKLESS), _p(n), n.shape[0], _p(t), t.shape[0], _p(v),
                                  v.shape[0], _p(e), e.shape[0], _p(r), r.shape[0], _p(out))
    return out


def ref_glsl_collide(layout, vertices, tris, nodes, entities, boxes):
    """The reference's CollideScene (CollideBVHStack[less].glsl compiled as C++): (n, 4) int32
    {collided, entity, mesh, tri}, -1 where the shader leaves an output unwritten."""
    L = C.CDLL(str(REF_GLSL_SO))
    P = C.c_void_p
    L.ref_glsl_collide.restype = None
    L.ref_glsl_collide.argtypes = [C.c_int, P, C.c_int64, P, C.c_int64, P, C.c_int64, P, C.c_int32, P, C.c_int64, P]
    v, t = np.ascontiguousarray(vertices), np.ascontiguousarray(tris, dtype=np.int32)
    n, e = np.ascontiguousarray(nodes, dtype=np.float32), np.ascontiguousarray(entities)
    b = np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 8)
    out = np.empty((b.shape[0], 4), dtype=np.int32)
    L.ref_glsl_collide(int(layout == ORC_STACKLESS), _p(n), n.shape[0], _p(t), t.shape[0], _p(v), v.shape[0], _p(e),
                       e.shape[0], _p(b), b.shape[0], _p(out))
    return out


def ref_glsl_getdata(vertices, tris, entities, model_color, albedo_ref, hits):
    """The reference's GetData (TraverseBVHStack.glsl:422-455 compiled as C++) per hit: (n, 8)
    floats Normal, Albedo, Emissivity, Alpha; its texture() reports (u, v, texture index)."""
    L = C.CDLL(str(REF_GLSL_SO))
    P = C.c_void_p
    L.ref_glsl_getdata.restype = None
    L.ref_glsl_getdata.argtypes = [P, C.c_int64, P, C.c_int64, P, C.c_int32, P, C.c_int32, P, C.c_int64, P]
    v, t, e = np.ascontiguousarray(vertices), np.ascontiguousarray(tris, dtype=np.int32), np.ascontiguousarray(entities)
    mc = np.asarray(model_color, dtype=np.float32).reshape(-1, 3)
    refs = np.zeros((mc.shape[0], 8), dtype=np.float32)     # vec4 ModelColor, int Albedo, Normal, Pad[2]
    refs[:, :3] = mc
    refs.view(np.int32)[:, 4] = np.asarray(albedo_ref, dtype=np.int32)
    refs.view(np.int32)[:, 5] = -1
    h = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    out = np.empty((h.shape[0], 8), dtype=np.float32)
    L.ref_glsl_getdata(_p(t), t.shape[0], _p(v), v.shape[0], _p(e), e.shape[0], _p(refs), refs.shape[0], _p(h),
                       h.shape[0], _p(out))
    return out


def spec_direction(incident, normals, roughness, seed, rid):
    """The restatement's StochasticReflectionDirection for (n, 3) incident directions and normals."""
    i3 = np.ascontiguousarray(incident, dtype=np.float32).reshape(-1, 3)
    n3 = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    rr = np.ascontiguousarray(rid, dtype=np.uint32)
    out = np.empty_like(i3)
    orc().orc_spec_direction(_p(i3), _p(n3), i3.shape[0], roughness, seed & 0xFFFFFFFF, _p(rr), _p(out))
    return out


def ref_glsl_spec_direction(incident, normals, roughness, seed, rid):
    """The reference's StochasticReflectionDirection(I, N, 0.9 R) and SampleGGXVNDF compiled as C++,
    hash2() drawing the same counter-based samples."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_spec_direction.restype = None
    L.ref_glsl_spec_direction.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_uint32, C.c_void_p,
                                          C.c_void_p]
    i3 = np.ascontiguousarray(incident, dtype=np.float32).reshape(-1, 3)
    n3 = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    rr = np.ascontiguousarray(rid, dtype=np.uint32)
    out = np.empty_like(i3)
    L.ref_glsl_spec_direction(_p(i3), _p(n3), i3.shape[0], roughness, seed & 0xFFFFFFFF, _p(rr), _p(out))
    return out


def ref_glsl_shade(specular, rays, hits, albedo, normals, lit, sun_dir, sun_color, sky, probe=(0.0, 0.0, 0.0),
                   roughness=0.0):
    """The reference's shading statements compiled as C++: the diffuse pass's hit shading
    (DiffuseTrace.glsl:486-494, GetDirect :368-372) giving (FinalRadiance, AO), or the specular
    pass's (SpecularTrace.glsl:554-563, 588-596, SampleLighting :420-425, Sky :435-437) giving the
    stored (radiance, t / 48).  albedo: (n, 4) rgb + emissive as GetData returns them; normals:
    (n, 3) GetData's normal; lit: what GetDirectShadow returns (0 / 1); sky: what the sky
    textures return; probe: what SampleProbes returns."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_shade.restype = None
    L.ref_glsl_shade.argtypes = [C.c_int, C.c_void_p, C.c_int64] + [C.c_void_p] * 4 + [C.c_float, C.c_void_p]
    rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
    hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    n = rays.shape[0]
    x = np.empty((n, 18), dtype=np.float32)
    x[:, 0:3], x[:, 3:6] = rays["o"], rays["d"]
    x[:, 6], x[:, 7], x[:, 8], x[:, 9] = hits["t"], hits["u"], hits["v"], hits["w"]
    x[:, 10:14] = albedo
    x[:, 14:17] = normals
    x[:, 17] = np.asarray(lit, dtype=np.float32)
    f3 = lambda v: np.ascontiguousarray(v, dtype=np.float32)  # noqa: E731
    sd, sc, sk, pr = f3(sun_dir), f3(sun_color), f3(sky), f3(probe)
    out = np.empty((n, 4), dtype=np.float32)
    L.ref_glsl_shade(int(specular), _p(x), n, _p(sd), _p(sc), _p(sk), _p(pr), roughness, _p(out))
    return out


def ref_glsl_sun_colors():
    """SUN_COLOR_DIFF and SUN_COLOR_SPEC (ColorConstants.h) as the reference's shaders evaluate them."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_sun_colors.restype = None
    out = np.empty(6, dtype=np.float32)
    L.ref_glsl_sun_colors(_p(out))
    return out[:3].copy(), out[3:].copy()


def ref_glsl_probe(p, rays, hits, albedo, normals, lit, prev_sh, prev_raw, probe_map):
    """UpdateRadianceProbes.glsl main compiled as C++ for every probe of p's grid, fed the ray
    directions, hits (TUVW), GetData's albedo (n, 4: rgb, emissive) and normal, and the sun
    visibility.  Returns (out_sh (n, 8), out_raw (n, 4), the updated map (n, 128))."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_probe.restype = None
    L.ref_glsl_probe.argtypes = [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 9
    n = probe_count(p)
    rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
    hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    x = np.zeros((n, 16), dtype=np.float32)
    x[:, 0:3] = rays["d"]
    x[:, 3], x[:, 4], x[:, 5], x[:, 6] = hits["t"], hits["u"], hits["v"], hits["w"]
    x[:, 7:11] = albedo
    x[:, 11:14] = normals
    x[:, 14] = np.asarray(lit, dtype=np.float32)
    arr = lambda v, t=np.float32: np.ascontiguousarray(np.array(v[:], dtype=t))  # noqa: E731
    grid = arr(p.grid, np.int32)
    org, prev, size = arr(p.origin), arr(p.prev_origin), arr(p.size)
    sd, sc, sk = arr(p.sun_dir), arr(p.sun_color), arr(p.sky_color)
    psh = np.ascontiguousarray(prev_sh, dtype=np.uint32).reshape(n, 8)
    praw = np.ascontiguousarray(prev_raw, dtype=np.float32).reshape(n, 4)
    pmap = np.array(probe_map, dtype=np.float32, copy=True).reshape(n, 128)
    osh = np.zeros((n, 8), dtype=np.uint32)
    oraw = np.zeros((n, 4), dtype=np.float32)
    L.ref_glsl_probe(_p(grid), _p(org), _p(prev), _p(size), int(p.temporal), _p(sd), _p(sc), _p(sk), _p(x), _p(psh),
                     _p(praw), _p(pmap), _p(osh), _p(oraw))
    return osh, oraw, pmap


def ref_glsl_bounce(slot, per_bounce, sun_dir, sun_color, sky):
    """The RT second-bounce loop (DiffuseTrace.glsl:499-535) compiled as C++ per GI slot: slot
    (n, 20) {GI ray origin, direction, TUVW, Albedo, faced normal, FinalRadiance}; per_bounce
    (n, bounces, 15) {direction, TUVW, Albedo, normal, sun visibility}.  Returns (FinalRadiance
    (n, 3), bounce ray origins (n, bounces, 3))."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_bounce.restype = None
    L.ref_glsl_bounce.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_int64] + [C.c_void_p] * 5
    sl = np.ascontiguousarray(slot, dtype=np.float32)
    pb = np.ascontiguousarray(per_bounce, dtype=np.float32)
    f3 = lambda v: np.ascontiguousarray(v, dtype=np.float32)  # noqa: E731
    sd, sc, sk = f3(sun_dir), f3(sun_color), f3(sky)
    fr = np.empty((sl.shape[0], 3), dtype=np.float32)
    org = np.empty((sl.shape[0], pb.shape[1], 3), dtype=np.float32)
    L.ref_glsl_bounce(pb.shape[1], _p(sl), _p(pb), sl.shape[0], _p(sd), _p(sc), _p(sk), _p(fr), _p(org))
    return fr, org


def ref_glsl_lambert_direction(h):
    """normalize(LambertBRDF(h)) (UpdateRadianceProbes.glsl:351-372) for (n, 3) hash values."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_lambert_direction.restype = None
    L.ref_glsl_lambert_direction.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
    hh = np.ascontiguousarray(h, dtype=np.float32).reshape(-1, 3)
    out = np.empty_like(hh)
    L.ref_glsl_lambert_direction(_p(hh), hh.shape[0], _p(out))
    return out


def ref_glsl_probe_sun_color():
    """SUN_COLOR_PROBES (ColorConstants.h) as the probe shader evaluates it."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_probe_sun_color.restype = None
    out = np.empty(3, dtype=np.float32)
    L.ref_glsl_probe_sun_color(_p(out))
    return out


def cos_hemisphere(normals, r):
    """The restatement's CosWeightedHemisphere (turn-based sine / cosine) for (n, 3) normals and
    (n, 2) samples."""
    nn = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    rr = np.ascontiguousarray(r, dtype=np.float32).reshape(-1, 2)
    out = np.empty_like(nn)
    orc().orc_cos_hemisphere(_p(nn), _p(rr), nn.shape[0], _p(out))
    return out


def ref_glsl_cos_hemisphere(normals, r):
    """The reference's CosWeightedHemisphere (Sampling.glsl compiled as C++, C-library cos / sin)."""
    L = C.CDLL(str(REF_GLSL_SO))
    L.ref_glsl_cos_hemisphere.restype = None
    L.ref_glsl_cos_hemisphere.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    nn = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    rr = np.ascontiguousarray(r, dtype=np.float32).reshape(-1, 2)
    out = np.empty_like(nn)
    L.ref_glsl_cos_hemisphere(_p(nn), _p(rr), nn.shape[0], _p(out))
    return out


def ref_physics_available() -> bool:
    return REF_PHYSICS_SO.exists()


def ref_collide_boxes(vertices, tris, nodes, entities, boxes) -> np.ndarray:
    """The reference's Physics::CollideBox (Physics.cpp:203-228, compiled from its source by
    oracle/Makefile) for each box over a stackless scene: uint8 collided flags."""
    L = C.CDLL(str(REF_PHYSICS_SO))
    L.ref_collide_boxes.restype = None
    L.ref_collide_boxes.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                    C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]
    v = np.ascontiguousarray(vertices)
    t = np.ascontiguousarray(tris, dtype=np.int32)
    n = np.ascontiguousarray(nodes, dtype=np.float32)
    e = np.ascontiguousarray(entities)
    b = np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 8)
    out = np.zeros(b.shape[0], dtype=np.uint8)
    L.ref_collide_boxes(_p(n), n.shape[0], _p(t), t.shape[0], _p(v), v.shape[0], _p(e), e.shape[0], _p(b),
                        b.shape[0], _p(out))
    return out


def ref_available(leaf4: bool = False) -> bool:
    so = REF_LEAF4_SO if leaf4 else REF_SO
    root = reference_root()
    if not so.exists() and root is not None and (root / "Source").exists():
        try:
            build(reference=True)
        except Exception:
            return False
    return so.exists()


def _refl(leaf4: bool) -> C.CDLL:
    key = "leaf4" if leaf4 else "leaf2"
    if key not in _ref:
        L = C.CDLL(str(REF_LEAF4_SO if leaf4 else REF_SO))
        L.refbvh_build.restype = C.c_void_p
        L.refbvh_build.argtypes = [C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                   C.c_void_p, C.c_int32, C.c_int, C.c_uint32]
        L.refbvh_info.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 6
        L.refbvh_copy.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.refbvh_free.argtypes = [C.c_void_p]
        _ref[key] = L
    return _ref[key]


def ref_build_bvh(vertices, indices, mesh_ids=None, tri_offset=0, stackless=False,
                  swap_mode=0, swap_seed=0, leaf4=False):
    """Runs the reference constructor; returns (nodes float32 (N,16|8), tris int32 (T,4), info)."""
    L = _refl(leaf4)
    v = np.ascontiguousarray(vertices)
    idx = np.ascontiguousarray(indices, dtype=np.uint32).ravel()
    mid = None if mesh_ids is None else np.ascontiguousarray(mesh_ids, dtype=np.int32)
    h = L.refbvh_build(1 if stackless else 0, _p(v), v.shape[0], _p(idx), idx.size, _p(mid),
                       tri_offset, swap_mode, swap_seed)
    if not h:
        raise ValueError("reference builder rejected the input")
    try:
        vals = [C.c_int64() for _ in range(6)]
        L.refbvh_info(h, *[C.byref(x) for x in vals])
        n_nodes, n_tris, last, leaves, fails, depth = (x.value for x in vals)
        nodes = np.zeros((n_nodes, 8 if stackless else 16), dtype=np.float32)
        tris = np.zeros((n_tris, 4), dtype=np.int32)
        L.refbvh_copy(h, _p(nodes), _p(tris))
        return nodes, tris, dict(last_node_index=last, leaf_count=leaves, split_fails=fails,
                                 max_depth=depth)
    finally:
        L.refbvh_free(h)
