"""Seeded procedural scenes and ray sets for the ray-query engine.

Every generator uses only IEEE-exact numpy operations (+, -, *, /, sqrt, floor) so the same seed
gives byte-identical scenes on x86 and on the aarch64 GPU hosts; the few transcendental functions
needed (sin, exp) are evaluated by the fixed polynomials below rather than by libm/SVML, whose
last-ulp results differ between platforms.

Scenes follow the reference's buffer conventions:
  * vertices are 32-byte records {float4 position (w = 1), uint32 packed[4]}, with the vertex
    normal packed as half2x16 the way the reference's model loader does (ModelFileLoader.cpp and
    UnpackNormal, Include/TraverseBVHStack.glsl:417-420): packed[0] = half2(n.x, n.y),
    packed[1] = half2(n.z, 0), packed[2] = 0, packed[3] = texcoords (0 here);
  * indices are uint32, three per triangle; mesh ids are one int per triangle.

Parameters for the named workloads (heightfield 256x256, icosphere sets, camera rays) are the ones
the benchmark and the tests use; the generator parameters are returned so they can be reported.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

VERTEX_DTYPE = np.dtype([("pos", "<f4", (4,)), ("packed", "<u4", (4,))])
RAY_DTYPE = np.dtype([("o", "<f4", (3,)), ("tmin", "<f4"), ("d", "<f4", (3,)), ("tmax", "<f4")])


# ---------------------------------------------------------------------------------------------
# Deterministic elementary functions (float64, IEEE-exact operations only)

_TWO_PI = 6.283185307179586


def sin_turns(s: np.ndarray) -> np.ndarray:
    """sin(2*pi*s) by reduction to [-1/4, 1/4] turn and a degree-21 Taylor polynomial."""
    s = np.asarray(s, dtype=np.float64)
    f = s - np.floor(s)                      # [0, 1)
    f = np.where(f > 0.5, f - 1.0, f)        # (-0.5, 0.5]
    f = np.where(f > 0.25, 0.5 - f, f)       # reflect: sin(pi - x) = sin(x)
    f = np.where(f < -0.25, -0.5 - f, f)
    x = f * _TWO_PI                          # |x| <= pi/2
    x2 = x * x
    acc = np.zeros_like(x)
    for n in range(21, 0, -2):               # sum_{k} (-1)^k x^(2k+1)/(2k+1)!
        coef = ((-1.0) ** ((n - 1) // 2)) / math.factorial(n)
        acc = acc * x2 + coef
    # acc currently = sum c_n x^(n-1) over odd n, in powers of x2 -> multiply by x
    return acc * x


def cos_turns(s: np.ndarray) -> np.ndarray:
    return sin_turns(np.asarray(s, dtype=np.float64) + 0.25)


def exp_det(x: np.ndarray) -> np.ndarray:
    """exp(x) = 2^k * exp(r), |r| <= ln2/2, with a 20-term Taylor series."""
    x = np.asarray(x, dtype=np.float64)
    ln2 = 0.6931471805599453
    k = np.floor(x / ln2 + 0.5)
    r = x - k * ln2
    acc = np.ones_like(r)
    for n in range(20, 0, -1):
        acc = 1.0 + acc * r / n
    return np.ldexp(acc, k.astype(np.int64))


# ---------------------------------------------------------------------------------------------
# Counter-based random numbers (pcg_hash, Jarzynski & Olano 2020, JCGT 9(3))

def pcg_hash(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.uint32)
    with np.errstate(over="ignore"):
        state = x * np.uint32(747796405) + np.uint32(2891336453)
        word = ((state >> ((state >> np.uint32(28)) + np.uint32(4))) ^ state) * np.uint32(277803737)
    return (word >> np.uint32(22)) ^ word


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n float64 uniforms in [0,1) for (seed, stream): 53-bit values from two hashes."""
    idx = np.arange(n, dtype=np.uint64)
    base = pcg_hash(np.uint32(seed & 0xFFFFFFFF)) ^ pcg_hash(np.uint32((stream * 0x9E3779B9) & 0xFFFFFFFF))
    with np.errstate(over="ignore"):
        lo = pcg_hash((idx * 2).astype(np.uint32) ^ base)
        hi = pcg_hash((idx * 2 + 1).astype(np.uint32) ^ pcg_hash(base))
    v = (hi.astype(np.uint64) >> np.uint64(5)) * np.uint64(1 << 26) + (lo.astype(np.uint64) >> np.uint64(6))
    return v.astype(np.float64) * (1.0 / 9007199254740992.0)


# ---------------------------------------------------------------------------------------------
# Half-float packing of normals (exact float32 -> binary16 round-to-nearest-even)

def _len3(v: np.ndarray) -> np.ndarray:
    """Row lengths with a fixed summation order ((x*x + y*y) + z*z)."""
    return np.sqrt(v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1] + v[..., 2] * v[..., 2])


def float_to_half_bits(x: np.ndarray) -> np.ndarray:
    return np.asarray(x, dtype=np.float32).astype(np.float16).view(np.uint16).astype(np.uint32)


def pack_normals(n: np.ndarray) -> np.ndarray:
    """(N,3) float normals -> (N,4) uint32 packed words (see module docstring)."""
    h = float_to_half_bits(n)
    out = np.zeros((n.shape[0], 4), dtype=np.uint32)
    out[:, 0] = h[:, 0] | (h[:, 1] << np.uint32(16))
    out[:, 1] = h[:, 2]
    return out


def make_vertices(pos: np.ndarray, normals: np.ndarray) -> np.ndarray:
    v = np.zeros(pos.shape[0], dtype=VERTEX_DTYPE)
    p = np.asarray(pos, dtype=np.float32) + np.float32(0.0)  # +0.0 folds -0.0 into +0.0
    v["pos"][:, :3] = p
    v["pos"][:, 3] = 1.0
    v["packed"] = pack_normals(normals)
    return v


def with_texcoords(vertices: np.ndarray, uv: np.ndarray) -> np.ndarray:
    """A copy of VERTEX_DTYPE records with texture coordinates (n, 2) half-packed into the last
    word (Vertex.PackedData.w: u in the low half, v in the high half, as packHalf2x16)."""
    v = np.array(vertices, copy=True)
    h = float_to_half_bits(np.asarray(uv, dtype=np.float32))
    v["packed"][:, 3] = (h[:, 0] | (h[:, 1] << np.uint32(16))).astype(np.uint32)
    return v


def noise_texture(size: int, seed: int) -> np.ndarray:
    """A (size, size, 4) uint8 RGBA texture: seeded value noise per channel plus a checker."""
    u = uniform(seed, 606, size * size * 3).reshape(size, size, 3)
    yy, xx = np.mgrid[0:size, 0:size]
    checker = ((xx // max(1, size // 8) + yy // max(1, size // 8)) % 2)[..., None]
    img = np.zeros((size, size, 4), np.uint8)
    img[..., :3] = np.clip(40 + 150 * u + 60 * checker, 0, 255).astype(np.uint8)
    img[..., 3] = 255
    return img


# ---------------------------------------------------------------------------------------------
# Meshes

@dataclass
class Mesh:
    vertices: np.ndarray          # VERTEX_DTYPE records
    indices: np.ndarray           # uint32, 3 per triangle
    mesh_ids: np.ndarray          # int32, one per triangle
    params: dict = field(default_factory=dict)

    @property
    def n_tris(self) -> int:
        return self.indices.size // 3

    def positions(self) -> np.ndarray:
        return self.vertices["pos"][:, :3]


def heightfield(n: int = 256, seed: int = 1, extent: float = 1.0, n_waves: int = 4,
                amp=(0.05, 0.2), freq=(1.0, 8.0), mesh_id: int = 0) -> Mesh:
    """n x n quads (2 n^2 triangles) over [-extent, extent]^2 with
    z = sum_k a_k sin(2 pi (fx_k x + fy_k y) + phi_k): a_k uniform in amp, cycles uniform in freq
    with a random direction, phase uniform in [0, 2 pi)."""
    u = uniform(seed, 101, 5 * n_waves).reshape(n_waves, 5)
    a = amp[0] + (amp[1] - amp[0]) * u[:, 0]
    cyc = freq[0] + (freq[1] - freq[0]) * u[:, 1]
    ang = u[:, 2]
    fx = cyc * cos_turns(ang) / (2.0 * extent)
    fy = cyc * sin_turns(ang) / (2.0 * extent)
    ph = u[:, 3]
    g = np.arange(n + 1, dtype=np.float64)
    x = -extent + (2.0 * extent) * g / n
    X, Y = np.meshgrid(x, x, indexing="xy")       # row j = y index, column i = x index
    X = X.ravel()
    Y = Y.ravel()
    Z = np.zeros_like(X)
    dzdx = np.zeros_like(X)
    dzdy = np.zeros_like(X)
    for k in range(n_waves):
        arg = fx[k] * X + fy[k] * Y + ph[k]
        Z = Z + a[k] * sin_turns(arg)
        c = a[k] * _TWO_PI * cos_turns(arg)
        dzdx = dzdx + c * fx[k]
        dzdy = dzdy + c * fy[k]
    pos = np.stack([X, Y, Z], axis=1)
    nrm = np.stack([-dzdx, -dzdy, np.ones_like(Z)], axis=1)
    nrm = nrm / _len3(nrm)[:, None]
    i = np.arange(n, dtype=np.uint32)
    I, J = np.meshgrid(i, i, indexing="xy")
    v00 = (J * (n + 1) + I).ravel()
    v10 = v00 + 1
    v01 = v00 + (n + 1)
    v11 = v01 + 1
    tris = np.stack([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 1).reshape(-1, 3)
    params = dict(kind="heightfield", n=n, seed=seed, extent=extent,
                  amp=a.tolist(), cycles=cyc.tolist(), phase_turns=ph.tolist())
    return Mesh(make_vertices(pos, nrm), tris.astype(np.uint32).ravel(),
                np.full(tris.shape[0], mesh_id, dtype=np.int32), params)


_ICO_CACHE: dict = {}


def unit_icosphere(subdiv: int):
    """Unit icosphere: 20 * 4^subdiv triangles (float64 positions, int64 faces)."""
    if subdiv in _ICO_CACHE:
        return _ICO_CACHE[subdiv]
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
             (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = np.array(verts, dtype=np.float64)
    V = V / _len3(V)[:, None]
    F = np.array(faces, dtype=np.int64)
    for _ in range(subdiv):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], 0)
        key = np.minimum(e[:, 0], e[:, 1]) * (1 << 32) + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq >> 32
        b = uniq & ((1 << 32) - 1)
        mid = (V[a] + V[b]) * 0.5
        mid = mid / _len3(mid)[:, None]
        base = V.shape[0]
        V = np.concatenate([V, mid], 0)
        m = inv.reshape(3, -1) + base
        m01, m12, m20 = m[0], m[1], m[2]
        F = np.concatenate([np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
                            np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)], 0)
    _ICO_CACHE[subdiv] = (V, F)
    return V, F


def _value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Trilinear value noise in [-1, 1] with smoothstep weights on the integer lattice."""
    fl = np.floor(p)
    f = p - fl
    w = f * f * (3.0 - 2.0 * f)
    c = fl.astype(np.int64)
    out = np.zeros(p.shape[0], dtype=np.float64)
    s = np.uint32(seed & 0xFFFFFFFF)
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                h = pcg_hash(((c[:, 0] + dx) & 0xFFFFFFFF).astype(np.uint32) ^ pcg_hash(s))
                h = pcg_hash(h ^ ((c[:, 1] + dy) & 0xFFFFFFFF).astype(np.uint32))
                h = pcg_hash(h ^ ((c[:, 2] + dz) & 0xFFFFFFFF).astype(np.uint32))
                val = (h >> np.uint32(8)).astype(np.float64) * (2.0 / 16777216.0) - 1.0
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out = out + val * (wx * wy * wz)
    return out


def icosphere_set(n_spheres: int = 64, subdiv: int = 5, seed: int = 2,
                  lo=(-4.0, -4.0, 0.0), hi=(4.0, 4.0, 2.0), radius=(0.1, 0.5),
                  disp: float = 0.05, octaves: int = 3, ground: float | None = 6.0) -> Mesh:
    """n displaced icospheres (radii log-uniform, centres uniform in [lo, hi]) plus an optional
    2-triangle ground plane at z = 0 spanning [-ground, ground]^2.  Displacement is 3-octave value
    noise along the normal with amplitude disp * radius.  Mesh id = sphere index; plane = n."""
    V, F = unit_icosphere(subdiv)
    u = uniform(seed, 202, n_spheres * 5).reshape(n_spheres, 5)
    lo = np.array(lo, dtype=np.float64)
    hi = np.array(hi, dtype=np.float64)
    centres = lo + (hi - lo) * u[:, :3]
    radii = radius[0] * exp_det(u[:, 3] * (math.log(radius[1]) - math.log(radius[0])))
    pos_all, nrm_all, idx_all, mid_all = [], [], [], []
    base = 0
    for s in range(n_spheres):
        p = V * 2.0 + u[s, 4] * 64.0
        n = np.zeros(V.shape[0], dtype=np.float64)
        amp, frq, tot = 1.0, 1.0, 0.0
        for _ in range(octaves):
            n = n + amp * _value_noise(p * frq, seed * 7919 + s)
            tot += amp
            amp *= 0.5
            frq *= 2.0
        n = n / tot
        r = radii[s] * (1.0 + disp * n)
        pos = centres[s] + V * r[:, None]
        pos_all.append(pos)
        nrm_all.append(V)
        idx_all.append(F + base)
        mid_all.append(np.full(F.shape[0], s, dtype=np.int32))
        base += V.shape[0]
    if ground is not None:
        g = float(ground)
        pos_all.append(np.array([[-g, -g, 0.0], [g, -g, 0.0], [g, g, 0.0], [-g, g, 0.0]]))
        nrm_all.append(np.tile([[0.0, 0.0, 1.0]], (4, 1)))
        idx_all.append(np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int64) + base)
        mid_all.append(np.full(2, n_spheres, dtype=np.int32))
    pos = np.concatenate(pos_all, 0)
    nrm = np.concatenate(nrm_all, 0)
    idx = np.concatenate(idx_all, 0).astype(np.uint32).ravel()
    params = dict(kind="icospheres", n_spheres=n_spheres, subdiv=subdiv, seed=seed,
                  lo=lo.tolist(), hi=hi.tolist(), radius=list(radius), disp=disp,
                  octaves=octaves, ground=ground)
    return Mesh(make_vertices(pos, nrm), idx, np.concatenate(mid_all), params)


# ---------------------------------------------------------------------------------------------
# Rays

def camera_rays(width: int, height: int, eye, target, up=(0.0, 0.0, 1.0), vfov_deg: float = 60.0,
                tmax: float = 1000000.0) -> np.ndarray:
    """Pinhole camera: one ray through each pixel centre, row-major from the top-left pixel."""
    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - eye
    fwd = fwd / float(_len3(fwd))
    right = np.cross(fwd, np.asarray(up, dtype=np.float64))
    right = right / float(_len3(right))
    upv = np.cross(right, fwd)
    half = vfov_deg / 360.0  # turns of the full field of view / 2
    th = float(sin_turns(np.array(half * 0.5)) / cos_turns(np.array(half * 0.5)))  # tan(vfov/2)
    aspect = width / height
    px = (np.arange(width, dtype=np.float64) + 0.5) / width * 2.0 - 1.0
    py = 1.0 - (np.arange(height, dtype=np.float64) + 0.5) / height * 2.0
    PX, PY = np.meshgrid(px * th * aspect, py * th, indexing="xy")
    d = fwd[None, :] + PX.ravel()[:, None] * right[None, :] + PY.ravel()[:, None] * upv[None, :]
    d = d / _len3(d)[:, None]
    r = np.zeros(width * height, dtype=RAY_DTYPE)
    r["o"] = eye.astype(np.float32)
    r["d"] = d.astype(np.float32) + np.float32(0.0)
    r["tmin"] = 0.0
    r["tmax"] = tmax
    return r


def sphere_rays(n: int, lo, hi, seed: int = 4, tmax: float = 1000000.0) -> np.ndarray:
    """Origins uniform in the box [lo, hi], directions uniform on the unit sphere."""
    u = uniform(seed, 303, n * 5).reshape(n, 5)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    o = lo + (hi - lo) * u[:, :3]
    z = 2.0 * u[:, 3] - 1.0
    rxy = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d = np.stack([rxy * cos_turns(u[:, 4]), rxy * sin_turns(u[:, 4]), z], 1)
    d = d / _len3(d)[:, None]
    r = np.zeros(n, dtype=RAY_DTYPE)
    r["o"] = o.astype(np.float32)
    r["d"] = d.astype(np.float32) + np.float32(0.0)
    r["tmax"] = tmax
    return r


def instance_transforms(n: int, lo, hi, scale_lo: float, scale_hi: float, seed: int = 8,
                        anisotropic: float = 0.1, tilt: float = 0.08) -> np.ndarray:
    """n model matrices ((n, 4, 4) float32, row-major): translation uniform in [lo, hi], a turn
    about z, a tilt about x of up to `tilt` turns, a uniform scale in [scale_lo, scale_hi]; a
    fraction `anisotropic` of them is scaled (1, 0.5, 1.5) on top."""
    u = uniform(seed, 505, n * 8).reshape(n, 8)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    t = lo + (hi - lo) * u[:, :3]
    cz, sz = cos_turns(u[:, 3]), sin_turns(u[:, 3])
    ax = tilt * (2.0 * u[:, 4] - 1.0)
    cx, sx = cos_turns(ax), sin_turns(ax)
    s = scale_lo + (scale_hi - scale_lo) * u[:, 5]
    m = np.zeros((n, 4, 4))
    for i in range(n):
        rz = np.array([[cz[i], -sz[i], 0.0], [sz[i], cz[i], 0.0], [0.0, 0.0, 1.0]])
        rx = np.array([[1.0, 0.0, 0.0], [0.0, cx[i], -sx[i]], [0.0, sx[i], cx[i]]])
        sc = np.array([1.0, 0.5, 1.5]) if u[i, 6] < anisotropic else np.ones(3)
        m[i, :3, :3] = rz @ rx @ np.diag(s[i] * sc)
        m[i, :3, 3] = t[i]
        m[i, 3, 3] = 1.0
    return m.astype(np.float32)


def query_boxes(n: int, lo, hi, half_lo: float, half_hi: float, seed: int = 6) -> np.ndarray:
    """Collision query boxes ((n, 8) float32 {min.xyz, 1, max.xyz, 1}): centres uniform in
    [lo, hi], half-extents per axis uniform in [half_lo, half_hi]."""
    u = uniform(seed, 404, n * 6).reshape(n, 6)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    c = lo + (hi - lo) * u[:, :3]
    h = half_lo + (half_hi - half_lo) * u[:, 3:]
    b = np.ones((n, 8), dtype=np.float32)
    b[:, 0:3] = (c - h).astype(np.float32)
    b[:, 4:7] = (c + h).astype(np.float32)
    return b


# ---------------------------------------------------------------------------------------------
# Named workloads

C1_CAMERA = dict(eye=(0.0, -2.5, 1.5), target=(0.0, 0.0, 0.0), vfov_deg=60.0)
C2_CAMERA = dict(eye=(0.0, -9.0, 4.5), target=(0.0, 0.0, 0.6), vfov_deg=60.0)


def c1_heightfield_scene() -> Mesh:
    """Heightfield 256x256 (131,072 triangles) over [-1,1]^2, seed 1."""
    return heightfield(256, seed=1)


def c2_icosphere_scene(n_spheres: int = 64) -> Mesh:
    """64 displaced subdivision-5 icospheres + 2-triangle ground plane (1,310,722 triangles)."""
    return icosphere_set(n_spheres=n_spheres, subdiv=5, seed=2)


def c4_icosphere_scene() -> Mesh:
    """256 displaced subdivision-5 icospheres over [-8,8]^2 x [0,4], no ground (5,242,880 triangles:
    256 x 20,480; the precision workload's stated 4,194,304 does not match that shape)."""
    return icosphere_set(n_spheres=256, subdiv=5, seed=4, lo=(-8.0, -8.0, 0.0), hi=(8.0, 8.0, 4.0),
                         ground=None)


C4_BOUNDS = ((-8.0, -8.0, 0.0), (8.0, 8.0, 4.0))

C5_CAMERA = dict(eye=(0.0, -1.6, 2.2), target=(0.0, 0.0, 0.0), vfov_deg=60.0)


def c5_heightfield_scene(seed: int = 5) -> Mesh:
    """Heightfield 512x512 (524,288 triangles) over [-1,1]^2; vertex z are the parameters."""
    return heightfield(512, seed=seed)
