// Radiance probe volume update: one frame of the reference's UpdateRadianceProbes.glsl (dispatched
// by ProbeGI::UpdateProbes, ProbeGI.cpp:162-238).  One ray per probe, traced by the engine's
// closest-hit launch, a shadow ray toward the sun from each hit (any hit), then one thread per probe
// shades the hit, adds the previous volume's irradiance (SampleProbes), encodes L1 spherical
// harmonics, blends them with the reprojected previous frame and packs them.  All arithmetic is
// explicit round-to-nearest in the shader's evaluation order (no contraction), so the volume is
// bit-identical to the CPU restatement.
#include <cuda_runtime.h>

#include "rq_gi.cuh"
#include "rq_objects.h"

namespace rq {
namespace {

using strict::f3;

struct ProbeArgs {
    int32_t gx, gy, gz;
    f3 res, size, origin, prev;
    uint32_t seed;
    int32_t temporal, normal_mode;
    float shadow_offset, ray_tmax;
    f3 sun_dir, sun_color, sky;
};

ProbeArgs probe_args(const rq_probe_params& p) {
    ProbeArgs a;
    a.gx = p.grid[0];
    a.gy = p.grid[1];
    a.gz = p.grid[2];
    a.res = {static_cast<float>(a.gx), static_cast<float>(a.gy), static_cast<float>(a.gz)};
    a.size = {p.size[0], p.size[1], p.size[2]};
    a.origin = {p.origin[0], p.origin[1], p.origin[2]};
    a.prev = {p.prev_origin[0], p.prev_origin[1], p.prev_origin[2]};
    a.seed = p.seed;
    a.temporal = p.temporal;
    a.normal_mode = p.normal_mode;
    a.shadow_offset = p.shadow_offset;
    a.ray_tmax = p.ray_tmax;
    a.sun_dir = {p.sun_dir[0], p.sun_dir[1], p.sun_dir[2]};
    a.sun_color = {p.sun_color[0], p.sun_color[1], p.sun_color[2]};
    a.sky = {p.sky_color[0], p.sky_color[1], p.sky_color[2]};
    return a;
}

// SphericalHarmonics.glsl: struct SH {L00, L11, L10, L1_1} and its first-order basis constants.
struct SH4 {
    f3 l00, l11, l10, l1_1;
};
constexpr float kY00 = 0.28209479177387814347f;
constexpr float kY11 = -0.48860251190291992159f;
constexpr float kY10 = 0.48860251190291992159f;
constexpr float kY1_1 = -0.48860251190291992159f;

__device__ __forceinline__ f3 vdiv(f3 a, f3 b) { return {__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y), __fdiv_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 vdivs(f3 a, float s) { return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)}; }
__device__ __forceinline__ f3 vadds(f3 a, float s) { return {__fadd_rn(a.x, s), __fadd_rn(a.y, s), __fadd_rn(a.z, s)}; }
__device__ __forceinline__ f3 vmaxs(f3 a, float s) {
    return {strict::gmax(a.x, s), strict::gmax(a.y, s), strict::gmax(a.z, s)};
}
__device__ __forceinline__ float clamp01(float x) { return strict::gmin(strict::gmax(x, 0.0f), 1.0f); }
// GLSL mix(x, y, a) = x * (1 - a) + y * a.
__device__ __forceinline__ float mixf(float x, float y, float a) {
    return __fadd_rn(__fmul_rn(x, __fsub_rn(1.0f, a)), __fmul_rn(y, a));
}
__device__ __forceinline__ f3 vmix(f3 x, f3 y, float a) { return {mixf(x.x, y.x, a), mixf(x.y, y.y, a), mixf(x.z, y.z, a)}; }

__device__ __forceinline__ bool inside(const ProbeArgs& a, int x, int y, int z) {
    return x >= 0 && x < a.gx && y >= 0 && y < a.gy && z >= 0 && z < a.gz;
}
__device__ __forceinline__ int64_t probe_index(const ProbeArgs& a, int x, int y, int z) {
    return (static_cast<int64_t>(z) * a.gy + y) * a.gx + x;
}

// base + (2 * vec3(Pixel) / u_Resolution - 1) * u_Size (:412-417; GetVisibility :178-180).
__device__ __forceinline__ f3 probe_position(const ProbeArgs& a, f3 base, int x, int y, int z) {
    const f3 tc = vdiv(f3{static_cast<float>(x), static_cast<float>(y), static_cast<float>(z)}, a.res);
    const f3 clip = vadds(strict::muls(tc, 2.0f), -1.0f);
    return strict::add(base, strict::mul(clip, a.size));
}

// Normalised LambertBRDF (:351-372) of hash dimensions 0 and 1 of the probe index: phi = 2 pi h.x,
// cos(theta) = 2 h.y - 1, sin(theta) = sqrt(1 - cos^2); the radius cancels in the normalisation.
__device__ __forceinline__ f3 probe_direction(uint32_t seed, uint32_t id) {
    const float hx = gi::u01(gi::sample_key(seed, id, 0u)), hy = gi::u01(gi::sample_key(seed, id, 1u));
    float sp, cp;
    gi::sincos_turns(hx, sp, cp);
    const float c = __fsub_rn(__fmul_rn(2.0f, hy), 1.0f);
    const float st = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(c, c)));
    return gi::normalize(f3{__fmul_rn(st, cp), __fmul_rn(st, sp), c});
}

// UnitVectorToOctahedron (Octahedral.glsl) scaled by 7 and truncated; pixel x * 8 + y (:470-472).
__device__ __forceinline__ int oct_pixel(f3 d) {
    const float s = strict::dot(f3{fabsf(d.x), fabsf(d.y), fabsf(d.z)}, f3{1.0f, 1.0f, 1.0f});
    float x = __fdiv_rn(d.x, s), z = __fdiv_rn(d.z, s);
    if (d.y < 0.0f) {
        const float ox = x, oz = z;
        x = __fmul_rn(ox >= 0.0f ? 1.0f : -1.0f, __fsub_rn(1.0f, fabsf(oz)));
        z = __fmul_rn(oz >= 0.0f ? 1.0f : -1.0f, __fsub_rn(1.0f, fabsf(ox)));
    }
    const float u = clamp01(__fadd_rn(__fmul_rn(0.5f, x), 0.5f));
    const float v = clamp01(__fadd_rn(__fmul_rn(0.5f, z), 0.5f));
    return static_cast<int>(__fmul_rn(u, 7.0f)) * 8 + static_cast<int>(__fmul_rn(v, 7.0f));
}

// EncodeSH: each coefficient is 0 + Y * radiance * A.
__device__ __forceinline__ SH4 encode_sh(f3 rad, f3 dir) {
    const float pi = 3.14159265359f, m = 2.0f;
    const float a0 = __fmul_rn(m, pi), a1 = __fmul_rn(__fdiv_rn(__fmul_rn(2.0f, pi), 3.0f), m);
    const f3 z = {0.0f, 0.0f, 0.0f};
    SH4 r;
    r.l00 = strict::add(z, strict::muls(strict::muls(rad, kY00), a0));
    r.l1_1 = strict::add(z, strict::muls(strict::muls(rad, __fmul_rn(kY1_1, dir.y)), a1));
    r.l10 = strict::add(z, strict::muls(strict::muls(rad, __fmul_rn(kY10, dir.z)), a1));
    r.l11 = strict::add(z, strict::muls(strict::muls(rad, __fmul_rn(kY11, dir.x)), a1));
    return r;
}

// SampleSH(sh, direction): four clamped lobes summed in the shader's order.
__device__ __forceinline__ f3 sample_sh(const SH4& sh, f3 d) {
    f3 r = {0.0f, 0.0f, 0.0f};
    r = strict::add(r, vmaxs(strict::muls(sh.l00, kY00), 0.0f));
    r = strict::add(r, vmaxs(strict::muls(strict::muls(sh.l1_1, kY1_1), d.y), 0.0f));
    r = strict::add(r, vmaxs(strict::muls(strict::muls(sh.l10, kY10), d.z), 0.0f));
    r = strict::add(r, vmaxs(strict::muls(strict::muls(sh.l11, kY11), d.x), 0.0f));
    return r;
}

// packSnorm2x16 of one component: round(clamp(c, -1, 1) * 32767), half to even, NaN as 0.
__device__ __forceinline__ uint32_t snorm16(float c) {
    const float s = __fmul_rn(strict::gmin(strict::gmax(c, -1.0f), 1.0f), 32767.0f);
    if (s != s) return 0u;
    return static_cast<uint32_t>(static_cast<uint16_t>(static_cast<int16_t>(__float2int_rn(s))));
}
__device__ __forceinline__ uint32_t pack_snorm2(float a, float b) { return snorm16(a) | (snorm16(b) << 16); }
// f / 32767 for an int16 f, correctly rounded, by Markstein's correction step (P. Markstein, IBM J.
// Res. Dev. 34(1), 1990): q0 = f * y with y = RN(1/32767) = 0x1.0002p-15, r = f - q0 * 32767 (exact
// in one FMA), q = q0 + r * y.  Equal to the IEEE quotient for every one of the 65,536 numerators
// (checked exhaustively with exact rationals by tests/test_probe_math.py), at three instructions.
__device__ __forceinline__ float div32767(float f) {
    const float y = 0x1.0002p-15f;
    const float q0 = __fmul_rn(f, y);
    const float r = __fmaf_rn(-q0, 32767.0f, f);
    return __fmaf_rn(r, y, q0);
}
__device__ __forceinline__ float unsnorm16(uint32_t h) {
    const float f = static_cast<float>(static_cast<int16_t>(static_cast<uint16_t>(h & 0xFFFFu)));
    return strict::gmin(strict::gmax(div32767(f), -1.0f), 1.0f);
}
__device__ __forceinline__ float max3abs(f3 x) {
    return strict::gmax(strict::gmax(fabsf(x.x), fabsf(x.y)), fabsf(x.z));
}

// PackSH: coefficients divided by the largest magnitude (from -1000), six snorm pairs, the scale.
__device__ __forceinline__ void pack_sh(const SH4& sh, uint4& A, uint4& B) {
    float m = -1000.0f;
    m = strict::gmax(m, max3abs(sh.l00));
    m = strict::gmax(m, max3abs(sh.l11));
    m = strict::gmax(m, max3abs(sh.l10));
    m = strict::gmax(m, max3abs(sh.l1_1));
    const f3 a = vdivs(sh.l00, m), b = vdivs(sh.l11, m), c = vdivs(sh.l10, m), d = vdivs(sh.l1_1, m);
    A = make_uint4(pack_snorm2(a.x, a.y), pack_snorm2(a.z, b.x), pack_snorm2(b.y, b.z), pack_snorm2(c.x, c.y));
    B = make_uint4(pack_snorm2(c.z, d.x), pack_snorm2(d.y, d.z), __float_as_uint(m), 0u);
}

// UnpackSH: the snorm pairs times the scale stored in B.z.
__device__ __forceinline__ SH4 unpack_sh(const uint4 A, const uint4 B) {
    const float k = __uint_as_float(B.z);
    const uint32_t w[6] = {A.x, A.y, A.z, A.w, B.x, B.y};
    float u[12];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        u[2 * i] = __fmul_rn(unsnorm16(w[i]), k);
        u[2 * i + 1] = __fmul_rn(unsnorm16(w[i] >> 16), k);
    }
    return SH4{{u[0], u[1], u[2]}, {u[3], u[4], u[5]}, {u[6], u[7], u[8]}, {u[9], u[10], u[11]}};
}

// The previous volume's texel: zeros outside the volume.
__device__ __forceinline__ void load_texel(const ProbeArgs& a, const uint4* __restrict__ vol, int x, int y, int z,
                                           uint4& A, uint4& B) {
    if (!inside(a, x, y, z)) {
        A = B = make_uint4(0u, 0u, 0u, 0u);
        return;
    }
    const int64_t i = probe_index(a, x, y, z);
    A = __ldg(vol + 2 * i);
    B = __ldg(vol + 2 * i + 1);
}

// GetVisibility (:176-188) of the probe at pp: clamp(dot(N, direction to it), 0, 1)^2 (pow(x, 2)
// as x * x).
__device__ __forceinline__ float probe_visibility(f3 pp, f3 wp, f3 n) {
    f3 v = strict::sub(pp, wp);
    const float len = __fsqrt_rn(strict::dot(v, v));
    v = vdivs(v, len);
    const float w = clamp01(strict::dot(n, v));
    return __fmul_rn(w, w);
}

// SampleProbes (:190-237) over the previous volume.
__device__ f3 sample_probes(const ProbeArgs& a, const uint4* __restrict__ vol, f3 wp, f3 n) {
    wp = strict::add(wp, strict::muls(n, 0.45f));
    f3 sp = vdiv(strict::sub(wp, a.prev), a.size);
    sp = vadds(strict::muls(sp, 0.5f), 0.5f);
    if (!(sp.x == clamp01(sp.x) && sp.y == clamp01(sp.y) && sp.z == clamp01(sp.z))) return {0.0f, 0.0f, 0.0f};
    const f3 vc = strict::mul(sp, a.res);
    const f3 mn = {floorf(vc.x), floorf(vc.y), floorf(vc.z)};
    const f3 mx = {ceilf(vc.x), ceilf(vc.y), ceilf(vc.z)};
    const f3 ext = strict::sub(mx, mn);
    const float inv = __fdiv_rn(1.0f, __fmul_rn(__fmul_rn(ext.x, ext.y), ext.z));
    const float ax = __fsub_rn(mx.x, vc.x), ay = __fsub_rn(mx.y, vc.y), az = __fsub_rn(mx.z, vc.z);
    const float bx = __fsub_rn(vc.x, mn.x), by = __fsub_rn(vc.y, mn.y), bz = __fsub_rn(vc.z, mn.z);
    auto w3 = [&](float p, float q, float r) { return __fmul_rn(__fmul_rn(__fmul_rn(p, q), r), inv); };
    float w[8] = {w3(ax, ay, az), w3(ax, by, az), w3(bx, by, az), w3(bx, ay, az),
                  w3(ax, ay, bz), w3(ax, by, bz), w3(bx, by, bz), w3(bx, ay, bz)};
    const int x0 = static_cast<int>(mn.x), y0 = static_cast<int>(mn.y), z0 = static_cast<int>(mn.z);
    const int x1 = static_cast<int>(mx.x), y1 = static_cast<int>(mx.y), z1 = static_cast<int>(mx.z);
    const int tx[8] = {x0, x0, x1, x1, x0, x0, x1, x1}, ty[8] = {y0, y1, y1, y0, y0, y1, y1, y0};
    const int tz[8] = {z0, z0, z0, z0, z1, z1, z1, z1};
    // the corners' probe positions, one coordinate per axis and bound (each component of
    // probe_position depends on its own axis only)
    const f3 p0 = probe_position(a, a.prev, x0, y0, z0), p1 = probe_position(a, a.prev, x1, y1, z1);
    float alpha = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const bool bx1 = i == 2 || i == 3 || i == 6 || i == 7, by1 = i == 1 || i == 2 || i == 5 || i == 6;
        const f3 pp = {bx1 ? p1.x : p0.x, by1 ? p1.y : p0.y, i >= 4 ? p1.z : p0.z};
        const float vis = probe_visibility(pp, wp, n);
        alpha = __fadd_rn(alpha, __fmul_rn(w[i], __fsub_rn(1.0f, vis)));
        w[i] = __fmul_rn(w[i], vis);
    }
    const float ws = strict::gmax(__fsub_rn(1.0f, alpha), 0.000001f);
    SH4 f = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        uint4 A, B;
        load_texel(a, vol, tx[i], ty[i], tz[i], A, B);
        const SH4 s = unpack_sh(A, B);
        const float k = __fdiv_rn(w[i], ws);
        f.l00 = strict::add(f.l00, strict::muls(s.l00, k));
        f.l1_1 = strict::add(f.l1_1, strict::muls(s.l1_1, k));
        f.l10 = strict::add(f.l10, strict::muls(s.l10, k));
        f.l11 = strict::add(f.l11, strict::muls(s.l11, k));
    }
    return vmaxs(sample_sh(f, n), 0.0f);
}

// Reproject (:298-313): the previous volume's texel under the world position, or false.
__device__ __forceinline__ bool reproject(const ProbeArgs& a, f3 wp, int& x, int& y, int& z) {
    f3 sp = vdiv(strict::sub(wp, a.prev), a.size);
    sp = vadds(strict::muls(sp, 0.5f), 0.5f);
    if (!(sp.x > 0.0f && sp.x < 1.0f && sp.y > 0.0f && sp.y < 1.0f && sp.z > 0.0f && sp.z < 1.0f)) return false;
    sp = vadds(strict::mul(sp, a.res), 0.5f);
    x = static_cast<int>(sp.x);
    y = static_cast<int>(sp.y);
    z = static_cast<int>(sp.z);
    return true;
}

__device__ __forceinline__ void put(rq_ray* out, int64_t i, f3 o, f3 d, float tmax) {
    float4* p = reinterpret_cast<float4*>(out) + 2 * i;
    p[0] = make_float4(o.x, o.y, o.z, 0.0f);
    p[1] = make_float4(d.x, d.y, d.z, tmax);
}

// One ray per probe from the probe position (:410-427).
__global__ void k_probe_raygen(ProbeArgs a, int64_t n, rq_ray* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = static_cast<int>(i % a.gx), y = static_cast<int>((i / a.gx) % a.gy);
    const int z = static_cast<int>(i / (static_cast<int64_t>(a.gx) * a.gy));
    put(out, i, probe_position(a, a.origin, x, y, z), probe_direction(a.seed, static_cast<uint32_t>(i)), a.ray_tmax);
}

// Shadow ray toward the sun from the hit of probe i (inactive without a hit).
__global__ void k_probe_shadow(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                               int64_t n, ProbeArgs a, rq_ray* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* hp = reinterpret_cast<const float4*>(hits) + 2 * i;
    const float4 h0 = __ldg(hp), h1f = __ldg(hp + 1);
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * i;
    const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    if (!(h0.x > 0.0f) || !(r1.w > r0.w)) {
        put(out, i, f3{0.0f, 0.0f, 0.0f}, f3{0.0f, 0.0f, 1.0f}, -1.0f);
        return;
    }
    const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
    const f3 P = strict::add(ro, strict::muls(rd, h0.x));
    f3 N = gi::hit_normal(s, __float_as_int(h1f.x), h0.y, h0.z, h0.w, a.normal_mode);
    if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
    put(out, i, strict::add(P, strict::muls(N, a.shadow_offset)), strict::neg(a.sun_dir), 1000000.0f);
}

// The value an unsigned float with a 5-bit exponent (bias 15) and `mbits` mantissa bits holds
// for x: the R and G (6 bits) and B (5 bits) channels of GL_R11F_G11F_B10F, the format of the
// reference's raw radiance images (UpdateRadianceProbes.glsl:17-18, ProbeGI.cpp:100, 110).  As the
// GL specification converts: finite values to the closest representable one (ties to even here),
// negative values and -inf to 0, values above the largest finite one to it, +inf and NaN kept.
// Every step is an exact binary32 operation (power-of-two scaling, round to integer).
__device__ __forceinline__ float to_small_ufloat(float x, int mbits) {
    if (x != x || x == INFINITY) return x;
    if (!(x > 0.0f)) return 0.0f;
    const float maxf = ldexpf(2.0f - ldexpf(1.0f, -mbits), 15);
    if (x >= maxf) return maxf;
    int k;
    frexpf(x, &k);                      // x in [2^(k-1), 2^k)
    const int e = max(k - 1, -14);      // subnormals share the step of the smallest binade
    const float step = ldexpf(1.0f, e - mbits);
    const float q = __fmul_rn(rintf(__fdiv_rn(x, step)), step);
    return q > maxf ? maxf : q;
}
__device__ __forceinline__ f3 to_r11g11b10(f3 v) {
    return {to_small_ufloat(v.x, 6), to_small_ufloat(v.y, 6), to_small_ufloat(v.z, 5)};
}

// UpdateRadianceProbes.glsl main after the trace (:440-519), one thread per probe.  raw_r11: store
// the raw radiance as the r11f_g11f_b10f image holds it (RQ_FLAG_REF_COMPAT).
__global__ void k_probe_shade(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                              const uint8_t* __restrict__ occl, int64_t n, const Materials mat, ProbeArgs a,
                              const uint4* __restrict__ prev_sh, const float4* __restrict__ prev_raw,
                              float2* __restrict__ map, uint4* __restrict__ out_sh, float4* __restrict__ out_raw,
                              int raw_r11) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * i;
    const f3 o = strict::xyz(__ldg(pr)), d = strict::xyz(__ldg(pr + 1));
    const float4* hp = reinterpret_cast<const float4*>(hits) + 2 * i;
    const float4 h0 = __ldg(hp), h1f = __ldg(hp + 1);
    const float t = h0.x;
    f3 N = {-1.0f, -1.0f, -1.0f}, alb = {0.0f, 0.0f, 0.0f};
    float em = 0.0f;
    if (t > 0.0f) {
        const int4 h1 = make_int4(__float_as_int(h1f.x), __float_as_int(h1f.y), __float_as_int(h1f.z), 0);
        N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
        alb = gi::hit_albedo(s, mat, h0, h1);
        em = __int_as_float(s.ents[h1.z].data[0]);
    }
    if (strict::dot(N, d) > 0.0001f) N = strict::neg(N);
    const f3 wp = strict::add(o, strict::muls(d, t));
    const float lsky = clamp01(strict::dot(d, f3{0.0f, 1.0f, 0.0f}));
    f3 fr;
    if (t < 0.0f) {
        fr = strict::muls(strict::muls(a.sky, 2.2f), lsky);
    } else {
        const float shadow = occl ? (occl[i] ? 0.0f : 1.0f) : 1.0f;
        const float ndl = clamp01(strict::dot(N, strict::neg(a.sun_dir)));
        const f3 direct = vmaxs(strict::muls(strict::muls(strict::mul(alb, a.sun_color), shadow), ndl), 0.0f);
        fr = strict::add(direct, strict::muls(strict::muls(alb, em), 1.0f));
    }
    if (t > 0.0f) {
        const f3 b = sample_probes(a, prev_sh, strict::add(wp, strict::muls(N, 0.001f)), N);
        fr = strict::add(fr, strict::mul(strict::muls(b, 0.999f), alb));
    }
    float2* px = map + 64 * i + oct_pixel(d);
    const float depth = t < 0.0f ? 256.0f : t, depth2 = __fmul_rn(depth, depth);
    SH4 sh = encode_sh(fr, d);
    int32_t frames = 0;
    int rx, ry, rz;
    if (reproject(a, o, rx, ry, rz)) {
        uint4 A, B;
        load_texel(a, prev_sh, rx, ry, rz, A, B);
        frames = static_cast<int32_t>(B.w + 1u);
        const float ta = a.temporal
                             ? strict::gmin(__fsub_rn(1.0f, __fdiv_rn(1.0f, __int2float_rn(frames))), 0.98f)
                             : 0.0f;
        const float2 m = *px;
        *px = make_float2(mixf(depth, m.x, ta), mixf(depth2, m.y, ta));
        const SH4 ps = unpack_sh(A, B);
        sh.l00 = vmix(sh.l00, ps.l00, ta);
        sh.l11 = vmix(sh.l11, ps.l11, ta);
        sh.l10 = vmix(sh.l10, ps.l10, ta);
        sh.l1_1 = vmix(sh.l1_1, ps.l1_1, ta);
        f3 praw = {0.0f, 0.0f, 0.0f};
        if (inside(a, rx, ry, rz)) praw = strict::xyz(__ldg(prev_raw + probe_index(a, rx, ry, rz)));
        fr = vmix(fr, praw, ta);
    } else {
        *px = make_float2(depth, depth2);
    }
    uint4 A, B;
    pack_sh(sh, A, B);
    B.w = static_cast<uint32_t>(frames);
    out_sh[2 * i] = A;
    out_sh[2 * i + 1] = B;
    if (raw_r11) fr = to_r11g11b10(fr);
    out_raw[i] = make_float4(fr.x, fr.y, fr.z, 0.0f);
}

inline unsigned grid(int64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace
}  // namespace rq

using rq::fail;

extern "C" {

rq_status rq_probe_update(rq_ctx* ctx, const rq_scene* sc, const rq_probe_params* p, const uint32_t* prev_sh,
                          const float* prev_raw, float* probe_map, uint32_t* out_sh, float* out_raw,
                          const rq_opts* opts, void* stream) {
    if (!ctx || !sc || !p) return fail(ctx, RQ_EINVAL, "bad arguments");
    if (p->grid[0] < 1 || p->grid[1] < 1 || p->grid[2] < 1 || p->grid[0] > 4096 || p->grid[1] > 4096 ||
        p->grid[2] > 4096)
        return fail(ctx, RQ_EINVAL, "probe grid dimensions must be in [1, 4096]");
    const int64_t n = static_cast<int64_t>(p->grid[0]) * p->grid[1] * p->grid[2];
    if (n > (int64_t(1) << 31)) return fail(ctx, RQ_EINVAL, "more than 2^31 probes");
    if (!prev_sh || !prev_raw || !probe_map || !out_sh || !out_raw) return fail(ctx, RQ_EINVAL, "null buffer");
    if (p->normal_mode != 0 && p->normal_mode != 1) return fail(ctx, RQ_EINVAL, "bad normal_mode");
    rq::QueryConfig q{};
    rq_status s;
    if ((s = rq::resolve_query(ctx, sc, opts, q)) != RQ_OK) return s;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool host = (q.flags & RQ_FLAG_HOST_BUFFERS) != 0;
    q.flags &= ~RQ_FLAG_HOST_BUFFERS;
    const size_t b_sh = 32 * static_cast<size_t>(n), b_raw = 16 * static_cast<size_t>(n);
    const size_t b_map = 512 * static_cast<size_t>(n);
    void *d_ray = nullptr, *d_hit = nullptr, *d_sh = nullptr, *d_occ = nullptr;
    // scratch: the GI pass's slots (passes on one context are stream-ordered, never concurrent)
    if ((s = rq::scratch(ctx, rq::kSlotRays, sizeof(rq_ray) * n, &d_ray)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotHits, sizeof(rq_hit) * n, &d_hit)) != RQ_OK)
        return s;
    const uint32_t* psh = prev_sh;
    const float* praw = prev_raw;
    float* pmap = probe_map;
    uint32_t* osh = out_sh;
    float* oraw = out_raw;
    if (host) {
        void *a = nullptr, *b = nullptr, *c = nullptr, *d = nullptr, *e = nullptr;
        if ((s = rq::scratch(ctx, rq::kSlotProbeStageSh, b_sh, &a)) != RQ_OK || (s = rq::scratch(ctx, rq::kSlotProbeStageRaw, b_raw, &b)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotProbeStageMap, b_map, &c)) != RQ_OK || (s = rq::scratch(ctx, rq::kSlotProbeStageOutSh, b_sh, &d)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotStageOut, b_raw, &e)) != RQ_OK)
            return s;
        RQ_CUDA(ctx, cudaMemcpyAsync(a, prev_sh, b_sh, cudaMemcpyHostToDevice, st));
        RQ_CUDA(ctx, cudaMemcpyAsync(b, prev_raw, b_raw, cudaMemcpyHostToDevice, st));
        RQ_CUDA(ctx, cudaMemcpyAsync(c, probe_map, b_map, cudaMemcpyHostToDevice, st));
        psh = static_cast<const uint32_t*>(a);
        praw = static_cast<const float*>(b);
        pmap = static_cast<float*>(c);
        osh = static_cast<uint32_t*>(d);
        oraw = static_cast<float*>(e);
    } else {
        auto misaligned = [](const void* ptr, uintptr_t k) { return (reinterpret_cast<uintptr_t>(ptr) % k) != 0; };
        if (misaligned(prev_sh, 16) || misaligned(out_sh, 16) || misaligned(prev_raw, 16) ||
            misaligned(out_raw, 16) || misaligned(probe_map, 8))
            return fail(ctx, RQ_EINVAL, "probe volumes must be 16-byte aligned (the map 8-byte)");
        const char* lo_a = reinterpret_cast<const char*>(prev_sh);
        const char* lo_b = reinterpret_cast<const char*>(out_sh);
        const char* lo_c = reinterpret_cast<const char*>(prev_raw);
        const char* lo_d = reinterpret_cast<const char*>(out_raw);
        if ((lo_a < lo_b + b_sh && lo_b < lo_a + b_sh) || (lo_c < lo_d + b_raw && lo_d < lo_c + b_raw))
            return fail(ctx, RQ_EINVAL, "previous and output volumes overlap");
    }
    const rq::ProbeArgs a = rq::probe_args(*p);
    rq_ray* ray = static_cast<rq_ray*>(d_ray);
    rq_hit* hit = static_cast<rq_hit*>(d_hit);
    rq::k_probe_raygen<<<rq::grid(n, 256), 256, 0, st>>>(a, n, ray);
    RQ_CUDA(ctx, cudaGetLastError());
    RQ_CUDA(ctx, rq::launch_closest(sc->view, q, ray, n, hit, rq::queue_counter(ctx, 1), st));
    const uint8_t* occ = nullptr;
    if (p->shadow_rays) {
        if ((s = rq::scratch(ctx, rq::kSlotShadowRays, sizeof(rq_ray) * n, &d_sh)) != RQ_OK || (s = rq::scratch(ctx, rq::kSlotOccluded, n, &d_occ)) != RQ_OK)
            return s;
        rq::k_probe_shadow<<<rq::grid(n, 256), 256, 0, st>>>(sc->view, ray, hit, n, a, static_cast<rq_ray*>(d_sh));
        RQ_CUDA(ctx, cudaGetLastError());
        RQ_CUDA(ctx, rq::launch_anyhit(sc->view, q, static_cast<rq_ray*>(d_sh), n, static_cast<uint8_t*>(d_occ),
                                       rq::queue_counter(ctx, 2), st));
        occ = static_cast<const uint8_t*>(d_occ);
    }
    rq::k_probe_shade<<<rq::grid(n, 128), 128, 0, st>>>(
        sc->view, ray, hit, occ, n, rq::materials_of(sc), a, reinterpret_cast<const uint4*>(psh),
        reinterpret_cast<const float4*>(praw), reinterpret_cast<float2*>(pmap), reinterpret_cast<uint4*>(osh),
        reinterpret_cast<float4*>(oraw), (q.flags & RQ_FLAG_REF_COMPAT) ? 1 : 0);
    RQ_CUDA(ctx, cudaGetLastError());
    if (host) {
        RQ_CUDA(ctx, cudaMemcpyAsync(out_sh, osh, b_sh, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaMemcpyAsync(out_raw, oraw, b_raw, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaMemcpyAsync(probe_map, pmap, b_map, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return RQ_OK;
}

}  // extern "C"
