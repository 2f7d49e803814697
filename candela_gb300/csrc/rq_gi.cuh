// Diffuse-GI / RTAO ray generation and hit shading (device side).
//
// Follows Shaders/DiffuseTrace.glsl:439-494 and Shaders/Include/Sampling.glsl:1-12.  The
// reference draws its random numbers from a fract(sin()) hash whose value depends on the driver's
// sin; here they come from a counter-based integer hash (pcg_hash, Jarzynski & Olano 2020), and
// cos/sin(2*pi*x) come from the fixed polynomial in sincos_turns, so that ray generation is
// bit-reproducible between the GPU and the CPU restatement.  All arithmetic is explicit
// round-to-nearest (no contraction), like the strict traversal.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "rq_strict.cuh"

namespace rq {
namespace gi {

using strict::f3;

__device__ __forceinline__ uint32_t pcg_hash(uint32_t x) {
    const uint32_t state = x * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ __forceinline__ uint32_t sample_key(uint32_t seed, uint32_t ray, uint32_t dim) {
    return pcg_hash(pcg_hash(pcg_hash(seed) + ray) + dim);
}
__device__ __forceinline__ float u01(uint32_t h) {
    return __fmul_rn(__uint2float_rn(h >> 8), 1.0f / 16777216.0f);
}

// sin(2*pi*x), cos(2*pi*x), x in [0,1): quadrant reduction, reflection to [0, pi/4] and Taylor
// polynomials (sin to degree 9, cos to degree 10) in Horner form.
__device__ __forceinline__ void sincos_turns(float x, float& so, float& co) {
    const float x4 = __fmul_rn(x, 4.0f);
    const float q = floorf(x4);
    float f = __fsub_rn(x4, q);
    const int quad = static_cast<int>(q) & 3;
    const bool refl = f > 0.5f;
    if (refl) f = __fsub_rn(1.0f, f);
    const float th = __fmul_rn(f, 1.57079637f);
    const float t2 = __fmul_rn(th, th);
    float sp = 2.75573192e-06f;
    sp = __fadd_rn(__fmul_rn(sp, t2), -1.98412698e-04f);
    sp = __fadd_rn(__fmul_rn(sp, t2), 8.33333333e-03f);
    sp = __fadd_rn(__fmul_rn(sp, t2), -1.66666667e-01f);
    sp = __fadd_rn(__fmul_rn(sp, t2), 1.0f);
    float S = __fmul_rn(th, sp);
    float cp = -2.75573192e-07f;
    cp = __fadd_rn(__fmul_rn(cp, t2), 2.48015873e-05f);
    cp = __fadd_rn(__fmul_rn(cp, t2), -1.38888889e-03f);
    cp = __fadd_rn(__fmul_rn(cp, t2), 4.16666667e-02f);
    cp = __fadd_rn(__fmul_rn(cp, t2), -0.5f);
    cp = __fadd_rn(__fmul_rn(cp, t2), 1.0f);
    float C = cp;
    if (refl) {
        const float tmp = S;
        S = C;
        C = tmp;
    }
    switch (quad) {
        case 0: so = S; co = C; break;
        case 1: so = C; co = -S; break;
        case 2: so = -S; co = -C; break;
        default: so = -C; co = S; break;
    }
}

__device__ __forceinline__ f3 normalize(f3 v) {
    const float l = __fsqrt_rn(strict::dot(v, v));
    return {__fdiv_rn(v.x, l), __fdiv_rn(v.y, l), __fdiv_rn(v.z, l)};
}

// CosWeightedHemisphere, Sampling.glsl:1-12.
__device__ __forceinline__ f3 cos_weighted_hemisphere(f3 n, float r0, float r1) {
    const f3 uu = normalize(strict::cross(n, f3{0.0f, 1.0f, 1.0f}));
    const f3 vv = strict::cross(uu, n);
    const float ra = __fsqrt_rn(r1);
    float s, c;
    sincos_turns(r0, s, c);
    const float rx = __fmul_rn(ra, c);
    const float ry = __fmul_rn(ra, s);
    const float rz = __fsqrt_rn(__fsub_rn(1.0f, r1));
    const f3 rr = strict::add(strict::add(strict::muls(uu, rx), strict::muls(vv, ry)),
                              strict::muls(n, rz));
    return normalize(rr);
}

__device__ __forceinline__ float half_bits(uint32_t h) {
    return __half2float(__ushort_as_half(static_cast<unsigned short>(h & 0xFFFFu)));
}

// UnpackNormal, TraverseBVHStack.glsl:417-420.
__device__ __forceinline__ f3 unpack_normal(const SceneView& s, int32_t vi) {
    const float4 w = __ldg(s.verts + 2 * static_cast<int64_t>(vi) + 1);
    const uint32_t a = __float_as_uint(w.x), b = __float_as_uint(w.y);
    return {half_bits(a), half_bits(a >> 16), half_bits(b)};
}

// Shading normal: interpolated vertex normal (GetData, TraverseBVHStack.glsl:438) or geometric.
__device__ __forceinline__ f3 hit_normal(const SceneView& s, int32_t tri, float u, float v,
                                         float w, int mode) {
    const int4 tr = __ldg(s.tris + tri);
    if (mode == 0) {
        const f3 a = strict::muls(unpack_normal(s, tr.x), u);
        const f3 b = strict::muls(unpack_normal(s, tr.y), v);
        const f3 c = strict::muls(unpack_normal(s, tr.z), w);
        return normalize(strict::add(strict::add(a, b), c));
    }
    const f3 A = strict::vpos(s, tr.x), B = strict::vpos(s, tr.y), C = strict::vpos(s, tr.z);
    return normalize(strict::cross(strict::sub(B, A), strict::sub(C, A)));
}

}  // namespace gi
}  // namespace rq
