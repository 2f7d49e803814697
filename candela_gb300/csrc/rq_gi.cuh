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

// ModelColor of a mesh (GetData, TraverseBVHStack.glsl:440-451); 0.8 grey without an entry.
__device__ __forceinline__ f3 mesh_albedo(const Materials& mat, int32_t mesh) {
    if (mesh >= 0 && mesh < mat.n_albedo)
        return {__ldg(mat.albedo + 3 * mesh), __ldg(mat.albedo + 3 * mesh + 1), __ldg(mat.albedo + 3 * mesh + 2)};
    return {0.8f, 0.8f, 0.8f};
}

// The colour channels of texel (i, j): byte / 255, or the sRGB table for an sRGB texture.
__device__ __forceinline__ f3 texel(const Materials& mat, int32_t first, int32_t w, int32_t i, int32_t j, bool srgb) {
    const uint32_t t = __ldg(mat.texels + first + static_cast<int64_t>(j) * w + i);
    const uint32_t r = t & 0xFFu, g = (t >> 8) & 0xFFu, b = (t >> 16) & 0xFFu;
    if (srgb) return {__ldg(mat.srgb + r), __ldg(mat.srgb + g), __ldg(mat.srgb + b)};
    return {__fdiv_rn(static_cast<float>(r), 255.0f), __fdiv_rn(static_cast<float>(g), 255.0f),
            __fdiv_rn(static_cast<float>(b), 255.0f)};
}

// Texel index along one axis: GL_REPEAT (positive modulo) or GL_CLAMP_TO_EDGE.
__device__ __forceinline__ int32_t wrap_texel(int32_t i, int32_t n, bool clamp) {
    if (clamp) return i < 0 ? 0 : (i >= n ? n - 1 : i);
    const int32_t r = i % n;
    return r < 0 ? r + n : r;
}

// texture(Textures[Ref], uv).xyz in a compute shader: level 0 (no derivatives), bilinear (the
// GL_LINEAR magnification filter), texel centres at half-integers: x = u * width - 0.5,
// i0 = floor(x), a = x - i0, and the four texels weighted (1-a)(1-b), a(1-b), (1-a)b, ab, summed
// in that order.  sRGB channels are decoded before filtering.  Coordinates beyond +-2^30 texels
// are clamped there (the float has no fraction left at that size).
__device__ inline f3 sample_texture(const Materials& mat, int32_t t, float u, float v) {
    const int4 d = __ldg(mat.tex + t);
    const bool srgb = d.w & 1, clamp = d.w & 2;
    const float x = __fsub_rn(__fmul_rn(u, static_cast<float>(d.y)), 0.5f);
    const float y = __fsub_rn(__fmul_rn(v, static_cast<float>(d.z)), 0.5f);
    const float fx = fminf(fmaxf(floorf(x), -1073741824.0f), 1073741824.0f);
    const float fy = fminf(fmaxf(floorf(y), -1073741824.0f), 1073741824.0f);
    const float a = fminf(fmaxf(__fsub_rn(x, fx), 0.0f), 1.0f), b = fminf(fmaxf(__fsub_rn(y, fy), 0.0f), 1.0f);
    const int32_t ix = static_cast<int32_t>(fx), iy = static_cast<int32_t>(fy);
    const int32_t i0 = wrap_texel(ix, d.y, clamp), i1 = wrap_texel(ix + 1, d.y, clamp);
    const int32_t j0 = wrap_texel(iy, d.z, clamp), j1 = wrap_texel(iy + 1, d.z, clamp);
    const float na = __fsub_rn(1.0f, a), nb = __fsub_rn(1.0f, b);
    const float w00 = __fmul_rn(na, nb), w10 = __fmul_rn(a, nb), w01 = __fmul_rn(na, b), w11 = __fmul_rn(a, b);
    const f3 t00 = texel(mat, d.x, d.y, i0, j0, srgb), t10 = texel(mat, d.x, d.y, i1, j0, srgb);
    const f3 t01 = texel(mat, d.x, d.y, i0, j1, srgb), t11 = texel(mat, d.x, d.y, i1, j1, srgb);
    return strict::add(strict::add(strict::add(strict::muls(t00, w00), strict::muls(t10, w10)), strict::muls(t01, w01)),
                       strict::muls(t11, w11));
}

// Albedo of a hit (GetData, TraverseBVHStack.glsl:422-455): the mesh's texture at the hit's UV
// (texture coordinates half-packed in Vertex.PackedData.w, weighted by the barycentrics u, v, w)
// when it has one, else its ModelColor.
__device__ __forceinline__ f3 hit_albedo(const SceneView& s, const Materials& mat, const float4 h0, const int4 h1) {
    const int32_t mesh = h1.y;
    if (mesh >= 0 && mesh < mat.n_mesh_tex && h0.x > 0.0f) {
        const int32_t t = __ldg(mat.mesh_tex + mesh);
        if (t >= 0) {
            const int4 tr = __ldg(s.tris + h1.x);
            const uint32_t ta = __float_as_uint(__ldg(s.verts + 2 * static_cast<int64_t>(tr.x) + 1).w);
            const uint32_t tb = __float_as_uint(__ldg(s.verts + 2 * static_cast<int64_t>(tr.y) + 1).w);
            const uint32_t tc = __float_as_uint(__ldg(s.verts + 2 * static_cast<int64_t>(tr.z) + 1).w);
            const float u = __fadd_rn(__fadd_rn(__fmul_rn(half_bits(ta), h0.y), __fmul_rn(half_bits(tb), h0.z)),
                                      __fmul_rn(half_bits(tc), h0.w));
            const float v = __fadd_rn(__fadd_rn(__fmul_rn(half_bits(ta >> 16), h0.y),
                                                __fmul_rn(half_bits(tb >> 16), h0.z)),
                                      __fmul_rn(half_bits(tc >> 16), h0.w));
            return sample_texture(mat, t, u, v);
        }
    }
    return mesh_albedo(mat, mesh);
}

// reflect(I, N) = I - 2 dot(N, I) N (GLSL).
__device__ __forceinline__ f3 reflect(f3 i, f3 n) {
    return strict::sub(i, strict::muls(n, __fmul_rn(2.0f, strict::dot(n, i))));
}

// SampleGGXVNDF, Sampling.glsl:63-83 (a GGX half-vector sample about N; the turn-based sine and
// cosine stand in for cos(2 pi x) / sin(2 pi x)).
__device__ __forceinline__ f3 sample_ggx(f3 n, float roughness, float x0, float x1) {
    const float alpha = __fmul_rn(roughness, roughness);
    const float alpha2 = __fmul_rn(alpha, alpha);
    float sp, cp;
    sincos_turns(x0, sp, cp);
    const float ct = __fsqrt_rn(__fdiv_rn(__fsub_rn(1.0f, x1), __fadd_rn(1.0f, __fmul_rn(__fsub_rn(alpha2, 1.0f), x1))));
    const float st = __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(ct, ct)));
    const f3 h = {__fmul_rn(cp, st), __fmul_rn(sp, st), ct};
    const f3 up = fabsf(n.z) < 0.999f ? f3{0.0f, 0.0f, 1.0f} : f3{1.0f, 0.0f, 0.0f};
    const f3 tangent = normalize(strict::cross(up, n));
    const f3 bitangent = strict::cross(n, tangent);
    return normalize(strict::add(strict::add(strict::muls(tangent, h.x), strict::muls(bitangent, h.y)),
                                 strict::muls(n, h.z)));
}

}  // namespace gi
}  // namespace rq
