// Strict-mode device traversal: the reference's GLSL arithmetic and traversal order, bit-exact.
//
// Every floating-point operation is an explicit round-to-nearest intrinsic (__fmul_rn, __fadd_rn,
// __fsub_rn, __fdiv_rn), which the compiler never contracts into FMA, and min/max are the GLSL
// definitions min(x,y) = y < x ? y : x, max(x,y) = x < y ? y : x rather than the hardware
// min/max (whose NaN and signed-zero behaviour differs).  Operation order follows the GLSL
// source line by line; citations are to Source/Core/Shaders/Intersectors/Include/.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "rq_internal.h"
#include "rq_tlas.cuh"

namespace rq {
namespace strict {

struct f3 {
    float x, y, z;
};

__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) {
    return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 add(f3 a, f3 b) {
    return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 mul(f3 a, f3 b) {
    return {__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 muls(f3 a, float s) {
    return {__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
__device__ __forceinline__ f3 neg(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
            __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}
__device__ __forceinline__ f3 vmin(f3 a, f3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
__device__ __forceinline__ f3 vmax(f3 a, f3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
__device__ __forceinline__ f3 xyz(float4 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ f3 rcp3(f3 d) {
    return {__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z)};
}

// glm column-major mat4 * vec4(v, w), xyz; sums left to right.
__device__ __forceinline__ f3 xform(const float* m, f3 v, float w) {
    f3 r;
    r.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[4], v.y)),
                              __fmul_rn(m[8], v.z)), __fmul_rn(m[12], w));
    r.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[1], v.x), __fmul_rn(m[5], v.y)),
                              __fmul_rn(m[9], v.z)), __fmul_rn(m[13], w));
    r.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[2], v.x), __fmul_rn(m[6], v.y)),
                              __fmul_rn(m[10], v.z)), __fmul_rn(m[14], w));
    return r;
}

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }
__device__ __forceinline__ int4 ldg4i(const int4* p) { return __ldg(p); }
__device__ __forceinline__ f3 vpos(const SceneView& s, int32_t vi) {
    return xyz(ldg4(s.verts + 2 * static_cast<int64_t>(vi)));
}

// RayTriangle, TraverseBVHStack.glsl:87-105.  Returns t (or -1 outside the triangle).
__device__ __forceinline__ float ray_triangle(f3 ro, f3 rd, f3 v0, f3 v1, f3 v2) {
    const f3 v1v0 = sub(v1, v0);
    const f3 v2v0 = sub(v2, v0);
    const f3 rov0 = sub(ro, v0);
    const f3 n = cross(v1v0, v2v0);
    const f3 q = cross(rov0, rd);
    const float d = __fdiv_rn(1.0f, dot(rd, n));
    const float u = __fmul_rn(d, dot(neg(q), v2v0));
    const float v = __fmul_rn(d, dot(q, v1v0));
    float t = __fmul_rn(d, dot(neg(n), rov0));
    if (u < 0.0f || v < 0.0f || __fadd_rn(u, v) > 1.0f) t = -1.0f;
    return t;
}

// RayBounds (stack), TraverseBVHStack.glsl:107-116.
__device__ __forceinline__ float ray_bounds_stack(f3 ro, f3 inv, float4 bmin, float4 bmax,
                                                  float maxt) {
    const f3 f = mul(sub(xyz(bmax), ro), inv);
    const f3 n = mul(sub(xyz(bmin), ro), inv);
    const f3 tmax = vmax(f, n);
    const f3 tmin = vmin(f, n);
    const float t1 = gmin(gmin(tmax.x, gmin(tmax.y, tmax.z)), maxt);
    const float t0 = gmax(gmax(tmin.x, gmax(tmin.y, tmin.z)), 0.0f);
    return (t1 >= t0) ? (t0 > 0.0f ? t0 : t1) : -1.0f;
}

// RayBounds (stackless), TraverseBVHStackless.glsl:67-75, 100-109.
__device__ __forceinline__ float ray_bounds_stackless(float4 bmin, float4 bmax, f3 ro, f3 inv,
                                                      float t_min, float t_max) {
    const f3 t0 = mul(sub(xyz(bmin), ro), inv);
    const f3 t1 = mul(sub(xyz(bmax), ro), inv);
    const f3 a = vmin(t0, t1);
    const f3 b = vmax(t0, t1);
    const float tmin = gmax(gmax(gmax(a.x, a.y), a.z), t_min);
    const float tmax = gmin(gmin(b.x, gmin(b.y, b.z)), t_max);
    return (tmax >= tmin) ? tmin : -1.0f;
}

// ComputeBarycentrics, TraverseBVHStack.glsl:150-166.
__device__ __forceinline__ void barycentrics(f3 p, f3 a, f3 b, f3 c, float& u, float& v,
                                             float& w) {
    const f3 v0 = sub(b, a), v1 = sub(c, a), v2 = sub(p, a);
    const float d00 = dot(v0, v0);
    const float d01 = dot(v0, v1);
    const float d11 = dot(v1, v1);
    const float d20 = dot(v2, v0);
    const float d21 = dot(v2, v1);
    const float denom = __fsub_rn(__fmul_rn(d00, d11), __fmul_rn(d01, d01));
    v = __fdiv_rn(__fsub_rn(__fmul_rn(d11, d20), __fmul_rn(d01, d21)), denom);
    w = __fdiv_rn(__fsub_rn(__fmul_rn(d00, d21), __fmul_rn(d01, d20)), denom);
    u = __fsub_rn(__fsub_rn(1.0f, v), w);
}

struct Best {
    float tmax;
    float closest;
    int32_t tri;
    int32_t mesh;
};

template <bool kTieLower>
__device__ __forceinline__ bool accept(float t, float tmin, int32_t idx, const Best& b) {
    if (!(t > tmin)) return false;
    if (t < b.tmax) return true;
    return kTieLower && t == b.tmax && idx < b.tri;
}

// Leaf: triangles [start, start+len) (TraverseBVHStack.glsl:221-277).  kAny returns on the first
// accepted triangle.
template <bool kAny, bool kTieLower>
__device__ __forceinline__ bool test_leaf(const SceneView& s, f3 ro, f3 rd, int32_t start,
                                          int32_t len, float tmin, Best& b, int32_t& tests) {
    for (int32_t idx = start; idx < start + len; ++idx) {
        ++tests;
        const int4 tr = ldg4i(s.tris + idx);
        const float t = ray_triangle(ro, rd, vpos(s, tr.x), vpos(s, tr.y), vpos(s, tr.z));
        if (kAny) {
            if (t > tmin && t < b.tmax) {
                b.closest = t;
                return true;
            }
        } else if (accept<kTieLower>(t, tmin, idx, b)) {
            b.tmax = t;
            b.closest = t;
            b.mesh = tr.w;
            b.tri = idx;
        }
    }
    return false;
}

// IntersectBVHStack (:168-324) and IntersectBVHStackOcclusion (:509-657).  The 64-entry stack
// lives in local memory.  Returns the iteration count.
template <bool kAny, bool kTieLower>
__device__ int32_t bvh_stack(const SceneView& s, f3 ro, f3 rd, int32_t start, int32_t count,
                             float tmin, Best& b, int32_t& tests) {
    const f3 inv = rcp3(rd);
    int32_t stack[64];
    int32_t sp = 0;
    int32_t iters = 0;
    int32_t cur = start;
    while (iters < 1024) {
        if (sp >= 64 || sp < 0 || cur < start || cur > start + count || cur < 0 ||
            cur >= s.n_nodes)
            break;
        ++iters;
        const float4* nd = s.nodes + 4 * static_cast<int64_t>(cur);
        const float4 lmin = ldg4(nd + 0), lmax = ldg4(nd + 1);
        const float4 rmin = ldg4(nd + 2), rmax = ldg4(nd + 3);
        const int32_t lw = __float_as_int(lmin.w), rw = __float_as_int(rmin.w);
        const bool lleaf = lw != -1, rleaf = rw != -1;
        const float lt = lleaf ? -1.0f : ray_bounds_stack(ro, inv, lmin, lmax, b.tmax);
        const float rt = rleaf ? -1.0f : ray_bounds_stack(ro, inv, rmin, rmax, b.tmax);
        if (lleaf && test_leaf<kAny, kTieLower>(s, ro, rd, lw >> 4, lw & 0xF, tmin, b, tests)) break;
        if (rleaf && test_leaf<kAny, kTieLower>(s, ro, rd, rw >> 4, rw & 0xF, tmin, b, tests)) break;
        if (lt > 0.0f && rt > 0.0f) {
            cur = __float_as_int(lmax.w) + start;
            int32_t post = __float_as_int(rmax.w) + start;
            if (rt < lt) {
                const int32_t tmp = cur;
                cur = post;
                post = tmp;
            }
            if (sp >= 63) break;
            stack[sp++] = post;
            continue;
        } else if (lt > 0.0f) {
            cur = __float_as_int(lmax.w) + start;
            continue;
        } else if (rt > 0.0f) {
            cur = __float_as_int(rmax.w) + start;
            continue;
        }
        if (sp <= 0) break;
        cur = stack[--sp];
    }
    return iters;
}

// IntersectBVHStackless (:175-278) and IntersectBVHStacklessOcclusion (:463-556).
template <bool kAny, bool kTieLower>
__device__ int32_t bvh_stackless(const SceneView& s, f3 ro, f3 rd, int32_t start, int32_t count,
                                 float tmin, Best& b, int32_t& tests) {
    const f3 inv = rcp3(rd);
    int32_t iters = 0;
    int32_t ptr = start;
    while (ptr >= 0 && iters < 1024) {
        if (ptr < start || ptr > start + count || ptr < 0 || ptr >= s.n_nodes) break;
        ++iters;
        const float4* nd = s.nodes + 2 * static_cast<int64_t>(ptr);
        const float4 bmin = ldg4(nd), bmax = ldg4(nd + 1);
        const float bt = ray_bounds_stackless(bmin, bmax, ro, inv, 0.0001f, b.tmax);
        if (bt > 0.0f && bt < b.tmax) {
            const int32_t packed = __float_as_int(bmin.w);
            if (packed != -1) {
                if (test_leaf<kAny, kTieLower>(s, ro, rd, packed >> 4, packed & 0xF, tmin, b, tests))
                    break;
                ptr = __float_as_int(bmax.w);
                if (ptr < 0) break;
                ptr += start;
                continue;
            }
            ptr++;
            continue;
        }
        ptr = __float_as_int(bmax.w);
        if (ptr < 0) break;
        ptr += start;
    }
    return iters;
}

__device__ __forceinline__ float ent_alpha(const rq_entity& e) { return __int_as_float(e.data[1]); }

// IntersectScene's Iters under RQ_FLAG_REF_COMPAT: the shader hands one `out int Iters` to every
// entity's walk (TraverseBVHStack.glsl:337-349, :380-398), so it reports the iteration count of the
// last entity its loop walks: the last entity, or under IgnoreTransparent the last opaque one.
// `last_walked` / `last_count`: the last entity walked here and its count; an entity the top level
// passed over would have visited its root only (one iteration).  0 when the loop walks nothing.
__device__ __forceinline__ int32_t last_entity_iters(const SceneView& s, int flags, int32_t last_walked,
                                                     int32_t last_count) {
    int32_t L = s.n_ents - 1;
    if (flags & RQ_FLAG_IGNORE_TRANSPARENT)
        while (L >= 0 && ent_alpha(s.ents[L]) < 0.99f) --L;
    if (L < 0) return 0;
    return last_walked == L ? last_count : 1;
}

// IntersectScene / IntersectSceneIgnoreTransparent (:327-413; stackless :280-366).
template <bool kStackless, bool kTieLower, bool kTlas = true>
__device__ void scene_closest(const SceneView& s, const float4 r0, const float4 r1, int flags,
                              rq_hit& h, int32_t& tests) {
    h.t = h.u = h.v = h.w = -1.0f;
    h.tri = h.mesh = h.entity = -1;
    h.iters = 0;
    const float rtmin = r0.w, rtmax = r1.w;
    if (!(rtmax > rtmin)) return;
    const f3 o = xyz(r0), d = xyz(r1);
    float tmax = rtmax;
    float closest = -1.0f;
    int32_t mesh = -1, tri = -1, ent = -1, last_walked = -1, last_count = 0;
    const float3 wo = make_float3(o.x, o.y, o.z), wd = make_float3(d.x, d.y, d.z);
    int32_t cur = tlas::begin<kTlas>(s, wo, wd);
    const int counted = (flags & RQ_FLAG_IGNORE_TRANSPARENT) ? tlas::kOpaque : tlas::kAll;
    for (int i = -1; (i = tlas::next<kTlas>(s, cur, i, wo, wd, tmax, counted, h.iters)) >= 0;) {
        const rq_entity& e = s.ents[i];
        if ((flags & RQ_FLAG_IGNORE_TRANSPARENT) && ent_alpha(e) < 0.99f) continue;
        const f3 ro = xform(e.inverse, o, 1.0f);
        const f3 rd = xform(e.inverse, d, 0.0f);
        Best bb{tmax, -1.0f, kTieLower ? tri : -1, -1};
        const int32_t it =
            kStackless ? bvh_stackless<false, kTieLower>(s, ro, rd, e.node_offset, e.node_count, rtmin, bb, tests)
                       : bvh_stack<false, kTieLower>(s, ro, rd, e.node_offset, e.node_count, rtmin, bb, tests);
        h.iters += it;
        last_walked = i;
        last_count = it;
        const float T = bb.closest;
        if (T > 0.0f && (T < tmax || (kTieLower && T == tmax && bb.tri < tri))) {
            tmax = T;
            closest = T;
            mesh = bb.mesh;
            tri = bb.tri;
            ent = i;
        }
    }
    if (flags & RQ_FLAG_REF_COMPAT) h.iters = last_entity_iters(s, flags, last_walked, last_count);
    if (closest > 0.0f) {
        h.tri = tri;
        h.mesh = mesh;
        h.entity = ent;
        const bool report = (flags & RQ_FLAG_REF_COMPAT) ? tri > 0 : tri >= 0;
        if (report) {
            const rq_entity& e = s.ents[ent];
            const f3 ro = xform(e.inverse, o, 1.0f);
            const f3 rd = xform(e.inverse, d, 0.0f);
            const int4 tr = ldg4i(s.tris + tri);
            const f3 p = add(ro, muls(rd, closest));
            float u, v, w;
            barycentrics(p, vpos(s, tr.x), vpos(s, tr.y), vpos(s, tr.z), u, v, w);
            h.t = closest;
            h.u = u;
            h.v = v;
            h.w = w;
        }
    }
}

// IntersectSceneOcclusion (:659-676; stackless :558-575) with the per-ray TMax.
template <bool kStackless, bool kTlas = true>
__device__ bool scene_any(const SceneView& s, const float4 r0, const float4 r1, int32_t& iters,
                          int32_t& tests) {
    const float rtmin = r0.w, rtmax = r1.w;
    if (!(rtmax > rtmin)) return false;
    const f3 o = xyz(r0), d = xyz(r1);
    const float3 wo = make_float3(o.x, o.y, o.z), wd = make_float3(d.x, d.y, d.z);
    int32_t cur = tlas::begin<kTlas>(s, wo, wd);
    for (int i = -1; (i = tlas::next<kTlas>(s, cur, i, wo, wd, rtmax, tlas::kAll, iters)) >= 0;) {
        const rq_entity& e = s.ents[i];
        const f3 ro = xform(e.inverse, o, 1.0f);
        const f3 rd = xform(e.inverse, d, 0.0f);
        Best bb{rtmax, -1.0f, -1, -1};
        iters += kStackless
                     ? bvh_stackless<true, false>(s, ro, rd, e.node_offset, e.node_count, rtmin, bb, tests)
                     : bvh_stack<true, false>(s, ro, rd, e.node_offset, e.node_count, rtmin, bb, tests);
        if (bb.closest > 0.0f) return true;
    }
    return false;
}

}  // namespace strict
}  // namespace rq
