// Fast-mode BVH2 traversal (RQ_MODE_FAST): the reference's traversal order (near child first,
// push the far one; skip links for the stackless layout) with cheaper arithmetic:
//  * slab test t = fma(b, inv, -o*inv) with the origin term precomputed per ray and hardware
//    3-input min/max (IEEE minNum semantics);
//  * Moller-Trumbore with FMA on precomputed records {v0, mesh}, {e1, 0}, {e2, 0} (48 bytes, in the
//    reference triangle order), no index indirection;
//  * barycentrics straight from the triangle test; ties in t go to the lower triangle index.
// Results differ from strict mode only where rounding decides a grazing hit or a near tie.
#pragma once
#include <cuda_runtime.h>

#include "rq_bvh8.cuh"
#include "rq_strict.cuh"

namespace rq {
namespace fast {

using strict::f3;

struct Ray {
    f3 o, d, inv, oinv;
};

__device__ __forceinline__ Ray make_ray(f3 o, f3 d) {
    Ray r;
    r.o = o;
    r.d = d;
    auto safe = [](float x) { return fabsf(x) > 1e-30f ? x : copysignf(1e-30f, x); };
    r.inv = {1.0f / safe(d.x), 1.0f / safe(d.y), 1.0f / safe(d.z)};
    r.oinv = {o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z};
    return r;
}

// Reference RayBounds structure (stack): returns entry distance (or exit when inside), -1 on miss.
__device__ __forceinline__ float box_stack(const Ray& r, float4 bmin, float4 bmax, float maxt) {
    const float x0 = fmaf(bmin.x, r.inv.x, -r.oinv.x), x1 = fmaf(bmax.x, r.inv.x, -r.oinv.x);
    const float y0 = fmaf(bmin.y, r.inv.y, -r.oinv.y), y1 = fmaf(bmax.y, r.inv.y, -r.oinv.y);
    const float z0 = fmaf(bmin.z, r.inv.z, -r.oinv.z), z1 = fmaf(bmax.z, r.inv.z, -r.oinv.z);
    const float t1 = fminf(bvh8::min3f(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1)), maxt);
    const float t0 = fmaxf(bvh8::max3f(fminf(x0, x1), fminf(y0, y1), fminf(z0, z1)), 0.0f);
    return (t1 >= t0) ? (t0 > 0.0f ? t0 : t1) : -1.0f;
}

// Reference RayBounds structure (stackless, t_min = 1e-4).
__device__ __forceinline__ float box_stackless(const Ray& r, float4 bmin, float4 bmax, float tmax_) {
    const float x0 = fmaf(bmin.x, r.inv.x, -r.oinv.x), x1 = fmaf(bmax.x, r.inv.x, -r.oinv.x);
    const float y0 = fmaf(bmin.y, r.inv.y, -r.oinv.y), y1 = fmaf(bmax.y, r.inv.y, -r.oinv.y);
    const float z0 = fmaf(bmin.z, r.inv.z, -r.oinv.z), z1 = fmaf(bmax.z, r.inv.z, -r.oinv.z);
    const float tmin = fmaxf(bvh8::max3f(fminf(x0, x1), fminf(y0, y1), fminf(z0, z1)), 0.0001f);
    const float tmax = fminf(bvh8::min3f(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1)), tmax_);
    return (tmax >= tmin) ? tmin : -1.0f;
}

struct Best {
    float tmax, closest, u, v;
    int32_t tri, mesh;
};

// Moller-Trumbore on a fast record; returns t (or -1) and the weights of v1, v2.
__device__ __forceinline__ float mt(const Ray& r, const float4 a, const float4 b, const float4 c,
                                    float& bu, float& bv) {
    const f3 v0 = strict::xyz(a), e1 = strict::xyz(b), e2 = strict::xyz(c);
    const f3 p = {r.d.y * e2.z - r.d.z * e2.y, r.d.z * e2.x - r.d.x * e2.z, r.d.x * e2.y - r.d.y * e2.x};
    const float det = e1.x * p.x + e1.y * p.y + e1.z * p.z;
    const float id = 1.0f / det;
    const f3 tv = {r.o.x - v0.x, r.o.y - v0.y, r.o.z - v0.z};
    bu = (tv.x * p.x + tv.y * p.y + tv.z * p.z) * id;
    const f3 q = {tv.y * e1.z - tv.z * e1.y, tv.z * e1.x - tv.x * e1.z, tv.x * e1.y - tv.y * e1.x};
    bv = (r.d.x * q.x + r.d.y * q.y + r.d.z * q.z) * id;
    const float t = (e2.x * q.x + e2.y * q.y + e2.z * q.z) * id;
    return (bu >= 0.0f && bv >= 0.0f && bu + bv <= 1.0f) ? t : -1.0f;
}

template <bool kAny>
__device__ __forceinline__ bool leaf(const SceneView& s, const Ray& r, int32_t start, int32_t len,
                                     float tmin, Best& b, int32_t& tests) {
    for (int32_t idx = start; idx < start + len; ++idx) {
        ++tests;
        const float4* rec = s.tri_fast + 3 * static_cast<int64_t>(idx);
        const float4 A = __ldg(rec), B = __ldg(rec + 1), C = __ldg(rec + 2);
        float bu, bv;
        const float t = mt(r, A, B, C, bu, bv);
        if (kAny) {
            if (t > tmin && t < b.tmax) {
                b.closest = t;
                return true;
            }
        } else if (t > tmin && (t < b.tmax || (t == b.tmax && idx < b.tri))) {
            b.tmax = t;
            b.closest = t;
            b.u = bu;
            b.v = bv;
            b.tri = idx;
            b.mesh = __float_as_int(A.w);
        }
    }
    return false;
}

template <bool kAny>
__device__ int32_t bvh_stack(const SceneView& s, const Ray& r, int32_t start, int32_t count,
                             float tmin, Best& b, int32_t& tests) {
    int32_t stack[64];
    int32_t sp = 0, iters = 0, cur = start;
    while (iters < 1024) {
        if (sp >= 64 || cur < start || cur > start + count || cur >= s.n_nodes) break;
        ++iters;
        const float4* nd = s.nodes + 4 * static_cast<int64_t>(cur);
        const float4 lmin = __ldg(nd), lmax = __ldg(nd + 1), rmin = __ldg(nd + 2), rmax = __ldg(nd + 3);
        const int32_t lw = __float_as_int(lmin.w), rw = __float_as_int(rmin.w);
        const bool ll = lw != -1, rl = rw != -1;
        const float lt = ll ? -1.0f : box_stack(r, lmin, lmax, b.tmax);
        const float rt = rl ? -1.0f : box_stack(r, rmin, rmax, b.tmax);
        if (ll && leaf<kAny>(s, r, lw >> 4, lw & 0xF, tmin, b, tests)) break;
        if (rl && leaf<kAny>(s, r, rw >> 4, rw & 0xF, tmin, b, tests)) break;
        if (lt > 0.0f && rt > 0.0f) {
            int32_t a = __float_as_int(lmax.w) + start, c = __float_as_int(rmax.w) + start;
            if (rt < lt) {
                const int32_t x = a;
                a = c;
                c = x;
            }
            cur = a;
            if (sp >= 63) break;
            stack[sp++] = c;
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

template <bool kAny>
__device__ int32_t bvh_stackless(const SceneView& s, const Ray& r, int32_t start, int32_t count,
                                 float tmin, Best& b, int32_t& tests) {
    int32_t iters = 0, ptr = start;
    while (ptr >= 0 && iters < 1024) {
        if (ptr < start || ptr > start + count || ptr >= s.n_nodes) break;
        ++iters;
        const float4* nd = s.nodes + 2 * static_cast<int64_t>(ptr);
        const float4 bmin = __ldg(nd), bmax = __ldg(nd + 1);
        const float bt = box_stackless(r, bmin, bmax, b.tmax);
        if (bt > 0.0f && bt < b.tmax) {
            const int32_t packed = __float_as_int(bmin.w);
            if (packed != -1) {
                if (leaf<kAny>(s, r, packed >> 4, packed & 0xF, tmin, b, tests)) break;
                const int32_t nx = __float_as_int(bmax.w);
                if (nx < 0) break;
                ptr = nx + start;
                continue;
            }
            ++ptr;
            continue;
        }
        const int32_t nx = __float_as_int(bmax.w);
        if (nx < 0) break;
        ptr = nx + start;
    }
    return iters;
}

// Scene loop (IntersectScene structure), closest or any hit.
template <bool kAny, bool kStackless, bool kTlas = true>
__device__ void scene(const SceneView& s, const float4 r0, const float4 r1, int flags, rq_hit& h,
                      bool& occluded, int32_t& tests) {
    h.t = h.u = h.v = h.w = -1.0f;
    h.tri = h.mesh = h.entity = -1;
    h.iters = 0;
    occluded = false;
    const float rtmin = r0.w, rtmax = r1.w;
    if (!(rtmax > rtmin)) return;
    const f3 o = strict::xyz(r0), d = strict::xyz(r1);
    Best best{rtmax, -1.0f, 0.0f, 0.0f, -1, -1};
    int32_t ent = -1, last_walked = -1, last_count = 0;
    const bool skip_transparent = !kAny && (flags & RQ_FLAG_IGNORE_TRANSPARENT);
    const float3 wo = make_float3(o.x, o.y, o.z), wd = make_float3(d.x, d.y, d.z);
    int32_t cur = tlas::begin<kTlas>(s, wo, wd);
    for (int i = -1; (i = tlas::next<kTlas>(s, cur, i, wo, wd, kAny ? rtmax : best.tmax,
                                skip_transparent ? tlas::kOpaque : tlas::kAll, h.iters)) >= 0;) {
        const rq_entity& e = s.ents[i];
        if (skip_transparent && strict::ent_alpha(e) < 0.99f) continue;
        const Ray r = make_ray(strict::xform(e.inverse, o, 1.0f), strict::xform(e.inverse, d, 0.0f));
        Best bb = best;
        bb.closest = -1.0f;
        if (kAny) bb.tmax = rtmax;
        const int32_t it = kStackless ? bvh_stackless<kAny>(s, r, e.node_offset, e.node_count, rtmin, bb, tests)
                                      : bvh_stack<kAny>(s, r, e.node_offset, e.node_count, rtmin, bb, tests);
        h.iters += it;
        last_walked = i;
        last_count = it;
        if (kAny) {
            if (bb.closest > 0.0f) {
                occluded = true;
                return;
            }
        } else if (bb.closest > 0.0f) {
            best = bb;
            ent = i;
        }
    }
    if (!kAny && (flags & RQ_FLAG_REF_COMPAT)) h.iters = strict::last_entity_iters(s, flags, last_walked, last_count);
    if (!kAny && best.closest > 0.0f) {
        h.tri = best.tri;
        h.mesh = best.mesh;
        h.entity = ent;
        if (!(flags & RQ_FLAG_REF_COMPAT) || best.tri > 0) {
            h.t = best.closest;
            h.u = 1.0f - best.u - best.v;
            h.v = best.u;
            h.w = best.v;
        }
    }
}

}  // namespace fast
}  // namespace rq
