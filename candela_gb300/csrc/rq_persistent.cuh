// Persistent "while-if" traversal driver.
//
// A grid of (SM count x resident blocks) threads loops until the ray queue is empty.  Each
// iteration advances every lane's ray by one BVH node; a lane whose ray has finished takes the
// next ray from a global counter (one warp-aggregated atomicAdd per refill) in the same iteration,
// so lanes stay busy while long rays in the warp continue.  Per ray, the node order, iteration
// caps and acceptance tests are exactly those of the one-thread-per-ray strict functions in
// rq_strict.cuh (same arithmetic helpers), so results are bit-identical; only the assignment of
// rays to threads changes.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>

#include "rq_strict.cuh"

namespace rq {

// Resident-grid size of a persistent kernel (SM count x resident blocks), cached per device.
template <class K>
int persistent_grid(K kernel, int block) {
    static std::mutex mu;
    static std::unordered_map<long long, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    const long long key = (reinterpret_cast<long long>(reinterpret_cast<const void*>(kernel)) << 6) ^ dev;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    const int g = sms * (per_sm > 0 ? per_sm : 1);
    cache[key] = g;
    return g;
}
namespace persist {

using strict::f3;

// Traversal of one ray through the scene's entities, one node per step().
template <bool kAny, bool kStackless, bool kTieLower, bool kTlas = true>
struct StrictRay {
    // world ray
    f3 o, d;
    float rtmin, rtmax;
    // scene-level result (IntersectScene, TraverseBVHStack.glsl:327-366)
    float tmax, closest;
    int32_t mesh, tri, ent_hit, iters_total;
    int32_t last_walked, last_count;  // the last entity walked and its count (RQ_FLAG_REF_COMPAT)
    // current entity traversal (IntersectBVHStack / IntersectBVHStackless)
    int32_t ent, start, count, cur, sp, iters;
    int32_t ents;  // entity cursor (rq_tlas.cuh); `ent` is the last entity it gave
    f3 ro, rd, inv;
    strict::Best bb;
    bool occluded;

    __device__ __forceinline__ void setup_entity(const rq_entity& e) {
        ro = strict::xform(e.inverse, o, 1.0f);
        rd = strict::xform(e.inverse, d, 0.0f);
        inv = strict::rcp3(rd);
        start = e.node_offset;
        count = e.node_count;
        cur = start;
        sp = 0;
        iters = 0;
        bb = strict::Best{kAny ? rtmax : tmax, -1.0f, (!kAny && kTieLower) ? tri : -1, -1};
    }

    // Skips to the next entity that is traversed (ignore-transparent filter); false when done.
    __device__ __forceinline__ bool begin_entity(const SceneView& s, int flags) {
        const bool skip_transparent = !kAny && (flags & RQ_FLAG_IGNORE_TRANSPARENT);
        const float3 wo = make_float3(o.x, o.y, o.z), wd = make_float3(d.x, d.y, d.z);
        while ((ent = tlas::next<kTlas>(s, ents, ent, wo, wd, kAny ? rtmax : tmax,
                                 skip_transparent ? tlas::kOpaque : tlas::kAll, iters_total)) >= 0) {
            const rq_entity& e = s.ents[ent];
            if (skip_transparent && strict::ent_alpha(e) < 0.99f) continue;
            setup_entity(e);
            return true;
        }
        return false;
    }

    // begin_entity() in bounded steps of at most `budget` top-level nodes: 1 = the walk of entity
    // `ent` is set up, 0 = keep seeking, -1 = no entity left.
    __device__ __forceinline__ int seek(const SceneView& s, int flags, int budget) {
        const bool skip_transparent = !kAny && (flags & RQ_FLAG_IGNORE_TRANSPARENT);
        const int32_t e = tlas::next_n<kTlas>(s, ents, ent, make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z),
                                              kAny ? rtmax : tmax, skip_transparent ? tlas::kOpaque : tlas::kAll,
                                              iters_total, budget);
        if (e == tlas::kMore) return 0;
        if (e < 0) return -1;
        ent = e;
        const rq_entity& E = s.ents[ent];
        if (skip_transparent && strict::ent_alpha(E) < 0.99f) return 0;
        setup_entity(E);
        return 1;
    }

    // The world ray's state; false for an inactive ray.
    __device__ __forceinline__ bool init_ray(const SceneView& s, float4 r0, float4 r1) {
        o = strict::xyz(r0);
        d = strict::xyz(r1);
        rtmin = r0.w;
        rtmax = r1.w;
        tmax = rtmax;
        closest = -1.0f;
        mesh = tri = ent_hit = -1;
        iters_total = 0;
        last_walked = -1;
        last_count = 0;
        occluded = false;
        ent = -1;
        if (!(rtmax > rtmin)) return false;  // inactive ray
        ents = tlas::begin<kTlas>(s, make_float3(o.x, o.y, o.z), make_float3(d.x, d.y, d.z));
        return true;
    }

    __device__ __forceinline__ bool init(const SceneView& s, float4 r0, float4 r1, int flags) {
        return init_ray(s, r0, r1) && begin_entity(s, flags);
    }

    // Scene-level acceptance at the end of an entity's walk; false when the ray is done (any hit).
    __device__ __forceinline__ bool accept_entity() {
        iters_total += iters;
        last_walked = ent;
        last_count = iters;
        const float T = bb.closest;
        if (kAny) {
            if (T > 0.0f) {
                occluded = true;
                return false;
            }
        } else if (T > 0.0f && (T < tmax || (kTieLower && T == tmax && bb.tri < tri))) {
            tmax = T;
            closest = T;
            mesh = bb.mesh;
            tri = bb.tri;
            ent_hit = ent;
        }
        return true;
    }

    // Ends the current entity: scene-level acceptance, then the next entity.  false = ray done.
    __device__ __forceinline__ bool end_entity(const SceneView& s, int flags) {
        return accept_entity() && begin_entity(s, flags);
    }

    // One node of the current entity.  Returns true when this entity's traversal has ended.
    // `stack` is the lane's 64-entry traversal stack (kept outside the struct so that the struct's
    // scalar state stays in registers).
    __device__ __forceinline__ bool step(const SceneView& s, int32_t* stack, int32_t& tests) {
        if (kStackless) {
            if (!(cur >= 0 && iters < 1024)) return true;
            if (cur < start || cur > start + count || cur >= s.n_nodes) return true;
            ++iters;
            const float4* nd = s.nodes + 2 * static_cast<int64_t>(cur);
            const float4 bmin = strict::ldg4(nd), bmax = strict::ldg4(nd + 1);
            const float bt = strict::ray_bounds_stackless(bmin, bmax, ro, inv, 0.0001f, bb.tmax);
            if (bt > 0.0f && bt < bb.tmax) {
                const int32_t packed = __float_as_int(bmin.w);
                if (packed != -1) {
                    if (strict::test_leaf<kAny, kTieLower>(s, ro, rd, packed >> 4, packed & 0xF,
                                                           rtmin, bb, tests))
                        return true;
                    const int32_t nx = __float_as_int(bmax.w);
                    if (nx < 0) return true;
                    cur = nx + start;
                    return false;
                }
                ++cur;
                return false;
            }
            const int32_t nx = __float_as_int(bmax.w);
            if (nx < 0) return true;
            cur = nx + start;
            return false;
        } else {
            if (iters >= 1024) return true;
            if (sp >= 64 || sp < 0 || cur < start || cur > start + count || cur < 0 ||
                cur >= s.n_nodes)
                return true;
            ++iters;
            const float4* nd = s.nodes + 4 * static_cast<int64_t>(cur);
            const float4 lmin = strict::ldg4(nd + 0), lmax = strict::ldg4(nd + 1);
            const float4 rmin = strict::ldg4(nd + 2), rmax = strict::ldg4(nd + 3);
            const int32_t lw = __float_as_int(lmin.w), rw = __float_as_int(rmin.w);
            const bool lleaf = lw != -1, rleaf = rw != -1;
            const float lt = lleaf ? -1.0f : strict::ray_bounds_stack(ro, inv, lmin, lmax, bb.tmax);
            const float rt = rleaf ? -1.0f : strict::ray_bounds_stack(ro, inv, rmin, rmax, bb.tmax);
            if (lleaf && strict::test_leaf<kAny, kTieLower>(s, ro, rd, lw >> 4, lw & 0xF, rtmin,
                                                            bb, tests))
                return true;
            if (rleaf && strict::test_leaf<kAny, kTieLower>(s, ro, rd, rw >> 4, rw & 0xF, rtmin,
                                                            bb, tests))
                return true;
            if (lt > 0.0f && rt > 0.0f) {
                int32_t a = __float_as_int(lmax.w) + start;
                int32_t b = __float_as_int(rmax.w) + start;
                if (rt < lt) {
                    const int32_t t = a;
                    a = b;
                    b = t;
                }
                cur = a;
                if (sp >= 63) return true;
                stack[sp++] = b;
                return false;
            } else if (lt > 0.0f) {
                cur = __float_as_int(lmax.w) + start;
                return false;
            } else if (rt > 0.0f) {
                cur = __float_as_int(rmax.w) + start;
                return false;
            }
            if (sp <= 0) return true;
            cur = stack[--sp];
            return false;
        }
    }

    // Closest-hit record (barycentrics from the hit point, :351-363).
    __device__ __forceinline__ void finish(const SceneView& s, int flags, rq_hit& h) const {
        h.t = h.u = h.v = h.w = -1.0f;
        h.tri = h.mesh = h.entity = -1;
        h.iters = iters_total;
        if ((flags & RQ_FLAG_REF_COMPAT) && rtmax > rtmin)
            h.iters = strict::last_entity_iters(s, flags, last_walked, last_count);
        if (closest > 0.0f) {
            h.tri = tri;
            h.mesh = mesh;
            h.entity = ent_hit;
            const bool report = (flags & RQ_FLAG_REF_COMPAT) ? tri > 0 : tri >= 0;
            if (report) {
                const rq_entity& e = s.ents[ent_hit];
                const f3 pro = strict::xform(e.inverse, o, 1.0f);
                const f3 prd = strict::xform(e.inverse, d, 0.0f);
                const int4 tr = strict::ldg4i(s.tris + tri);
                const f3 p = strict::add(pro, strict::muls(prd, closest));
                float u, v, w;
                strict::barycentrics(p, strict::vpos(s, tr.x), strict::vpos(s, tr.y),
                                     strict::vpos(s, tr.z), u, v, w);
                h.t = closest;
                h.u = u;
                h.v = v;
                h.w = w;
            }
        }
    }
};

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-aggregated fetch of the next ray index for every lane with need == true.
__device__ __forceinline__ int64_t fetch(unsigned long long* next, bool need) {
    const unsigned mask = __activemask();
    const unsigned want = __ballot_sync(mask, need);
    unsigned long long base = 0;
    const int leader = __ffs(want) - 1;
    if (want && static_cast<int>(threadIdx.x & 31) == leader)
        base = atomicAdd(next, static_cast<unsigned long long>(__popc(want)));
    base = __shfl_sync(mask, base, leader < 0 ? 0 : leader);
    return need ? static_cast<int64_t>(base + __popc(want & lanemask_lt())) : -1;
}

}  // namespace persist
}  // namespace rq
