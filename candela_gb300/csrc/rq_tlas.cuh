// Entity cursor over the top-level BVH (tlas.h): the entities a ray can touch, in ascending index
// order, so the scene loops keep the reference's order, TMax and tie handling.  A scene without a
// top level, or a ray with a non-finite origin or direction, walks every entity.
//
// The cursor state is one int: the next top-level node (>= 0), kEnd once the walk has run past
// the last node, kDone once the remaining entities have been counted, or kPlain for the plain
// loop.  The caller keeps the last entity it was given (`prev`, -1 before the first).
#pragma once
#include <cuda_runtime.h>

#include "rq_internal.h"

namespace rq {
namespace tlas {

// Which entities the caller's loop would have walked (each skipped one adds one iteration).
enum Count : int { kAll = -1, kOpaque = 0, kBvh8 = 1, kBvh8Opaque = 2 };

constexpr int32_t kEnd = -1, kDone = -2, kPlain = -3;

__device__ __forceinline__ bool finite3(float x, float y, float z) {
    return isfinite(x) && isfinite(y) && isfinite(z);
}

// kTlas = false: the kernel was launched for a scene without a top level (plain loop only).
template <bool kTlas>
__device__ __forceinline__ int32_t begin(const SceneView& s, float3 o, float3 d) {
    if (!kTlas) return kPlain;
    return s.tlas != nullptr && finite3(o.x, o.y, o.z) && finite3(d.x, d.y, d.z) ? 0 : kPlain;
}

// Entities in [lo, hi) that the caller's loop would have walked.
__device__ __forceinline__ int32_t walked(const SceneView& s, int32_t lo, int32_t hi, int count) {
    if (hi <= lo) return 0;
    if (count == kAll) return hi - lo;
    const int* p = reinterpret_cast<const int*>(s.tlas_pre);
    return __ldg(p + 4 * hi + count) - __ldg(p + 4 * lo + count);
}

// next() with a budget: at most `budget` top-level nodes are tested per call; kMore when the
// budget ran out before an entity was found (the cursor keeps its place, so the next call
// continues the same walk).  The persistent kernels interleave these bounded steps with the node
// steps of the other lanes instead of running a whole top-level walk while the warp waits.
constexpr int32_t kMore = -4;

template <bool kTlas>
__device__ __forceinline__ int32_t next_n(const SceneView& s, int32_t& c, int32_t prev, float3 o, float3 d,
                                          float tmax, int count, int32_t& skipped, int budget) {
    if (!kTlas || c == kPlain) return prev + 1 < s.n_ents ? prev + 1 : -1;
    if (c == kDone) return -1;
    const float m = s.tlas_margin * fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    const float ix = __frcp_rn(d.x), iy = __frcp_rn(d.y), iz = __frcp_rn(d.z);
    const float tlim = tmax * (1.0f + 1.0f / 65536.0f);
    while (c >= 0) {
        if (budget-- <= 0) return kMore;
        const float4 a = __ldg(s.tlas + 2 * c), b = __ldg(s.tlas + 2 * c + 1);
        const float x0 = (a.x - m - o.x) * ix, x1 = (b.x + m - o.x) * ix;
        const float y0 = (a.y - m - o.y) * iy, y1 = (b.y + m - o.y) * iy;
        const float z0 = (a.z - m - o.z) * iz, z1 = (b.z + m - o.z) * iz;
        const float tn = fmaxf(fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fminf(z0, z1)), 0.0f);
        const float tf = fminf(fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1)), tlim);
        const int32_t link = __float_as_int(b.w);
        if (tn <= tf) {
            const int32_t e = __float_as_int(a.w);
            if (e >= 0) {
                skipped += walked(s, prev + 1, e, count);
                c = link;
                return e;
            }
            ++c;
        } else {
            c = link;
        }
    }
    skipped += walked(s, prev + 1, s.n_ents, count);
    c = kDone;
    return -1;
}

// Next entity after `prev` to walk, or -1 when none is left.  `tmax` is the loop's running TMax:
// subtrees whose widened boxes start beyond it are skipped (the walk of such an entity would
// stop at its root as well).  `skipped` receives the iterations of the entities passed over.
// The slab test runs on the widened box; fminf / fmaxf drop the NaN of a zero direction component
// whose origin lies on a widened face (outside the entity's own box by the margin).
template <bool kTlas>
__device__ __forceinline__ int32_t next(const SceneView& s, int32_t& c, int32_t prev, float3 o, float3 d,
                                        float tmax, int count, int32_t& skipped) {
    return next_n<kTlas>(s, c, prev, o, d, tmax, count, skipped, 0x7FFFFFFF);
}

// Nearest-first walk (BVH8 closest hit).  The closest hit over a scene is the lexicographic
// minimum of (t, triangle, entity) whatever order the entities are walked in, as long as each walk
// keeps everything at or below the running TMax (the BVH8 boxes are conservative) and an equal
// (t, triangle) from a lower entity replaces the current hit.  So the candidates can come in
// order of their widened boxes' entry distance, and a candidate whose box starts beyond the
// running TMax is dropped: fewer walks, the same hit.  Only the BVH8 visit count differs from the
// ascending walk.  Stack entries are (entry distance bits << 32 | node); the tree is at most
// 24 + log2(entities) deep, far below kNearStack.
constexpr int kNearStack = 64;

struct Near {
    int32_t sp;
};

// Entry distance of node c's widened box, or a negative value when the ray misses it or meets it
// only beyond tlim.
__device__ __forceinline__ float near_tn(const SceneView& s, int32_t c, float m, float3 o, float ix, float iy,
                                         float iz, float tlim) {
    const float4 a = __ldg(s.tlas + 2 * c), b = __ldg(s.tlas + 2 * c + 1);
    const float x0 = (a.x - m - o.x) * ix, x1 = (b.x + m - o.x) * ix;
    const float y0 = (a.y - m - o.y) * iy, y1 = (b.y + m - o.y) * iy;
    const float z0 = (a.z - m - o.z) * iz, z1 = (b.z + m - o.z) * iz;
    const float tn = fmaxf(fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fminf(z0, z1)), 0.0f);
    const float tf = fminf(fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1)), tlim);
    return tn <= tf ? tn : -1.0f;
}

__device__ __forceinline__ void near_push(uint64_t* st, Near& w, int32_t node, float tn, unsigned& status) {
    if (w.sp >= kNearStack) {
        status |= 1u;  // stack overflow (cannot happen below 2^39 entities)
        return;
    }
    st[w.sp++] = (static_cast<uint64_t>(__float_as_uint(tn)) << 32) | static_cast<uint32_t>(node);
}

// Starts the walk: the root on the stack when the ray meets its box.
__device__ __forceinline__ void near_begin(const SceneView& s, Near& w, uint64_t* st, float3 o, float3 d,
                                           float tmax, unsigned& status) {
    w.sp = 0;
    const float m = s.tlas_margin * fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    const float tn = near_tn(s, 0, m, o, __frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z),
                             tmax * (1.0f + 1.0f / 65536.0f));
    if (tn >= 0.0f) near_push(st, w, 0, tn, status);
}

// Next candidate entity, nearest box first; -1 when none is left, kMore when `budget` interior
// nodes were expanded without reaching one.
__device__ __forceinline__ int32_t near_next(const SceneView& s, Near& w, uint64_t* st, float3 o, float3 d,
                                             float tmax, int budget, unsigned& status) {
    const float m = s.tlas_margin * fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    const float ix = __frcp_rn(d.x), iy = __frcp_rn(d.y), iz = __frcp_rn(d.z);
    const float tlim = tmax * (1.0f + 1.0f / 65536.0f);
    while (w.sp > 0) {
        const uint64_t top = st[--w.sp];
        const int32_t c = static_cast<int32_t>(static_cast<uint32_t>(top));
        if (__uint_as_float(static_cast<uint32_t>(top >> 32)) > tlim) continue;  // beyond the running TMax
        const int32_t e = __float_as_int(__ldg(s.tlas + 2 * c).w);
        if (e >= 0) return e;
        if (budget-- <= 0) {
            ++w.sp;  // the node stays on top for the next call
            return kMore;
        }
        const int32_t l = c + 1, r = __float_as_int(__ldg(s.tlas + 2 * l + 1).w);
        const float tl = near_tn(s, l, m, o, ix, iy, iz, tlim), tr = near_tn(s, r, m, o, ix, iy, iz, tlim);
        if (tl >= 0.0f && tr >= 0.0f) {
            if (tr < tl) {
                near_push(st, w, l, tl, status);
                near_push(st, w, r, tr, status);
            } else {
                near_push(st, w, r, tr, status);
                near_push(st, w, l, tl, status);
            }
        } else if (tl >= 0.0f) {
            near_push(st, w, l, tl, status);
        } else if (tr >= 0.0f) {
            near_push(st, w, r, tr, status);
        }
    }
    return -1;
}

}  // namespace tlas
}  // namespace rq
