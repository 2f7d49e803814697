// AABB collision queries (the reference's Collide.comp): for each query box, the first entity and
// triangle it overlaps, walking each entity's BVH with box/box tests and testing leaf triangles
// with the reference's separating-axis test.  Stack layout: Intersectors/Include/CollideBVHStack.glsl:
// 154-323; stackless layout: Intersectors/Include/CollideBVHStackless.glsl:131-247 (the walk of
// Physics.cpp:79-174).
// Arithmetic is the strict IEEE binary32 form of rq_strict.cuh (no contraction, GLSL min/max),
// so results equal the CPU restatement bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "rq_objects.h"
#include "rq_persistent.cuh"
#include "rq_strict.cuh"

namespace rq {
namespace {

using strict::f3;

__device__ __forceinline__ f3 mid3(f3 a, f3 b) {
    return {__fdiv_rn(__fadd_rn(a.x, b.x), 2.0f), __fdiv_rn(__fadd_rn(a.y, b.y), 2.0f),
            __fdiv_rn(__fadd_rn(a.z, b.z), 2.0f)};
}

// BoxTriangleOverlap (CollideBVHStack.glsl:104-152, Physics.cpp:29-77): nine edge cross-product axes, full box extent
// as e.  ref_axis repeats cross(u2, f2) in slot 5 as the reference does (cross(u1, f2) belongs
// there).
__device__ bool box_triangle_overlap(f3 v0, f3 v1, f3 v2, f3 bmin, f3 bmax, bool ref_axis) {
    const f3 c = mid3(bmin, bmax);
    const f3 e = strict::sub(bmax, bmin);
    v0 = strict::sub(v0, c);
    v1 = strict::sub(v1, c);
    v2 = strict::sub(v2, c);
    const f3 f0 = strict::sub(v1, v0), f1 = strict::sub(v2, v1), f2 = strict::sub(v0, v2);
    const f3 u0 = {1.0f, 0.0f, 0.0f}, u1 = {0.0f, 1.0f, 0.0f}, u2 = {0.0f, 0.0f, 1.0f};
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        f3 a;
        switch (i) {
            case 0: a = strict::cross(u0, f0); break;
            case 1: a = strict::cross(u0, f1); break;
            case 2: a = strict::cross(u0, f2); break;
            case 3: a = strict::cross(u1, f0); break;
            case 4: a = strict::cross(u1, f1); break;
            case 5: a = ref_axis ? strict::cross(u2, f2) : strict::cross(u1, f2); break;
            case 6: a = strict::cross(u2, f0); break;
            case 7: a = strict::cross(u2, f1); break;
            default: a = strict::cross(u2, f2); break;
        }
        const float p0 = strict::dot(v0, a), p1 = strict::dot(v1, a), p2 = strict::dot(v2, a);
        float r = __fmul_rn(e.x, fabsf(strict::dot(u0, a)));
        r = __fadd_rn(r, __fmul_rn(e.y, fabsf(strict::dot(u1, a))));
        r = __fadd_rn(r, __fmul_rn(e.z, fabsf(strict::dot(u2, a))));
        if (strict::gmax(-strict::gmax(strict::gmax(p0, p1), p2), strict::gmin(strict::gmin(p0, p1), p2)) > r)
            return false;
    }
    return true;
}

// AABBAABBOverlap / AABBAABBOverlapF (CollideBVHStack.glsl:90-102).
__device__ __forceinline__ bool aabb_overlap(f3 amin, f3 amax, f3 bmin, f3 bmax) {
    return (amin.x <= bmax.x && amax.x >= bmin.x) && (amin.y <= bmax.y && amax.y >= bmin.y) &&
           (amin.z <= bmax.z && amax.z >= bmin.z);
}
__device__ __forceinline__ float aabb_overlap_f(f3 amin, f3 amax, f3 bmin, f3 bmax) {
    const bool hit = aabb_overlap(amin, amax, bmin, bmax);
    const f3 d = strict::sub(mid3(bmin, bmax), mid3(amin, amax));
    const float dist = strict::dot(d, d);
    return hit ? dist : -1.0f;
}

__device__ __forceinline__ bool collide_leaf(const SceneView& s, int32_t packed, f3 bmin, f3 bmax, bool ref_axis,
                                             bool leaf_index, int32_t& mesh, int32_t& tri) {
    const int32_t st = packed >> 4, len = packed & 0xF;
    for (int32_t i = 0; i < len; ++i) {
        if (st + i < 0 || st + i >= s.n_tris) return false;
        const int4 t = strict::ldg4i(s.tris + st + i);
        if (box_triangle_overlap(strict::vpos(s, t.x), strict::vpos(s, t.y), strict::vpos(s, t.z), bmin, bmax,
                                 ref_axis)) {
            mesh = t.w;
            tri = leaf_index ? i : st + i;
            return true;
        }
    }
    return false;
}

// One box's walk through one entity's BVH2, one node per step: the stack walk of
// CollideBVHStack.glsl:154-299 and the pointer walk of CollideBVHStackless.glsl:131-223, cut at
// their iteration boundary (the same guards, the 1024-iteration and 63-push caps, the order and the
// tests).
struct CollideWalk {
    int32_t stack[64];
    int32_t sp, iters, cur, start, count;
};

// One iteration of the stack walk: 1 = keep walking, 0 = the walk ended without a collision,
// 2 = collision (mesh, tri set).
__device__ __forceinline__ int collide_stack_step(const SceneView& s, CollideWalk& w, f3 bmin, f3 bmax, bool ref,
                                                  int32_t& mesh, int32_t& tri) {
    if (w.iters >= 1024) return 0;
    if (w.sp >= 64 || w.sp < 0 || w.cur < w.start || w.cur > w.start + w.count || w.cur < 0 || w.cur >= s.n_nodes)
        return 0;
    ++w.iters;
    const float4* nd = s.nodes + 4 * static_cast<int64_t>(w.cur);
    const float4 lmin = strict::ldg4(nd), lmax = strict::ldg4(nd + 1), rmin = strict::ldg4(nd + 2),
                 rmax = strict::ldg4(nd + 3);
    const int32_t lw = __float_as_int(lmin.w), rw = __float_as_int(rmin.w);
    const bool ll = lw != -1, rl = rw != -1;
    const float lt = ll ? -1.0f : aabb_overlap_f(strict::xyz(lmin), strict::xyz(lmax), bmin, bmax);
    const float rt = rl ? -1.0f : aabb_overlap_f(strict::xyz(rmin), strict::xyz(rmax), bmin, bmax);
    if (ll && collide_leaf(s, lw, bmin, bmax, ref, ref, mesh, tri)) return 2;
    if (rl && collide_leaf(s, rw, bmin, bmax, ref, ref, mesh, tri)) return 2;
    if (lt > 0.0f && rt > 0.0f) {
        int32_t a = __float_as_int(lmax.w) + w.start, b = __float_as_int(rmax.w) + w.start;
        if (rt < lt) {
            const int32_t x = a;
            a = b;
            b = x;
        }
        w.cur = a;
        if (w.sp >= 63) return 0;
        w.stack[w.sp++] = b;
        return 1;
    } else if (lt > 0.0f) {
        w.cur = __float_as_int(lmax.w) + w.start;
        return 1;
    } else if (rt > 0.0f) {
        w.cur = __float_as_int(rmax.w) + w.start;
        return 1;
    }
    if (w.sp <= 0) return 0;
    w.cur = w.stack[--w.sp];
    return 1;
}

// One iteration of the pointer walk (w.cur is the node pointer).
__device__ __forceinline__ int collide_stackless_step(const SceneView& s, CollideWalk& w, f3 bmin, f3 bmax,
                                                      bool ref, int32_t& mesh, int32_t& tri) {
    if (!(w.cur >= 0 && w.iters < 1024)) return 0;
    if (w.cur < w.start || w.cur > w.start + w.count || w.cur >= s.n_nodes) return 0;
    ++w.iters;
    const float4* nd = s.nodes + 2 * static_cast<int64_t>(w.cur);
    const float4 nmin = strict::ldg4(nd), nmax = strict::ldg4(nd + 1);
    if (aabb_overlap(strict::xyz(nmin), strict::xyz(nmax), bmin, bmax)) {
        const int32_t packed = __float_as_int(nmin.w);
        if (packed != -1) {
            if (collide_leaf(s, packed, bmin, bmax, ref, false, mesh, tri)) return 2;
            const int32_t nx = __float_as_int(nmax.w);
            if (nx < 0) return 0;
            w.cur = nx + w.start;
            return 1;
        }
        ++w.cur;
        return 1;
    }
    const int32_t nx = __float_as_int(nmax.w);
    if (nx < 0) return 0;
    w.cur = nx + w.start;
    return 1;
}

// CollideScene (CollideBVHStack.glsl:301-323, CollideBVHStackless.glsl:225-247) with a persistent
// box queue: each warp hands its idle lanes boxes from a warp-private pool of 64 consecutive indices
// (one atomicAdd on `queue` per refill), and each lane advances its box's walk by one node per
// iteration, entity after entity until the first collision.  Per box the entities, nodes, caps and
// tests are those of the shader's loops, so the records are those of one thread per box walking to
// its end (measured against that form on C2's 1M boxes: the same records, stack layout 3.17 ->
// 0.65 ms, stackless 1.49 -> 0.50 ms); only the assignment of boxes to lanes changes.
// Occupancy target: 7 blocks per SM for the stack walk (72 registers; its 64-entry stack state
// spilled at 8 blocks: 0.651 -> 0.596 ms on C2's 1M boxes), 8 for the pointer walk (0.498 ms; 7
// blocks: 0.502, 6: 0.552).
template <bool kStackless>
__global__ void __launch_bounds__(128, kStackless ? 8 : 7) k_collide_queue(SceneView s, const float4* __restrict__ boxes, int64_t n,
                                                          int4* __restrict__ out, int flags,
                                                          unsigned long long* queue) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    constexpr unsigned long long kPool = 64;
    const unsigned lane = threadIdx.x & 31u;
    const bool ref = (flags & RQ_FLAG_REF_COMPAT) != 0;
    CollideWalk w;
    f3 wmin{0.0f, 0.0f, 0.0f}, wmax = wmin, bmin = wmin, bmax = wmin;
    int64_t i = -1;
    int32_t e = -1;
    bool live = false, exhausted = false;
    unsigned long long pool_next = 0, pool_end = 0;  // warp-uniform
    // Starts the walk of the box's next entity; false when none is left.
    auto next_entity = [&]() -> bool {
        if (++e >= s.n_ents) return false;
        const rq_entity& E = s.ents[e];
        bmin = strict::xform(E.inverse, wmin, 1.0f);
        bmax = strict::xform(E.inverse, wmax, 1.0f);
        w.start = E.node_offset;
        w.count = E.node_count;
        w.cur = w.start;
        w.sp = 0;
        w.iters = 0;
        return true;
    };
    while (true) {
        while (true) {  // refill idle lanes (warp-uniform loop)
            const unsigned want = __ballot_sync(kFull, !live && !exhausted);
            if (!want) break;
            const unsigned cnt = __popc(want);
            const unsigned rank = __popc(want & persist::lanemask_lt());
            const unsigned long long avail = pool_end - pool_next;
            unsigned long long mine = pool_next + rank;
            if (avail >= cnt) {
                pool_next += cnt;
            } else {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(queue, kPool);
                base = __shfl_sync(kFull, base, 0);
                if (rank >= avail) mine = base + (rank - avail);
                pool_next = base + (cnt - avail);
                pool_end = base + kPool;
            }
            if (!live && !exhausted) {
                if (static_cast<int64_t>(mine) >= n) {
                    exhausted = true;
                } else {
                    i = static_cast<int64_t>(mine);
                    wmin = strict::xyz(__ldg(boxes + 2 * i));
                    wmax = strict::xyz(__ldg(boxes + 2 * i + 1));
                    e = -1;
                    live = next_entity();
                    if (!live) out[i] = make_int4(0, -1, -1, -1);
                }
            }
        }
        if (!__any_sync(kFull, live)) break;
        if (!live) continue;
        int32_t mesh = -1, tri = -1;
        const int g = kStackless ? collide_stackless_step(s, w, bmin, bmax, ref, mesh, tri)
                                 : collide_stack_step(s, w, bmin, bmax, ref, mesh, tri);
        if (g == 1) continue;
        if (g == 2) {
            out[i] = make_int4(1, e, mesh, tri);
            live = false;
        } else if (!next_entity()) {
            out[i] = make_int4(0, -1, -1, -1);
            live = false;
        }
    }
}

}  // namespace
}  // namespace rq

using rq::fail;

extern "C" {

rq_status rq_collide(rq_ctx* ctx, const rq_scene* sc, const rq_box* boxes, int64_t n, rq_collision* out,
                     const rq_opts* opts, void* stream) {
    if (!ctx || !sc || n < 0 || (n > 0 && (!boxes || !out))) return fail(ctx, RQ_EINVAL, "bad arguments");
    rq_opts d{};
    if (!opts) opts = &d;
    const int32_t layout = opts->layout == RQ_LAYOUT_DEFAULT ? sc->layout : opts->layout;
    if (layout != sc->layout || (layout != RQ_LAYOUT_BVH2_STACK && layout != RQ_LAYOUT_BVH2_STACKLESS))
        return fail(ctx, RQ_ENOTSUP, "collision queries walk the scene's BVH2 (stack or stackless)");
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = the default stream
    const bool host = (opts->flags & RQ_FLAG_HOST_BUFFERS) != 0;
    const float4* d_boxes = reinterpret_cast<const float4*>(boxes);
    int4* d_out = reinterpret_cast<int4*>(out);
    if (host) {
        void *a = nullptr, *b = nullptr;
        rq_status s;
        if ((s = rq::scratch(ctx, rq::kSlotCollideBoxes, sizeof(rq_box) * n, &a)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotCollideOut, sizeof(rq_collision) * n, &b)) != RQ_OK)
            return s;
        RQ_CUDA(ctx, cudaMemcpyAsync(a, boxes, sizeof(rq_box) * n, cudaMemcpyHostToDevice, st));
        d_boxes = static_cast<const float4*>(a);
        d_out = static_cast<int4*>(b);
    }
    // the persistent box queue (one resident grid), counter 12 of the context's queue block
    unsigned long long* queue = rq::queue_counter(ctx, 12);
    RQ_CUDA(ctx, cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st));
    if (layout == RQ_LAYOUT_BVH2_STACKLESS) {
        const int64_t g = std::min<int64_t>(rq::persistent_grid(rq::k_collide_queue<true>, 128), (n + 127) / 128);
        rq::k_collide_queue<true><<<static_cast<unsigned>(g), 128, 0, st>>>(sc->view, d_boxes, n, d_out, opts->flags,
                                                                            queue);
    } else {
        const int64_t g = std::min<int64_t>(rq::persistent_grid(rq::k_collide_queue<false>, 128), (n + 127) / 128);
        rq::k_collide_queue<false><<<static_cast<unsigned>(g), 128, 0, st>>>(sc->view, d_boxes, n, d_out,
                                                                             opts->flags, queue);
    }
    RQ_CUDA(ctx, cudaGetLastError());
    if (host) {
        RQ_CUDA(ctx, cudaMemcpyAsync(out, d_out, sizeof(rq_collision) * n, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return RQ_OK;
}

}  // extern "C"
