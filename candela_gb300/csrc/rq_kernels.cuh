// Ray-query kernels and their per-variant launchers, compiled once per top-level form: kTlas =
// false for scenes without a top level over their entities (the plain entity loop only), true for
// scenes with one (rq_kernels.cu and rq_kernels_tlas.cu instantiate one form each).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include <mutex>
#include <unordered_map>

#include "rq_internal.h"
#include "rq_bvh8.cuh"
#include "rq_bvh8_walk.cuh"
#include "rq_fast.cuh"
#include "rq_persistent.cuh"
#include "rq_strict.cuh"

namespace rq {
namespace {

// Warp-aggregated work counters: counters[0] += node visits, counters[1] += triangle tests.
__device__ __forceinline__ void count_work(unsigned long long* counters, int32_t nodes,
                                           int32_t tests) {
    const unsigned a = __reduce_add_sync(0xFFFFFFFFu, static_cast<unsigned>(nodes));
    const unsigned b = __reduce_add_sync(0xFFFFFFFFu, static_cast<unsigned>(tests));
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counters + 0, static_cast<unsigned long long>(a));
        atomicAdd(counters + 1, static_cast<unsigned long long>(b));
    }
}

// One thread per ray, strict arithmetic and reference traversal order.
template <bool kStackless, bool kTieLower, int kB, int kM, bool kTlas>
__global__ void __launch_bounds__(kB, kM) k_closest_strict(SceneView s, const rq_ray* __restrict__ rays,
                                                        int64_t n, rq_hit* __restrict__ hits,
                                                        int flags, unsigned long long* counters) {
    if (s.ray_count && static_cast<int64_t>(*s.ray_count) < n) n = static_cast<int64_t>(*s.ray_count);
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    rq_hit h;
    int32_t tests = 0;
    h.iters = 0;
    if (i < n) {
        float4 r0, r1;
        load_ray(rays, i, r0, r1);
        strict::scene_closest<kStackless, kTieLower, kTlas>(s, r0, r1, flags, h, tests);
        store_hit(hits, i, h);
    }
    if (counters) count_work(counters, h.iters, tests);
}

template <bool kStackless, int kB, int kM, bool kTlas>
__global__ void __launch_bounds__(kB, kM) k_anyhit_strict(SceneView s, const rq_ray* __restrict__ rays,
                                                       int64_t n, uint8_t* __restrict__ occ,
                                                       unsigned long long* counters) {
    if (s.ray_count && static_cast<int64_t>(*s.ray_count) < n) n = static_cast<int64_t>(*s.ray_count);
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int32_t iters = 0, tests = 0;
    if (i < n) {
        float4 r0, r1;
        load_ray(rays, i, r0, r1);
        occ[i] = strict::scene_any<kStackless, kTlas>(s, r0, r1, iters, tests) ? 1 : 0;
    }
    if (counters) count_work(counters, iters, tests);
}

// Persistent strict traversal (closest or any hit): see rq_persistent.cuh.
template <bool kAny, bool kStackless, bool kTieLower, int kM, bool kTlas>
__global__ void __launch_bounds__(128, kM) k_persistent_strict(SceneView s, const rq_ray* __restrict__ rays,
                                                           int64_t n, rq_hit* __restrict__ hits,
                                                           uint8_t* __restrict__ occ, int flags,
                                                           unsigned long long* queue,
                                                           unsigned long long* counters) {
    if (s.ray_count && static_cast<int64_t>(*s.ray_count) < n) n = static_cast<int64_t>(*s.ray_count);
    persist::StrictRay<kAny, kStackless, kTieLower, kTlas> R{};
    int32_t stack[kStackless ? 1 : 64];
    int64_t id = -1;
    bool need = true;
    int32_t tests = 0, nodes = 0;
    auto store = [&]() {
        nodes += R.iters_total;
        if (kAny) {
            occ[id] = R.occluded ? 1 : 0;
        } else {
            rq_hit h;
            R.finish(s, flags, h);
            store_hit(hits, id, h);
        }
    };
    if constexpr (kTlas) {
        // Scenes with a top level: a ray looking for its next entity advances the top-level cursor
        // by at most 4 nodes per iteration (StrictRay::seek), interleaved with the node steps of
        // the other lanes; the entities, their order and every count are those of the loop below.
        bool seeking = false;
        while (true) {
            const int64_t nid = persist::fetch(queue, need);
            if (need) {
                id = nid;
                if (id >= n) break;
                float4 r0, r1;
                load_ray(rays, id, r0, r1);
                if (!R.init_ray(s, r0, r1)) {
                    store();
                    continue;
                }
                need = false;
                seeking = true;
            }
            if (seeking) {
                const int g = R.seek(s, flags, 4);
                if (g > 0) {
                    seeking = false;
                } else if (g < 0) {
                    store();
                    need = true;
                }
                continue;
            }
            if (R.step(s, stack, tests)) {
                if (R.accept_entity()) {
                    seeking = true;
                } else {
                    store();
                    need = true;
                }
            }
        }
    } else {
        while (true) {
            const int64_t nid = persist::fetch(queue, need);
            if (need) {
                id = nid;
                if (id >= n) break;
                float4 r0, r1;
                load_ray(rays, id, r0, r1);
                if (!R.init(s, r0, r1, flags)) {
                    store();
                    continue;
                }
                need = false;
            }
            if (R.step(s, stack, tests) && !R.end_entity(s, flags)) {
                store();
                need = true;
            }
        }
    }
    if (counters) count_work(counters, nodes, tests);
}

// BVH8 traversal, one thread per ray.
template <bool kAny, int kB, int kM, bool kTlas>
__global__ void __launch_bounds__(kB, kM) k_bvh8(SceneView s, const rq_ray* __restrict__ rays, int64_t n,
                                                 rq_hit* __restrict__ hits, uint8_t* __restrict__ occ,
                                                 int flags, unsigned* status_out,
                                                 unsigned long long* counters) {
    if (s.ray_count && static_cast<int64_t>(*s.ray_count) < n) n = static_cast<int64_t>(*s.ray_count);
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int32_t visits = 0, tests = 0;
    unsigned status = 0;
    if (i < n) {
        float4 r0, r1;
        load_ray(rays, i, r0, r1);
        if (s.ray_copy) {
            float4* c = reinterpret_cast<float4*>(s.ray_copy) + 2 * i;
            c[0] = r0;
            c[1] = r1;
        }
        rq_hit hh;
        bool occluded;
        bvh8_ray<kAny, kTlas>(s, r0, r1, flags, hh, occluded, visits, tests, status);
        if (kAny)
            occ[i] = occluded ? 1 : 0;
        else
            store_hit(hits, i, hh);
    }
    if (status) atomicOr(status_out, status);
    if (counters) count_work(counters, visits, tests);
}

// Persistent BVH8 traversal (bvh8_persistent_loop in rq_bvh8_walk.cuh), results as hit records
// or occlusion bytes.
template <bool kAny, int kB, int kM, bool kTlas, int kDepth = bvh8::kStack>
__global__ void __launch_bounds__(kB, kM) k_bvh8_persistent(SceneView s, const rq_ray* __restrict__ rays,
                                                            int64_t n, rq_hit* __restrict__ hits,
                                                            uint8_t* __restrict__ occ, int flags,
                                                            unsigned* status_out, unsigned long long* queue,
                                                            unsigned long long* counters) {
    if (s.ray_count && static_cast<int64_t>(*s.ray_count) < n) n = static_cast<int64_t>(*s.ray_count);
    int32_t tests = 0, nodes_total = 0;
    unsigned status = 0;
    const QuerySink sink{s, flags, hits, occ};
    bvh8_persistent_loop<kAny, QuerySink, kTlas, kDepth>(s, rays, n, flags, queue, sink, tests, nodes_total, status);
    if (status) atomicOr(status_out, status);
    if (counters) count_work(counters, nodes_total, tests);
}

// Fast-mode BVH2 traversal, one thread per ray.
template <bool kAny, bool kStackless, int kB, int kM, bool kTlas>
__global__ void __launch_bounds__(kB, kM) k_fast(SceneView s, const rq_ray* __restrict__ rays, int64_t n,
                                                 rq_hit* __restrict__ hits, uint8_t* __restrict__ occ,
                                                 int flags, unsigned long long* counters) {
    if (s.ray_count && static_cast<int64_t>(*s.ray_count) < n) n = static_cast<int64_t>(*s.ray_count);
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    rq_hit h;
    h.iters = 0;
    int32_t tests = 0;
    if (i < n) {
        float4 r0, r1;
        load_ray(rays, i, r0, r1);
        bool oc;
        fast::scene<kAny, kStackless, kTlas>(s, r0, r1, flags, h, oc, tests);
        if (kAny)
            occ[i] = oc ? 1 : 0;
        else
            store_hit(hits, i, h);
    }
    if (counters) count_work(counters, h.iters, tests);
}

inline unsigned grid_for(int64_t n, int block) {
    return static_cast<unsigned>((n + block - 1) / block);
}

template <bool kAny, bool kStackless, bool kTieLower, int kM, bool kTlas>
cudaError_t launch_persistent(const SceneView& s, const QueryConfig& q, const rq_ray* rays,
                              int64_t n, rq_hit* hits, uint8_t* occ, unsigned long long* queue,
                              cudaStream_t st) {
    const int block = 128;
    auto k = k_persistent_strict<kAny, kStackless, kTieLower, kM, kTlas>;
    const int64_t g = std::min<int64_t>(persistent_grid(k, block), (n + block - 1) / block);
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k<<<static_cast<unsigned>(g), block, 0, st>>>(s, rays, n, hits, occ, q.flags, queue, q.counters);
    return cudaGetLastError();
}

template <bool kAny, int kM, bool kTlas, int kDepth>
cudaError_t launch_bvh8_persistent(const SceneView& s, const QueryConfig& q, const rq_ray* rays,
                                   int64_t n, rq_hit* hits, uint8_t* occ, unsigned long long* queue,
                                   cudaStream_t st) {
    const int block = 128;
    auto k = k_bvh8_persistent<kAny, 128, kM, kTlas, kDepth>;
    const int64_t g = std::min<int64_t>(persistent_grid(k, block), (n + block - 1) / block);
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k<<<static_cast<unsigned>(g), block, 0, st>>>(s, rays, n, hits, occ, q.flags, q.status, queue, q.counters);
    return cudaGetLastError();
}

// Persistent launch of variant kM (min blocks per SM) for the query's layout; kDepth is the BVH8
// group-stack depth (the BVH2 walks keep the reference's 64-entry stack).
template <bool kAny, int kM, bool kTlas, int kDepth = bvh8::kStack>
cudaError_t persistent_variant(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                               rq_hit* hits, uint8_t* occ, unsigned long long* queue, cudaStream_t st) {
    if (q.layout == RQ_LAYOUT_BVH8Q)
        return launch_bvh8_persistent<kAny, kM, kTlas, kDepth>(s, q, rays, n, hits, occ, queue, st);
    const bool sl = q.layout == RQ_LAYOUT_BVH2_STACKLESS;
    if (kAny)
        return sl ? launch_persistent<true, true, false, kM, kTlas>(s, q, rays, n, nullptr, occ, queue, st)
                  : launch_persistent<true, false, false, kM, kTlas>(s, q, rays, n, nullptr, occ, queue, st);
    if (sl)
        return q.tie_lower ? launch_persistent<false, true, true, kM, kTlas>(s, q, rays, n, hits, nullptr, queue, st)
                           : launch_persistent<false, true, false, kM, kTlas>(s, q, rays, n, hits, nullptr, queue, st);
    return q.tie_lower ? launch_persistent<false, false, true, kM, kTlas>(s, q, rays, n, hits, nullptr, queue, st)
                       : launch_persistent<false, false, false, kM, kTlas>(s, q, rays, n, hits, nullptr, queue, st);
}

}  // namespace

namespace {

template <int kB, int kM, bool kTlas>
cudaError_t closest_variant(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                            rq_hit* hits, cudaStream_t st) {
    unsigned long long* cnt = q.counters;
    const unsigned g = grid_for(n, kB);
    if (q.layout == RQ_LAYOUT_BVH8Q)
        k_bvh8<false, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, hits, nullptr, q.flags, q.status, cnt);
    else if (q.mode == RQ_MODE_FAST)
        q.layout == RQ_LAYOUT_BVH2_STACKLESS
            ? k_fast<false, true, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, hits, nullptr, q.flags, cnt)
            : k_fast<false, false, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, hits, nullptr, q.flags, cnt);
    else if (q.layout == RQ_LAYOUT_BVH2_STACKLESS)
        q.tie_lower ? k_closest_strict<true, true, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, hits, q.flags, cnt)
                    : k_closest_strict<true, false, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, hits, q.flags, cnt);
    else
        q.tie_lower ? k_closest_strict<false, true, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, hits, q.flags, cnt)
                    : k_closest_strict<false, false, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, hits, q.flags, cnt);
    return cudaGetLastError();
}

template <int kB, int kM, bool kTlas>
cudaError_t anyhit_variant(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                           uint8_t* occ, cudaStream_t st) {
    unsigned long long* cnt = q.counters;
    const unsigned g = grid_for(n, kB);
    if (q.layout == RQ_LAYOUT_BVH8Q)
        k_bvh8<true, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, nullptr, occ, q.flags, q.status, cnt);
    else if (q.mode == RQ_MODE_FAST)
        q.layout == RQ_LAYOUT_BVH2_STACKLESS
            ? k_fast<true, true, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, nullptr, occ, q.flags, cnt)
            : k_fast<true, false, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, nullptr, occ, q.flags, cnt);
    else if (q.layout == RQ_LAYOUT_BVH2_STACKLESS)
        k_anyhit_strict<true, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, occ, cnt);
    else
        k_anyhit_strict<false, kB, kM, kTlas><<<g, kB, 0, st>>>(s, rays, n, occ, cnt);
    return cudaGetLastError();
}

}  // namespace

template <bool kTlas>
cudaError_t launch_closest_t(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                           rq_hit* hits, unsigned long long* queue, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int v = q.variant_closest < 0 ? 0 : q.variant_closest;
    if (kLaunchVariants[v].persistent && (!queue || q.mode == RQ_MODE_FAST)) v = non_persistent_variant(v);
    switch (v) {
        case 1: return closest_variant<128, 4, kTlas>(s, q, rays, n, hits, st);
        case 2: return closest_variant<128, 6, kTlas>(s, q, rays, n, hits, st);
        case 3: return closest_variant<128, 8, kTlas>(s, q, rays, n, hits, st);
        case 4: return closest_variant<256, 3, kTlas>(s, q, rays, n, hits, st);
        case 5: return closest_variant<64, 12, kTlas>(s, q, rays, n, hits, st);
        case 6: return persistent_variant<false, 1, kTlas>(s, q, rays, n, hits, nullptr, queue, st);
        case 7: return persistent_variant<false, 7, kTlas>(s, q, rays, n, hits, nullptr, queue, st);
        case 8: return persistent_variant<false, 7, kTlas, bvh8::kStackDepths[1]>(s, q, rays, n, hits, nullptr, queue, st);
        case 9: return persistent_variant<false, 7, kTlas, bvh8::kStackDepths[2]>(s, q, rays, n, hits, nullptr, queue, st);
        default: return closest_variant<128, 1, kTlas>(s, q, rays, n, hits, st);
    }
}

template <bool kTlas>
cudaError_t launch_anyhit_t(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                          uint8_t* occluded, unsigned long long* queue, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int v = q.variant_any < 0 ? 0 : q.variant_any;
    if (kLaunchVariants[v].persistent && (!queue || q.mode == RQ_MODE_FAST)) v = non_persistent_variant(v);
    switch (v) {
        case 1: return anyhit_variant<128, 4, kTlas>(s, q, rays, n, occluded, st);
        case 2: return anyhit_variant<128, 6, kTlas>(s, q, rays, n, occluded, st);
        case 3: return anyhit_variant<128, 8, kTlas>(s, q, rays, n, occluded, st);
        case 4: return anyhit_variant<256, 3, kTlas>(s, q, rays, n, occluded, st);
        case 5: return anyhit_variant<64, 12, kTlas>(s, q, rays, n, occluded, st);
        case 6: return persistent_variant<true, 1, kTlas>(s, q, rays, n, nullptr, occluded, queue, st);
        case 7: return persistent_variant<true, 7, kTlas>(s, q, rays, n, nullptr, occluded, queue, st);
        case 8: return persistent_variant<true, 7, kTlas, bvh8::kStackDepths[1]>(s, q, rays, n, nullptr, occluded, queue, st);
        case 9: return persistent_variant<true, 7, kTlas, bvh8::kStackDepths[2]>(s, q, rays, n, nullptr, occluded, queue, st);
        default: return anyhit_variant<128, 1, kTlas>(s, q, rays, n, occluded, st);
    }
}

}  // namespace rq
