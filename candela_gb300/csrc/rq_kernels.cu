// Ray-query kernels and their launchers.
#include <cuda_runtime.h>

#include "rq_internal.h"
#include "rq_strict.cuh"

namespace rq {
namespace {

__device__ __forceinline__ void load_ray(const rq_ray* rays, int64_t i, float4& r0, float4& r1) {
    const float4* p = reinterpret_cast<const float4*>(rays) + 2 * i;
    r0 = __ldg(p);
    r1 = __ldg(p + 1);
}

__device__ __forceinline__ void store_hit(rq_hit* hits, int64_t i, const rq_hit& h) {
    float4* p = reinterpret_cast<float4*>(hits) + 2 * i;
    p[0] = make_float4(h.t, h.u, h.v, h.w);
    p[1] = make_float4(__int_as_float(h.tri), __int_as_float(h.mesh), __int_as_float(h.entity),
                       __int_as_float(h.iters));
}

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
template <bool kStackless, bool kTieLower>
__global__ void __launch_bounds__(128) k_closest_strict(SceneView s, const rq_ray* __restrict__ rays,
                                                        int64_t n, rq_hit* __restrict__ hits,
                                                        int flags, unsigned long long* counters) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    rq_hit h;
    int32_t tests = 0;
    h.iters = 0;
    if (i < n) {
        float4 r0, r1;
        load_ray(rays, i, r0, r1);
        strict::scene_closest<kStackless, kTieLower>(s, r0, r1, flags, h, tests);
        store_hit(hits, i, h);
    }
    if (counters) count_work(counters, h.iters, tests);
}

template <bool kStackless>
__global__ void __launch_bounds__(128) k_anyhit_strict(SceneView s, const rq_ray* __restrict__ rays,
                                                       int64_t n, uint8_t* __restrict__ occ,
                                                       unsigned long long* counters) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int32_t iters = 0, tests = 0;
    if (i < n) {
        float4 r0, r1;
        load_ray(rays, i, r0, r1);
        occ[i] = strict::scene_any<kStackless>(s, r0, r1, iters, tests) ? 1 : 0;
    }
    if (counters) count_work(counters, iters, tests);
}

inline unsigned grid_for(int64_t n, int block) {
    return static_cast<unsigned>((n + block - 1) / block);
}

}  // namespace

cudaError_t launch_closest(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                           rq_hit* hits, int* /*work_counter*/, cudaStream_t st) {
    unsigned long long* cnt = q.counters;
    if (n <= 0) return cudaSuccess;
    const int block = 128;
    const bool stackless = q.layout == RQ_LAYOUT_BVH2_STACKLESS;
    if (stackless) {
        if (q.tie_lower)
            k_closest_strict<true, true><<<grid_for(n, block), block, 0, st>>>(s, rays, n, hits, q.flags, cnt);
        else
            k_closest_strict<true, false><<<grid_for(n, block), block, 0, st>>>(s, rays, n, hits, q.flags, cnt);
    } else {
        if (q.tie_lower)
            k_closest_strict<false, true><<<grid_for(n, block), block, 0, st>>>(s, rays, n, hits, q.flags, cnt);
        else
            k_closest_strict<false, false><<<grid_for(n, block), block, 0, st>>>(s, rays, n, hits, q.flags, cnt);
    }
    return cudaGetLastError();
}

cudaError_t launch_anyhit(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                          uint8_t* occluded, int* /*work_counter*/, cudaStream_t st) {
    unsigned long long* cnt = q.counters;
    if (n <= 0) return cudaSuccess;
    const int block = 128;
    if (q.layout == RQ_LAYOUT_BVH2_STACKLESS)
        k_anyhit_strict<true><<<grid_for(n, block), block, 0, st>>>(s, rays, n, occluded, cnt);
    else
        k_anyhit_strict<false><<<grid_for(n, block), block, 0, st>>>(s, rays, n, occluded, cnt);
    return cudaGetLastError();
}

}  // namespace rq
