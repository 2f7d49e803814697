// Ray-query launchers (the plain-loop kernel form), the batched-query kernel and the fast-mode
// triangle records.  The per-variant kernels and launchers are in rq_kernels.cuh; the top-level
// form is instantiated in rq_kernels_tlas.cu.
#include <cstdlib>

#include "rq_kernels.cuh"
#include "rq_objects.h"

namespace rq {

extern template cudaError_t launch_closest_t<true>(const SceneView&, const QueryConfig&, const rq_ray*, int64_t,
                                                   rq_hit*, unsigned long long*, cudaStream_t);
extern template cudaError_t launch_anyhit_t<true>(const SceneView&, const QueryConfig&, const rq_ray*, int64_t,
                                                  uint8_t*, unsigned long long*, cudaStream_t);
template cudaError_t launch_closest_t<false>(const SceneView&, const QueryConfig&, const rq_ray*, int64_t,
                                             rq_hit*, unsigned long long*, cudaStream_t);
template cudaError_t launch_anyhit_t<false>(const SceneView&, const QueryConfig&, const rq_ray*, int64_t,
                                            uint8_t*, unsigned long long*, cudaStream_t);

cudaError_t launch_closest(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                           rq_hit* hits, unsigned long long* queue, cudaStream_t st) {
    const SceneView sv = entity_view(s, q.flags);
    return sv.tlas ? launch_closest_t<true>(sv, q, rays, n, hits, queue, st)
                   : launch_closest_t<false>(sv, q, rays, n, hits, queue, st);
}

cudaError_t launch_anyhit(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                          uint8_t* occluded, unsigned long long* queue, cudaStream_t st) {
    const SceneView sv = entity_view(s, q.flags);
    return sv.tlas ? launch_anyhit_t<true>(sv, q, rays, n, occluded, queue, st)
                   : launch_anyhit_t<false>(sv, q, rays, n, occluded, queue, st);
}

namespace {

// Batched queries: one persistent launch; each warp takes 32 consecutive work items from a global
// counter, and every item finds its query by binary search over the queries' first work index.
template <int kB, int kM, int kFamily, int kDepth = bvh8::kStack>
__global__ void __launch_bounds__(kB, kM) k_batch(const QueryDesc* __restrict__ qd, int nq, int64_t total,
                                                  unsigned long long* queue, unsigned* status_out) {
    __shared__ int64_t base[kMaxBatchQueries + 1];
    for (int k = threadIdx.x; k <= nq; k += blockDim.x) base[k] = k < nq ? qd[k].base : total;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    unsigned status = 0;
    while (true) {
        unsigned long long start = 0;
        if (lane == 0) start = atomicAdd(queue, 32ull);
        start = __shfl_sync(0xFFFFFFFFu, start, 0);
        if (static_cast<int64_t>(start) >= total) break;
        const int64_t idx = static_cast<int64_t>(start) + lane;
        if (idx >= total) continue;
        int lo = 0, hi = nq - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (base[mid] <= idx) lo = mid; else hi = mid - 1;
        }
        const QueryDesc& Q = qd[lo];
        const int64_t i = idx - base[lo];
        float4 r0, r1;
        load_ray(Q.rays, i, r0, r1);
        rq_hit h;
        bool oc = false;
        int32_t visits = 0, tests = 0;
        if (kFamily == kFamilyBvh8) {
            if (Q.kind) bvh8_ray<true, true, kDepth>(Q.s, r0, r1, Q.flags, h, oc, visits, tests, status);
            else bvh8_ray<false, true, kDepth>(Q.s, r0, r1, Q.flags, h, oc, visits, tests, status);
        } else if (kFamily == kFamilyFast) {
            const bool sl = Q.s.layout == RQ_LAYOUT_BVH2_STACKLESS;
            if (Q.kind) {
                if (sl) fast::scene<true, true>(Q.s, r0, r1, Q.flags, h, oc, tests);
                else fast::scene<true, false>(Q.s, r0, r1, Q.flags, h, oc, tests);
            } else {
                if (sl) fast::scene<false, true>(Q.s, r0, r1, Q.flags, h, oc, tests);
                else fast::scene<false, false>(Q.s, r0, r1, Q.flags, h, oc, tests);
            }
        } else {
            const bool sl = Q.s.layout == RQ_LAYOUT_BVH2_STACKLESS;
            if (Q.kind) {
                oc = sl ? strict::scene_any<true>(Q.s, r0, r1, visits, tests)
                        : strict::scene_any<false>(Q.s, r0, r1, visits, tests);
            } else if (Q.tie_lower) {
                if (sl) strict::scene_closest<true, true>(Q.s, r0, r1, Q.flags, h, tests);
                else strict::scene_closest<false, true>(Q.s, r0, r1, Q.flags, h, tests);
            } else {
                if (sl) strict::scene_closest<true, false>(Q.s, r0, r1, Q.flags, h, tests);
                else strict::scene_closest<false, false>(Q.s, r0, r1, Q.flags, h, tests);
            }
        }
        if (Q.kind) Q.occ[i] = oc ? 1 : 0;
        else store_hit(Q.hits, i, h);
    }
    if (status) atomicOr(status_out, status);
}

// Lane-refill form of the batched BVH8 queries when no scene of the batch has a top level: the
// closest-hit queries' rays (work items [0, total_c): the descriptors list those queries first),
// then the any-hit queries' rays, each kind from its own ray queue (queue[0], queue[1]).  Results
// equal k_batch's (bvh8_batch_loop).
template <int kB, int kM, int kDepth = bvh8::kStack>
__global__ void __launch_bounds__(kB, kM) k_batch_b8(const QueryDesc* __restrict__ qd, int nq, int64_t total_c,
                                                     int64_t total, unsigned long long* queue,
                                                     unsigned* status_out) {
    __shared__ int64_t base[kMaxBatchQueries + 1];
    for (int k = threadIdx.x; k <= nq; k += blockDim.x) base[k] = k < nq ? qd[k].base : total;
    __syncthreads();
    unsigned status = 0;
    bvh8_batch_loop<false, kDepth>(qd, base, nq, 0, total_c, queue, status);
    bvh8_batch_loop<true, kDepth>(qd, base, nq, total_c, total, queue + 1, status);
    if (status) atomicOr(status_out, status);
}

__global__ void k_tri_fast(const int4* __restrict__ tris, int64_t n, const float4* __restrict__ verts,
                           float4* __restrict__ out) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int4 tr = tris[t];
    const float4 a = verts[2 * static_cast<int64_t>(tr.x)], b = verts[2 * static_cast<int64_t>(tr.y)];
    const float4 c = verts[2 * static_cast<int64_t>(tr.z)];
    out[3 * t] = make_float4(a.x, a.y, a.z, __int_as_float(tr.w));
    out[3 * t + 1] = make_float4(b.x - a.x, b.y - a.y, b.z - a.z, 0.0f);
    out[3 * t + 2] = make_float4(c.x - a.x, c.y - a.y, c.z - a.z, 0.0f);
}

}  // namespace

static_assert(bvh8::kStackDepths[0] == kBvh8Depths[0] && bvh8::kStackDepths[1] == kBvh8Depths[1] &&
                  bvh8::kStackDepths[2] == kBvh8Depths[2] && bvh8::kStack == kBvh8Depths[0],
              "the host's list of BVH8 stack depths must match the kernels'");
static_assert(bvh8::kStatusStackOverflow == kStatusOverflowBit, "status bit of a stack overflow");

const LaunchVariant kLaunchVariants[kNumLaunchVariants] = {
    {128, 1, 0, 0}, {128, 4, 0, 0}, {128, 6, 0, 0}, {128, 8, 0, 0}, {256, 3, 0, 0}, {64, 12, 0, 0},
    {128, 1, 1, 0}, {128, 7, 1, 0}, {128, 7, 1, bvh8::kStackDepths[1]}, {128, 7, 1, bvh8::kStackDepths[2]}};

int non_persistent_variant(int v) {
    if (v < 0 || v >= kNumLaunchVariants || !kLaunchVariants[v].persistent) return v;
    // same block size, the nearest occupancy target (the higher one on a tie)
    int best = 0, best_d = 1 << 30;
    for (int k = 0; k < kNumLaunchVariants; ++k) {
        if (kLaunchVariants[k].persistent || kLaunchVariants[k].block != kLaunchVariants[v].block) continue;
        const int d = std::abs(kLaunchVariants[k].min_blocks - kLaunchVariants[v].min_blocks);
        if (d < best_d || (d == best_d && kLaunchVariants[k].min_blocks > kLaunchVariants[best].min_blocks)) {
            best = k;
            best_d = d;
        }
    }
    return best;
}

const LaunchVariant kBatchVariants[kNumBatchVariants] = {{128, 1, 1, 0}, {128, 7, 1, 0}, {64, 12, 1, 0},
                                                         {256, 3, 1, 0}};

namespace {
// The BVH8 family's kernel for depth index di (bvh8::kStackDepths).
template <int kB, int kM>
int batch_bvh8_grid(int di) {
    switch (di) {
        case 1: return persistent_grid(k_batch<kB, kM, kFamilyBvh8, bvh8::kStackDepths[1]>, kB);
        case 2: return persistent_grid(k_batch<kB, kM, kFamilyBvh8, bvh8::kStackDepths[2]>, kB);
        default: return persistent_grid(k_batch<kB, kM, kFamilyBvh8>, kB);
    }
}
// The lane-refill kernel's grid for depth index di.
template <int kB, int kM>
int batch_b8_grid(int di) {
    switch (di) {
        case 1: return persistent_grid(k_batch_b8<kB, kM, bvh8::kStackDepths[1]>, kB);
        case 2: return persistent_grid(k_batch_b8<kB, kM, bvh8::kStackDepths[2]>, kB);
        default: return persistent_grid(k_batch_b8<kB, kM>, kB);
    }
}

template <int kB, int kM>
cudaError_t batch_variant(const QueryDesc* d, int nq, int64_t total, int family,
                          unsigned long long* queue, unsigned* status, cudaStream_t st, int di, int64_t total_c) {
    const bool refill = family == kFamilyBvh8 && total_c >= 0;
    int g = 0;
    switch (family) {
        case kFamilyBvh8: g = refill ? batch_b8_grid<kB, kM>(di) : batch_bvh8_grid<kB, kM>(di); break;
        case kFamilyFast: g = persistent_grid(k_batch<kB, kM, kFamilyFast>, kB); break;
        default: g = persistent_grid(k_batch<kB, kM, kFamilyStrict>, kB); break;
    }
    const int64_t need = (total + 31) / 32 * 32 / kB + 1;
    if (need < g) g = static_cast<int>(need);
    if (refill) {
        if (di == 1)
            k_batch_b8<kB, kM, bvh8::kStackDepths[1]><<<g, kB, 0, st>>>(d, nq, total_c, total, queue, status);
        else if (di == 2)
            k_batch_b8<kB, kM, bvh8::kStackDepths[2]><<<g, kB, 0, st>>>(d, nq, total_c, total, queue, status);
        else
            k_batch_b8<kB, kM><<<g, kB, 0, st>>>(d, nq, total_c, total, queue, status);
    } else if (family == kFamilyBvh8) {
        if (di == 1)
            k_batch<kB, kM, kFamilyBvh8, bvh8::kStackDepths[1]><<<g, kB, 0, st>>>(d, nq, total, queue, status);
        else if (di == 2)
            k_batch<kB, kM, kFamilyBvh8, bvh8::kStackDepths[2]><<<g, kB, 0, st>>>(d, nq, total, queue, status);
        else
            k_batch<kB, kM, kFamilyBvh8><<<g, kB, 0, st>>>(d, nq, total, queue, status);
    } else if (family == kFamilyFast) {
        k_batch<kB, kM, kFamilyFast><<<g, kB, 0, st>>>(d, nq, total, queue, status);
    } else {
        k_batch<kB, kM, kFamilyStrict><<<g, kB, 0, st>>>(d, nq, total, queue, status);
    }
    return cudaGetLastError();
}

template <int kB, int kM>
void batch_grids() {
    for (int di = 0; di < kNumBatchDepths; ++di) {
        batch_bvh8_grid<kB, kM>(di);
        batch_b8_grid<kB, kM>(di);
    }
    persistent_grid(k_batch<kB, kM, kFamilyStrict>, kB);
    persistent_grid(k_batch<kB, kM, kFamilyFast>, kB);
}
}  // namespace

cudaError_t launch_batch(const QueryDesc* d_desc, int nq, int64_t total, int family, int variant,
                         unsigned long long* queue, unsigned* status, cudaStream_t st, int depth_index,
                         int64_t total_c) {
    if (total <= 0 || nq <= 0) return cudaSuccess;
    const int di = (depth_index >= 0 && depth_index < kNumBatchDepths) ? depth_index : 0;
    if (!st && !queue) {  // grid-size query only (fills the occupancy cache outside stream capture)
        switch (variant) {
            case 1: batch_grids<128, 7>(); break;
            case 2: batch_grids<64, 12>(); break;
            case 3: batch_grids<256, 3>(); break;
            default: batch_grids<128, 1>(); break;
        }
        return cudaGetLastError();
    }
    switch (variant) {
        case 1: return batch_variant<128, 7>(d_desc, nq, total, family, queue, status, st, di, total_c);
        case 2: return batch_variant<64, 12>(d_desc, nq, total, family, queue, status, st, di, total_c);
        case 3: return batch_variant<256, 3>(d_desc, nq, total, family, queue, status, st, di, total_c);
        default: return batch_variant<128, 1>(d_desc, nq, total, family, queue, status, st, di, total_c);
    }
}

cudaError_t launch_tri_fast(const int4* tris, int64_t n_tris, const float4* verts, float4* out,
                            cudaStream_t st) {
    if (n_tris <= 0) return cudaSuccess;
    k_tri_fast<<<grid_for(n_tris, 256), 256, 0, st>>>(tris, n_tris, verts, out);
    return cudaGetLastError();
}

}  // namespace rq
