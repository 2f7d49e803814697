// GPU SAH BVH builder.  Produces the same buffers as the host builder (bvh_build.cpp), which are
// the reference constructor's buffers byte for byte (Source/Core/BVH/BVHConstructor.cpp): the
// split rule, partition, leaf rule, leaf numbering, child swaps and flatteners listed there.
//
// Schedule:
//   * per-triangle bounds and centroids, one thread per triangle (:406-424);
//   * nodes with more than kSmall triangles are split level by level over all triangles:
//     binning into per-node bins (shared-memory partial bins merged with atomics), the split
//     search of SearchSAHPlaneBinned (:276-363) with the host's rounding order, the Lomuto
//     partition (:532-550) in parallel (below), child bounds by position-keyed reductions;
//   * a node of at most kSmall triangles is finished by one warp, which builds its whole subtree
//     in shared memory (in place on its own triangle range);
//   * flattening on the GPU: leaf order, stackless DFS with escape links and swaps, stack BFS.
//
// Order-dependent details, reproduced exactly:
//   * glm::min(acc, x) keeps the later of equal values (node-root bounds) and glm::min(x, acc)
//     the earlier (child bounds, :573-597); min/max of floats depend on order only through +0/-0,
//     so bounds are reduced with 64-bit keys (value with -0 folded onto +0, then the position)
//     and the bound takes the bits of the element at the winning position;
//   * bin boxes only enter the SAH areas, whose values do not depend on the sign of a zero, so
//     bins are reduced with plain 32-bit atomics;
//   * Lomuto partition: with j(q) the number of elements below `border` before position q and
//     k their total, element q goes to start + j(q) when it is below the border; the tail
//     [start + k, end) holds val(q), where val(q) = orig[q] for an element not below the border
//     and val(q) = val(start + j(q)) for one below it (the element the swap brings to q), so
//     val follows a pointer chain that ends at an element not below the border and is resolved
//     by pointer jumping;
//   * leaves are numbered in the reference's LIFO walk, which visits upper (right) halves first,
//     i.e. in decreasing order of their triangle range: leaf X gets sorted offset
//     n - start(X) - len(X);
//   * stackless child swaps consume one mt19937 draw per internal node in that same walk order
//     (:599-609); the draws come from the host generator, indexed by each internal node's
//     position in the walk.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "rq_objects.h"

namespace rq {
namespace {

constexpr int kBins = 64;
constexpr float kArbMax = 10000000.0f;   // ARBITRARY_MAX (BVHConstructor.h:21)
constexpr float kArbMin = -10000000.0f;  // ARBITRARY_MIN (BVHConstructor.h:22)
constexpr float kInfCost = 1e29f;        // INF_COST (BVHConstructor.cpp:56)
constexpr int kSmall = 256;              // subtrees of at most this many triangles: one thread
constexpr int kChunk = 2048;             // triangles per block of a large node's level pass
constexpr int kMaxLevels = 4096;         // level passes before the build gives up (RQ_EBUDGET)
constexpr int kScanBlock = 1024;

__device__ __forceinline__ float gmin(float x, float y) { return x < y ? x : y; }  // glm::min
__device__ __forceinline__ float gmax(float x, float y) { return x > y ? x : y; }  // glm::max

// Order-preserving unsigned key of a float with -0 folded onto +0 (inputs hold no NaN).
__device__ __forceinline__ uint32_t okey(float f) {
    uint32_t u = __float_as_uint(f);
    if (u == 0x80000000u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float okey_value(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Per-triangle data, structure of arrays: tb[k*n + t] = min_k, tb[(3+k)*n + t] = max_k,
// tb[(6+k)*n + t] = centroid_k.
struct Tri {
    const float* tb;
    int64_t n;
    __device__ __forceinline__ float mn(int k, int32_t t) const { return tb[k * n + t]; }
    __device__ __forceinline__ float mx(int k, int32_t t) const { return tb[(3 + k) * n + t]; }
    __device__ __forceinline__ float cen(int k, int32_t t) const { return tb[(6 + k) * n + t]; }
};

// Node arrays (capacity cap): box[k*cap + id] (k < 3 min, 3..5 max).
struct Nodes {
    int32_t* start;
    int32_t* len;
    int32_t* left;  // -1: leaf
    int32_t* right;
    int32_t* parent;
    float* box;
    int64_t cap;
};

__global__ void k_tri_bounds(const float* __restrict__ verts, const uint32_t* __restrict__ idx, int64_t n,
                             float* __restrict__ tb, int32_t* __restrict__ refs) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float mn[3] = {kArbMax, kArbMax, kArbMax}, mx[3] = {kArbMin, kArbMin, kArbMin};
    for (int v = 0; v < 3; ++v) {
        const float* p = verts + static_cast<int64_t>(idx[t * 3 + v]) * 8;
        for (int k = 0; k < 3; ++k) {
            mn[k] = gmin(mn[k], p[k]);
            mx[k] = gmax(mx[k], p[k]);
        }
    }
    for (int k = 0; k < 3; ++k) {
        tb[k * n + t] = mn[k];
        tb[(3 + k) * n + t] = mx[k];
        tb[(6 + k) * n + t] = __fdiv_rn(__fadd_rn(mn[k], mx[k]), 2.0f);
    }
    refs[t] = static_cast<int32_t>(t);
}

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xFFFFFFFFu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_max64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xFFFFFFFFu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Root bounds (MinInitial / MaxInitial, :420-421): glm::min(acc, tri) over triangles in input
// order keeps the last of equal values.  keys[k] (min, k < 3) and keys[3+k] (max).
__global__ void k_root_keys(Tri T, unsigned long long* keys) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool ok = t < T.n;
    for (int k = 0; k < 3; ++k) {
        unsigned long long a = ~0ull, b = 0ull;
        if (ok) {
            a = (static_cast<unsigned long long>(okey(T.mn(k, t))) << 32) | (~static_cast<uint32_t>(t));
            b = (static_cast<unsigned long long>(okey(T.mx(k, t))) << 32) | static_cast<uint32_t>(t);
        }
        a = warp_min64(a);
        b = warp_max64(b);
        if ((threadIdx.x & 31) == 0) {
            if (a != ~0ull) atomicMin(keys + k, a);
            if (b != 0ull) atomicMax(keys + 3 + k, b);
        }
    }
}

__global__ void k_root_decode(Tri T, const unsigned long long* keys, Nodes N, int32_t root, int32_t n) {
    if (threadIdx.x != 0) return;
    for (int k = 0; k < 3; ++k) {
        const uint32_t tmn = ~static_cast<uint32_t>(keys[k]);
        const uint32_t tmx = static_cast<uint32_t>(keys[3 + k]);
        const float vmn = T.mn(k, static_cast<int32_t>(tmn)), vmx = T.mx(k, static_cast<int32_t>(tmx));
        // glm::min(acc = ARBITRARY_MAX, x): x unless the sentinel is strictly smaller
        N.box[k * N.cap + root] = vmn <= kArbMax ? vmn : kArbMax;
        N.box[(3 + k) * N.cap + root] = vmx >= kArbMin ? vmx : kArbMin;
    }
    N.start[root] = 0;
    N.len[root] = n;
    N.left[root] = N.right[root] = N.parent[root] = -1;
}

// ---- level pass over large nodes --------------------------------------------------------------

__global__ void k_gather_info(Nodes N, const int32_t* __restrict__ ids, int32_t count, int32_t* __restrict__ out) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    out[2 * i] = N.start[ids[i]];
    out[2 * i + 1] = N.len[ids[i]];
}

struct Chunk {
    int32_t slot;   // index in the level's node list
    int32_t begin;  // element range [begin, end)
    int32_t end;
};

struct Level {
    const int32_t* node;     // node id per slot
    int32_t n_slots;
    unsigned* bin_cnt;       // [slot][axis][bin]
    unsigned* bin_kmin;      // [slot][axis][bin][k] okey of the bin's min corner
    unsigned* bin_kmax;
    int32_t* axis;           // per slot
    float* border;
    int32_t* k_below;        // per slot: elements below the border
    int32_t* mid;            // per slot: split position
    int32_t* fallback;       // per slot: midpoint split
};

__device__ __forceinline__ void node_frame(const Nodes& N, int32_t id, float* mn, float* ext, float* scale,
                                           bool* active) {
    for (int a = 0; a < 3; ++a) {
        mn[a] = N.box[a * N.cap + id];
        const float mx = N.box[(3 + a) * N.cap + id];
        active[a] = !(mn[a] == mx);
        ext[a] = __fsub_rn(mx, mn[a]);
        scale[a] = __fdiv_rn(static_cast<float>(kBins), ext[a]);
    }
}

__device__ __forceinline__ int bin_of(float c, float mn, float scale) {
    const int b = __float2int_rz(__fmul_rn(__fsub_rn(c, mn), scale));
    // glm::min(BIN_COUNT - 1, idx); idx >= 0 for finite inputs (a centroid never lies below its
    // node's minimum), clamped anyway so that no input can index outside the bins
    return kBins - 1 < b ? kBins - 1 : (b < 0 ? 0 : b);
}

__global__ void __launch_bounds__(256) k_bin_large(Tri T, Nodes N, Level L, const Chunk* __restrict__ chunks,
                                                   const int32_t* __restrict__ refs) {
    __shared__ unsigned s_cnt[3 * kBins];
    __shared__ unsigned s_kmin[3 * kBins * 3];
    __shared__ unsigned s_kmax[3 * kBins * 3];
    const Chunk c = chunks[blockIdx.x];
    const int32_t id = L.node[c.slot];
    for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) s_cnt[i] = 0;
    for (int i = threadIdx.x; i < 3 * kBins * 3; i += blockDim.x) {
        s_kmin[i] = 0xFFFFFFFFu;
        s_kmax[i] = 0u;
    }
    float mn[3], ext[3], scale[3];
    bool active[3];
    node_frame(N, id, mn, ext, scale, active);
    __syncthreads();
    for (int32_t q = c.begin + threadIdx.x; q < c.end; q += blockDim.x) {
        const int32_t r = refs[q];
        uint32_t km[3], kx[3];
        for (int k = 0; k < 3; ++k) {
            km[k] = okey(T.mn(k, r));
            kx[k] = okey(T.mx(k, r));
        }
        for (int a = 0; a < 3; ++a) {
            if (!active[a]) continue;
            const int b = a * kBins + bin_of(T.cen(a, r), mn[a], scale[a]);
            atomicAdd(&s_cnt[b], 1u);
            for (int k = 0; k < 3; ++k) {
                atomicMin(&s_kmin[b * 3 + k], km[k]);
                atomicMax(&s_kmax[b * 3 + k], kx[k]);
            }
        }
    }
    __syncthreads();
    const int64_t base = static_cast<int64_t>(c.slot) * 3 * kBins;
    for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
        if (!s_cnt[i]) continue;
        atomicAdd(L.bin_cnt + base + i, s_cnt[i]);
        for (int k = 0; k < 3; ++k) {
            atomicMin(L.bin_kmin + (base + i) * 3 + k, s_kmin[i * 3 + k]);
            atomicMax(L.bin_kmax + (base + i) * 3 + k, s_kmax[i * 3 + k]);
        }
    }
}

struct Box3 {
    float mn[3], mx[3];
    __device__ __forceinline__ void reset() {
        mn[0] = mn[1] = mn[2] = kArbMax;
        mx[0] = mx[1] = mx[2] = kArbMin;
    }
    __device__ __forceinline__ void grow_acc_first(const float* bmn, const float* bmx) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = gmin(mn[k], bmn[k]);
            mx[k] = gmax(mx[k], bmx[k]);
        }
    }
    __device__ __forceinline__ float area() const {  // Bounds::GetArea, BVHConstructor.h:41-44
        const float ex = __fsub_rn(mx[0], mn[0]), ey = __fsub_rn(mx[1], mn[1]), ez = __fsub_rn(mx[2], mn[2]);
        float a = __fmul_rn(ex, ey);
        a = __fadd_rn(a, __fmul_rn(ey, ez));
        a = __fadd_rn(a, __fmul_rn(ez, ex));
        return a;
    }
};

// SearchSAHPlaneBinned's sweep over one axis given its bins; returns the first strictly smallest
// cost (kInfCost when none) and its bin index.
__device__ float sweep_axis(const unsigned* cnt, const float* bmn, const float* bmx, int& best_i) {
    float larea[kBins - 1], rarea[kBins - 1];
    int lcount[kBins - 1], rcount[kBins - 1];
    Box3 lb, rb;
    lb.reset();
    rb.reset();
    int lsum = 0, rsum = 0;
    for (int i = 0; i < kBins - 1; ++i) {
        lsum += static_cast<int>(cnt[i]);
        lcount[i] = lsum;
        lb.grow_acc_first(bmn + 3 * i, bmx + 3 * i);
        larea[i] = lb.area();
        const int ir = kBins - 1 - i;
        rsum += static_cast<int>(cnt[ir]);
        rcount[ir - 1] = rsum;
        rb.grow_acc_first(bmn + 3 * ir, bmx + 3 * ir);
        rarea[ir - 1] = rb.area();
    }
    float best = kInfCost;
    best_i = -1;
    for (int i = 0; i < kBins - 1; ++i) {
        float c = __fmul_rn(__int2float_rn(lcount[i]), larea[i]);
        c = __fadd_rn(c, __fmul_rn(__int2float_rn(rcount[i]), rarea[i]));
        if (c < best) {
            best = c;
            best_i = i;
        }
    }
    return best;
}

// One warp per large node: lanes 0..2 sweep one axis each; lane 0 combines in axis order.
__global__ void k_split_large(Nodes N, Level L) {
    const int slot = blockIdx.x;
    const int lane = threadIdx.x;
    const int32_t id = L.node[slot];
    float mn[3], ext[3], scale[3];
    bool active[3];
    node_frame(N, id, mn, ext, scale, active);
    __shared__ float s_cost[3];
    __shared__ int s_i[3];
    if (lane < 3) {
        const int a = lane;
        float cost = kInfCost;
        int bi = -1;
        if (active[a]) {
            unsigned cnt[kBins];
            float bmn[3 * kBins], bmx[3 * kBins];
            const int64_t base = (static_cast<int64_t>(slot) * 3 + a) * kBins;
            for (int b = 0; b < kBins; ++b) {
                cnt[b] = L.bin_cnt[base + b];
                for (int k = 0; k < 3; ++k) {
                    if (cnt[b]) {
                        bmn[3 * b + k] = okey_value(L.bin_kmin[(base + b) * 3 + k]);
                        bmx[3 * b + k] = okey_value(L.bin_kmax[(base + b) * 3 + k]);
                    } else {  // an empty bin keeps the reset box
                        bmn[3 * b + k] = kArbMax;
                        bmx[3 * b + k] = kArbMin;
                    }
                }
            }
            cost = sweep_axis(cnt, bmn, bmx, bi);
        }
        s_cost[a] = cost;
        s_i[a] = bi;
    }
    __syncwarp();
    if (lane == 0) {
        float best = kInfCost;
        int axis = 0;
        float border = mn[0];  // no split found: the partition finds nothing -> midpoint split
        for (int a = 0; a < 3; ++a) {
            if (!active[a] || s_i[a] < 0) continue;
            if (s_cost[a] < best) {
                best = s_cost[a];
                axis = a;
                const float step = __fdiv_rn(ext[a], static_cast<float>(kBins));
                border = __fadd_rn(mn[a], __fmul_rn(step, static_cast<float>(s_i[a] + 1)));
            }
        }
        L.axis[slot] = axis;
        L.border[slot] = border;
    }
}

__global__ void __launch_bounds__(256) k_pred_large(Tri T, Nodes N, Level L, const Chunk* __restrict__ chunks,
                                                    const int32_t* __restrict__ refs, uint32_t* __restrict__ pred) {
    const Chunk c = chunks[blockIdx.x];
    const int axis = L.axis[c.slot];
    const float border = L.border[c.slot];
    for (int32_t q = c.begin + threadIdx.x; q < c.end; q += blockDim.x)
        pred[q] = T.cen(axis, refs[q]) < border ? 1u : 0u;
}

// Exclusive scan of n values (three passes; block partial sums scanned by one block).
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(const uint32_t* __restrict__ in, int64_t n,
                                                            uint32_t* __restrict__ out, uint32_t* __restrict__ sums) {
    __shared__ uint32_t s[kScanBlock];
    const int64_t i = static_cast<int64_t>(blockIdx.x) * kScanBlock + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
        const uint32_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void __launch_bounds__(kScanBlock) k_scan_sums(uint32_t* sums, int64_t nb) {
    __shared__ uint32_t s[kScanBlock];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nb; b0 += kScanBlock) {
        const int64_t i = b0 + threadIdx.x;
        const uint32_t v = i < nb ? sums[i] : 0u;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kScanBlock; o <<= 1) {
            const uint32_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry += s[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void k_scan_add(uint32_t* out, int64_t n, const uint32_t* sums) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * kScanBlock + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
    if (i == 0) out[n] = sums[(n + kScanBlock - 1) / kScanBlock];
}

__global__ void k_split_counts(Nodes N, Level L, const uint32_t* __restrict__ P, int32_t* fails) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= L.n_slots) return;
    const int32_t id = L.node[slot];
    const int32_t s = N.start[id], len = N.len[id];
    const int32_t k = static_cast<int32_t>(P[s + len] - P[s]);
    const bool fb = k == 0 || k == len;
    L.k_below[slot] = k;
    L.fallback[slot] = fb ? 1 : 0;
    L.mid[slot] = fb ? s + len / 2 : s + k;
    if (fb) atomicAdd(fails, 1);
}

__global__ void __launch_bounds__(256) k_ptr_init(Nodes N, Level L, const Chunk* __restrict__ chunks,
                                                  const uint32_t* __restrict__ pred, const uint32_t* __restrict__ P,
                                                  int32_t* __restrict__ ptr) {
    const Chunk c = chunks[blockIdx.x];
    const int32_t s = N.start[L.node[c.slot]];
    const bool fb = L.fallback[c.slot] != 0;
    for (int32_t q = c.begin + threadIdx.x; q < c.end; q += blockDim.x)
        ptr[q] = (pred[q] && !fb) ? s + static_cast<int32_t>(P[q] - P[s]) : q;
}

__global__ void __launch_bounds__(256) k_ptr_jump(const Chunk* __restrict__ chunks, const int32_t* __restrict__ a,
                                                  int32_t* __restrict__ b) {
    const Chunk c = chunks[blockIdx.x];
    for (int32_t q = c.begin + threadIdx.x; q < c.end; q += blockDim.x) b[q] = a[a[q]];
}

__global__ void __launch_bounds__(256) k_scatter(Nodes N, Level L, const Chunk* __restrict__ chunks,
                                                 const uint32_t* __restrict__ pred, const uint32_t* __restrict__ P,
                                                 const int32_t* __restrict__ ptr, const int32_t* __restrict__ refs,
                                                 int32_t* __restrict__ out) {
    const Chunk c = chunks[blockIdx.x];
    const int32_t s = N.start[L.node[c.slot]];
    const int32_t k = L.k_below[c.slot];
    const bool fb = L.fallback[c.slot] != 0;
    for (int32_t q = c.begin + threadIdx.x; q < c.end; q += blockDim.x) {
        if (fb) {
            out[q] = refs[q];
            continue;
        }
        if (pred[q]) out[s + static_cast<int32_t>(P[q] - P[s])] = refs[q];
        if (q >= s + k) out[q] = refs[ptr[q]];
    }
}

// Children of every large node: ids base + 2*slot (+1), classified for the next level.
__global__ void k_children(Nodes N, Level L, int32_t base, int32_t leaf_size, int32_t* next_large,
                           int32_t* n_next_large, int32_t* small, int32_t* n_small,
                           unsigned long long* ckeys) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= L.n_slots) return;
    const int32_t id = L.node[slot];
    const int32_t s = N.start[id], e = s + N.len[id], m = L.mid[slot];
    const int32_t kids[2] = {base + 2 * slot, base + 2 * slot + 1};
    const int32_t b[2] = {s, m}, l[2] = {m - s, e - m};
    N.left[id] = kids[0];
    N.right[id] = kids[1];
    for (int j = 0; j < 2; ++j) {
        const int32_t c = kids[j];
        N.start[c] = b[j];
        N.len[c] = l[j];
        N.parent[c] = id;
        N.left[c] = N.right[c] = -1;
        for (int k = 0; k < 3; ++k) {
            ckeys[k * N.cap + c] = ~0ull;
            ckeys[(3 + k) * N.cap + c] = 0ull;
        }
        if (l[j] <= leaf_size || l[j] <= 1) continue;  // leaf (ShouldBeLeaf, :456)
        if (l[j] > kSmall)
            next_large[atomicAdd(n_next_large, 1)] = c;
        else
            small[atomicAdd(n_small, 1)] = c;
    }
}

// Child bounds (:573-597): glm::min(x, acc) over the child's range keeps the earlier of equal
// values.  Keys: min (value, position), max (value, ~position).
__global__ void __launch_bounds__(256) k_child_keys(Tri T, Nodes N, Level L, const Chunk* __restrict__ chunks,
                                                    const int32_t* __restrict__ refs, unsigned long long* ckeys) {
    const Chunk c = chunks[blockIdx.x];
    const int32_t id = L.node[c.slot];
    const int32_t m = L.mid[c.slot];
    const int32_t lc = N.left[id], rc = N.right[id];
    for (int32_t q0 = c.begin; q0 < c.end; q0 += blockDim.x) {
        const int32_t q = q0 + threadIdx.x;
        const bool ok = q < c.end;
        const int32_t child = ok ? (q < m ? lc : rc) : -1;
        const int32_t r = ok ? refs[q] : 0;
        const unsigned am = __activemask();
        const int32_t first = __shfl_sync(am, child, __ffs(am) - 1);
        // one atomic per warp when every lane holds an element of the same child (a warp past the
        // chunk's end holds none: first < 0, and it must not touch the keys)
        const bool uniform = am == 0xFFFFFFFFu && first >= 0 && __all_sync(am, child == first);
        for (int k = 0; k < 3; ++k) {
            unsigned long long a = ok ? (static_cast<unsigned long long>(okey(T.mn(k, r))) << 32) |
                                            static_cast<uint32_t>(q)
                                      : ~0ull;
            unsigned long long b = ok ? (static_cast<unsigned long long>(okey(T.mx(k, r))) << 32) |
                                            (0xFFFFFFFFu - static_cast<uint32_t>(q))
                                      : 0ull;
            if (uniform) {
                a = warp_min64(a);
                b = warp_max64(b);
                if ((threadIdx.x & 31) == 0) {
                    atomicMin(ckeys + k * N.cap + first, a);
                    atomicMax(ckeys + (3 + k) * N.cap + first, b);
                }
            } else if (ok) {
                atomicMin(ckeys + k * N.cap + child, a);
                atomicMax(ckeys + (3 + k) * N.cap + child, b);
            }
        }
    }
}

__global__ void k_child_decode(Tri T, Nodes N, int32_t base, int32_t count, const int32_t* __restrict__ refs,
                               const unsigned long long* ckeys) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int32_t c = base + i;
    for (int k = 0; k < 3; ++k) {
        const unsigned long long a = ckeys[k * N.cap + c], b = ckeys[(3 + k) * N.cap + c];
        const int32_t pa = static_cast<int32_t>(static_cast<uint32_t>(a));
        const int32_t pb = static_cast<int32_t>(0xFFFFFFFFu - static_cast<uint32_t>(b));
        const float vmn = T.mn(k, refs[pa]), vmx = T.mx(k, refs[pb]);
        // glm::min(x, acc = ARBITRARY_MAX): the first x strictly below the sentinel
        N.box[k * N.cap + c] = vmn < kArbMax ? vmn : kArbMax;
        N.box[(3 + k) * N.cap + c] = vmx > kArbMin ? vmx : kArbMin;
    }
}

// ---- small subtrees: one warp builds the subtree of a node of at most kSmall triangles --------
//
// Per node: bins in shared memory (shared atomics; bin boxes only feed the areas), the sweep of
// SearchSAHPlaneBinned as warp prefix / suffix scans over the 64 bins (min / max / sum are exact
// and associative, so each prefix equals the sequential running box), the first strictly
// smallest cost by a warp reduction over (cost, split index), the parallel Lomuto partition in
// shared memory, and the child bounds by position-keyed warp reductions.
constexpr int kSmallWarps = 4;
constexpr int kStackCap = kSmall + 4;

struct WarpSmem {
    unsigned cnt[3 * kBins];
    unsigned kmin[3 * kBins * 3];
    unsigned kmax[3 * kBins * 3];
    int32_t ref[kSmall];
    int32_t out[kSmall];
    int32_t ptr[kSmall];
    int32_t ptr2[kSmall];
    int32_t jj[kSmall];
    int32_t stack[kStackCap];
};

__device__ __forceinline__ void box_union(float* mn, float* mx, const float* bmn, const float* bmx) {
    for (int k = 0; k < 3; ++k) {
        mn[k] = gmin(mn[k], bmn[k]);
        mx[k] = gmax(mx[k], bmx[k]);
    }
}
__device__ __forceinline__ float box_area(const float* mn, const float* mx) {  // Bounds::GetArea
    const float ex = __fsub_rn(mx[0], mn[0]), ey = __fsub_rn(mx[1], mn[1]), ez = __fsub_rn(mx[2], mn[2]);
    float a = __fmul_rn(ex, ey);
    a = __fadd_rn(a, __fmul_rn(ey, ez));
    a = __fadd_rn(a, __fmul_rn(ez, ex));
    return a;
}

// Sweep of one axis by the whole warp: returns the key (cost, split) of the first strictly
// smallest cost below INF_COST, or ~0 when there is none.
__device__ unsigned long long warp_sweep(const WarpSmem& W, int a, unsigned lane) {
    float bmn[2][3], bmx[2][3];
    int c[2];
    for (int h = 0; h < 2; ++h) {
        const int b = a * kBins + 2 * static_cast<int>(lane) + h;
        c[h] = static_cast<int>(W.cnt[b]);
        for (int k = 0; k < 3; ++k) {
            bmn[h][k] = c[h] ? okey_value(W.kmin[b * 3 + k]) : kArbMax;
            bmx[h][k] = c[h] ? okey_value(W.kmax[b * 3 + k]) : kArbMin;
        }
    }
    // lane totals
    float tmn[3], tmx[3];
    for (int k = 0; k < 3; ++k) {
        tmn[k] = gmin(bmn[0][k], bmn[1][k]);
        tmx[k] = gmax(bmx[0][k], bmx[1][k]);
    }
    const int tc = c[0] + c[1];
    // exclusive prefix over lanes < lane (E) and exclusive suffix over lanes > lane (Q)
    float emn[3] = {kArbMax, kArbMax, kArbMax}, emx[3] = {kArbMin, kArbMin, kArbMin};
    float qmn[3] = {kArbMax, kArbMax, kArbMax}, qmx[3] = {kArbMin, kArbMin, kArbMin};
    int ec = 0, qc = 0;
    {
        float imn[3], imx[3];
        int ic = tc;
        for (int k = 0; k < 3; ++k) {
            imn[k] = tmn[k];
            imx[k] = tmx[k];
        }
        for (int o = 1; o < 32; o <<= 1) {  // inclusive prefix
            float umn[3], umx[3];
            for (int k = 0; k < 3; ++k) {
                umn[k] = __shfl_up_sync(0xFFFFFFFFu, imn[k], o);
                umx[k] = __shfl_up_sync(0xFFFFFFFFu, imx[k], o);
            }
            const int uc = __shfl_up_sync(0xFFFFFFFFu, ic, o);
            if (lane >= static_cast<unsigned>(o)) {
                box_union(imn, imx, umn, umx);
                ic += uc;
            }
        }
        for (int k = 0; k < 3; ++k) {
            emn[k] = __shfl_up_sync(0xFFFFFFFFu, imn[k], 1);
            emx[k] = __shfl_up_sync(0xFFFFFFFFu, imx[k], 1);
        }
        ec = __shfl_up_sync(0xFFFFFFFFu, ic, 1);
        if (lane == 0) {
            for (int k = 0; k < 3; ++k) {
                emn[k] = kArbMax;
                emx[k] = kArbMin;
            }
            ec = 0;
        }
        for (int k = 0; k < 3; ++k) {
            imn[k] = tmn[k];
            imx[k] = tmx[k];
        }
        ic = tc;
        for (int o = 1; o < 32; o <<= 1) {  // inclusive suffix
            float umn[3], umx[3];
            for (int k = 0; k < 3; ++k) {
                umn[k] = __shfl_down_sync(0xFFFFFFFFu, imn[k], o);
                umx[k] = __shfl_down_sync(0xFFFFFFFFu, imx[k], o);
            }
            const int uc = __shfl_down_sync(0xFFFFFFFFu, ic, o);
            if (lane + o < 32u) {
                box_union(imn, imx, umn, umx);
                ic += uc;
            }
        }
        for (int k = 0; k < 3; ++k) {
            qmn[k] = __shfl_down_sync(0xFFFFFFFFu, imn[k], 1);
            qmx[k] = __shfl_down_sync(0xFFFFFFFFu, imx[k], 1);
        }
        qc = __shfl_down_sync(0xFFFFFFFFu, ic, 1);
        if (lane == 31) {
            for (int k = 0; k < 3; ++k) {
                qmn[k] = kArbMax;
                qmx[k] = kArbMin;
            }
            qc = 0;
        }
    }
    unsigned long long best = ~0ull;
    // split i = 2*lane: left = E + bin0, right = Q + bin1
    {
        float lmn[3], lmx[3], rmn[3], rmx[3];
        for (int k = 0; k < 3; ++k) {
            lmn[k] = emn[k];
            lmx[k] = emx[k];
            rmn[k] = qmn[k];
            rmx[k] = qmx[k];
        }
        box_union(lmn, lmx, bmn[0], bmx[0]);
        box_union(rmn, rmx, bmn[1], bmx[1]);
        float cst = __fmul_rn(__int2float_rn(ec + c[0]), box_area(lmn, lmx));
        cst = __fadd_rn(cst, __fmul_rn(__int2float_rn(qc + c[1]), box_area(rmn, rmx)));
        if (cst < kInfCost)
            best = (static_cast<unsigned long long>(okey(cst)) << 32) | (2u * lane);
    }
    // split i = 2*lane + 1 (i <= 62): left = E + bin0 + bin1, right = Q
    if (lane < 31) {
        float lmn[3], lmx[3];
        for (int k = 0; k < 3; ++k) {
            lmn[k] = emn[k];
            lmx[k] = emx[k];
        }
        box_union(lmn, lmx, tmn, tmx);
        float cst = __fmul_rn(__int2float_rn(ec + tc), box_area(lmn, lmx));
        cst = __fadd_rn(cst, __fmul_rn(__int2float_rn(qc), box_area(qmn, qmx)));
        if (cst < kInfCost) {
            const unsigned long long key = (static_cast<unsigned long long>(okey(cst)) << 32) | (2u * lane + 1u);
            best = key < best ? key : best;
        }
    }
    best = warp_min64(best);
    return __shfl_sync(0xFFFFFFFFu, best, 0);
}

__device__ __forceinline__ unsigned lane_lt_mask() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__global__ void __launch_bounds__(32 * kSmallWarps) k_small(Tri T, Nodes N, const int32_t* __restrict__ list,
                                                            int32_t count, int32_t* refs, int32_t leaf_size,
                                                            int32_t* node_counter, int32_t* fails, int32_t* overflow) {
    __shared__ WarpSmem smem[kSmallWarps];
    const unsigned lane = threadIdx.x & 31u;
    const int w = threadIdx.x >> 5;
    const int32_t item = blockIdx.x * kSmallWarps + w;
    if (item >= count) return;  // whole warp
    WarpSmem& W = smem[w];
    int sp = 0;
    if (lane == 0) W.stack[0] = list[item];
    sp = 1;
    __syncwarp();
    for (int guard = 0; sp > 0 && guard < 4 * kSmall + 8; ++guard) {
        const int32_t id = W.stack[--sp];
        __syncwarp();
        const int32_t s = N.start[id], len = N.len[id];
        if (len <= leaf_size || len <= 1) continue;  // leaf: left/right stay -1
        float mn[3], ext[3], scale[3];
        bool active[3];
        node_frame(N, id, mn, ext, scale, active);
        for (int i = lane; i < 3 * kBins; i += 32) W.cnt[i] = 0u;
        for (int i = lane; i < 3 * kBins * 3; i += 32) {
            W.kmin[i] = 0xFFFFFFFFu;
            W.kmax[i] = 0u;
        }
        for (int i = lane; i < len; i += 32) W.ref[i] = refs[s + i];
        __syncwarp();
        for (int i = lane; i < len; i += 32) {
            const int32_t r = W.ref[i];
            uint32_t km[3], kx[3];
            for (int k = 0; k < 3; ++k) {
                km[k] = okey(T.mn(k, r));
                kx[k] = okey(T.mx(k, r));
            }
            for (int a = 0; a < 3; ++a) {
                if (!active[a]) continue;
                const int b = a * kBins + bin_of(T.cen(a, r), mn[a], scale[a]);
                atomicAdd(&W.cnt[b], 1u);
                for (int k = 0; k < 3; ++k) {
                    atomicMin(&W.kmin[b * 3 + k], km[k]);
                    atomicMax(&W.kmax[b * 3 + k], kx[k]);
                }
            }
        }
        __syncwarp();
        // split: axes in order, first strictly smaller cost (SearchSAHPlaneBinned)
        int axis = 0;
        float border = mn[0];
        {
            unsigned long long bkey = ~0ull;
            for (int a = 0; a < 3; ++a) {
                if (!active[a]) continue;
                const unsigned long long key = warp_sweep(W, a, lane);
                if (key == ~0ull) continue;
                if ((key >> 32) < (bkey >> 32)) {  // strictly smaller cost (okey order)
                    bkey = key;
                    axis = a;
                }
            }
            if (bkey != ~0ull) {
                const int bi = static_cast<int>(bkey & 0xFFFFFFFFull);
                const float step = __fdiv_rn(ext[axis], static_cast<float>(kBins));
                border = __fadd_rn(mn[axis], __fmul_rn(step, static_cast<float>(bi + 1)));
            }
        }
        // parallel Lomuto partition in shared memory (see the file header)
        int32_t k_below = 0;
        for (int i0 = 0; i0 < len; i0 += 32) {
            const int i = i0 + static_cast<int>(lane);
            const bool p = i < len && T.cen(axis, W.ref[i]) < border;
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, p);
            if (i < len) {
                const int32_t j = k_below + __popc(bal & lane_lt_mask());
                W.jj[i] = j;
                W.ptr[i] = p ? j : i;
            }
            k_below += __popc(bal);
        }
        __syncwarp();
        const bool fb = k_below == 0 || k_below == len;
        int32_t mid = fb ? len / 2 : k_below;
        if (fb) {
            if (lane == 0) atomicAdd(fails, 1);
        } else {
            int32_t* pa = W.ptr;
            int32_t* pb = W.ptr2;
            for (int r = 0; r < 9; ++r) {  // 2^8 = kSmall: chains are shorter than len <= kSmall
                for (int i = lane; i < len; i += 32) pb[i] = pa[pa[i]];
                __syncwarp();
                int32_t* t = pa;
                pa = pb;
                pb = t;
            }
            for (int i = lane; i < len; i += 32) {
                const int32_t r = W.ref[i];
                if (T.cen(axis, r) < border) W.out[W.jj[i]] = r;
                if (i >= k_below) W.out[i] = W.ref[pa[i]];
            }
            __syncwarp();
            for (int i = lane; i < len; i += 32) {
                refs[s + i] = W.out[i];
                W.ref[i] = W.out[i];
            }
            __syncwarp();
        }
        // children
        int32_t L = 0;
        if (lane == 0) L = atomicAdd(node_counter, 2);
        L = __shfl_sync(0xFFFFFFFFu, L, 0);
        if (L + 1 >= N.cap || sp + 2 > kStackCap) {
            if (lane == 0) atomicOr(overflow, 1);
            return;
        }
        const int32_t R = L + 1;
        const int32_t cb[2] = {0, mid}, cl[2] = {mid, len - mid}, kid[2] = {L, R};
        for (int j = 0; j < 2; ++j) {
            unsigned long long kmn[3], kmx[3];
            for (int k = 0; k < 3; ++k) {
                kmn[k] = ~0ull;
                kmx[k] = 0ull;
            }
            for (int i = cb[j] + static_cast<int>(lane); i < cb[j] + cl[j]; i += 32) {
                const int32_t r = W.ref[i];
                for (int k = 0; k < 3; ++k) {
                    const unsigned long long a =
                        (static_cast<unsigned long long>(okey(T.mn(k, r))) << 32) | static_cast<uint32_t>(i);
                    const unsigned long long b = (static_cast<unsigned long long>(okey(T.mx(k, r))) << 32) |
                                                 (0xFFFFFFFFu - static_cast<uint32_t>(i));
                    kmn[k] = a < kmn[k] ? a : kmn[k];
                    kmx[k] = b > kmx[k] ? b : kmx[k];
                }
            }
            for (int k = 0; k < 3; ++k) {
                kmn[k] = warp_min64(kmn[k]);
                kmx[k] = warp_max64(kmx[k]);
            }
            if (lane == 0) {
                const int32_t c = kid[j];
                N.start[c] = s + cb[j];
                N.len[c] = cl[j];
                N.parent[c] = id;
                N.left[c] = N.right[c] = -1;
                for (int k = 0; k < 3; ++k) {  // glm::min(x, acc): the first of equal values
                    const int32_t pmn = static_cast<int32_t>(static_cast<uint32_t>(kmn[k]));
                    const int32_t pmx = static_cast<int32_t>(0xFFFFFFFFu - static_cast<uint32_t>(kmx[k]));
                    const float vmn = T.mn(k, W.ref[pmn]), vmx = T.mx(k, W.ref[pmx]);
                    N.box[k * N.cap + c] = vmn < kArbMax ? vmn : kArbMax;
                    N.box[(3 + k) * N.cap + c] = vmx > kArbMin ? vmx : kArbMin;
                }
            }
        }
        if (lane == 0) {
            N.left[id] = L;
            N.right[id] = R;
            W.stack[sp] = R;
            W.stack[sp + 1] = L;
        }
        sp += 2;
        __syncwarp();
    }
}

// ---- flattening --------------------------------------------------------------------------------

// Leaves: sorted offset n - start - len (the LIFO walk visits higher ranges first) and triangles.
__global__ void k_leaves(Nodes N, int32_t total, int32_t n, const int32_t* __restrict__ refs,
                         int32_t* __restrict__ sorted, int32_t* leaf_count) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total || N.left[x] >= 0) return;
    const int32_t s = N.start[x], len = N.len[x], off = n - s - len;
    for (int32_t i = 0; i < len; ++i) sorted[off + i] = refs[s + i];
    atomicAdd(leaf_count, 1);
}

__global__ void k_tris_out(const uint32_t* __restrict__ idx, const int32_t* __restrict__ mesh, int64_t n,
                           const int32_t* __restrict__ sorted, int4* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t t = sorted[i];
    out[i] = make_int4(static_cast<int32_t>(idx[t * 3]), static_cast<int32_t>(idx[t * 3 + 1]),
                       static_cast<int32_t>(idx[t * 3 + 2]), mesh ? mesh[t] : 0);
}

// Subtree node counts, bottom-up: the second child to arrive at a parent continues upward.
__global__ void k_sizes(Nodes N, int32_t total, int32_t* size, int32_t* arrive) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total || N.left[x] >= 0) return;
    size[x] = 1;
    int32_t c = x;
    for (int guard = 0; guard < total; ++guard) {
        const int32_t p = N.parent[c];
        if (p < 0) return;
        __threadfence();
        if (atomicAdd(arrive + p, 1) == 0) return;
        __threadfence();
        const int32_t sl = __ldcg(size + N.left[p]), sr = __ldcg(size + N.right[p]);
        size[p] = 1 + sl + sr;
        c = p;
    }
}

// Path sums to the root by pointer jumping: out[x] = sum of val over x and its ancestors.
__global__ void k_jump_sum(int32_t total, const int32_t* anc, const int64_t* val, int32_t* anc2, int64_t* val2) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total) return;
    const int32_t a = anc[x];
    val2[x] = a >= 0 ? val[x] + val[a] : val[x];
    anc2[x] = a >= 0 ? anc[a] : -1;
}

// Position among internal nodes in the reference's LIFO walk (node, then right, then left):
// 1 per internal ancestor plus, when x lies in a left subtree, the internal nodes of the right
// sibling's subtree.
__global__ void k_walk_val(Nodes N, int32_t total, const int32_t* size, int64_t* val, int32_t* anc) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total) return;
    const int32_t p = N.parent[x];
    anc[x] = p;
    if (p < 0) {
        val[x] = 0;
        return;
    }
    val[x] = 1 + (N.left[p] == x ? (size[N.right[p]] - 1) / 2 : 0);
}

// Stackless DFS pre-order with the (swapped) first child first.
__global__ void k_pre_val(Nodes N, int32_t total, const int32_t* size, const int64_t* walk,
                          const int32_t* draws, int32_t use_swaps, int64_t* val, int32_t* anc,
                          int32_t* first_of) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total) return;
    if (N.left[x] >= 0) {
        const bool sw = use_swaps && draws[walk[x]] <= 2;
        first_of[x] = sw ? N.right[x] : N.left[x];
    } else {
        first_of[x] = -1;
    }
    // val depends on the parent's first child, filled by the parent's thread: done in a second
    // kernel (k_pre_val2) after this one.
    anc[x] = N.parent[x];
    val[x] = 0;
}
__global__ void k_pre_val2(Nodes N, int32_t total, const int32_t* size, const int32_t* first_of, int64_t* val) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total) return;
    const int32_t p = N.parent[x];
    if (p < 0) return;
    const int32_t f = first_of[p];
    val[x] = 1 + (f == x ? 0 : size[f]);
}

__device__ __forceinline__ float ibits(int32_t i) { return __int_as_float(i); }

__global__ void k_stackless_out(Nodes N, int32_t total, int32_t n, int32_t tri_offset, const int64_t* flat,
                                const int32_t* size, float* __restrict__ F) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total) return;
    const int64_t f = flat[x];
    float* o = F + f * 8;
    for (int k = 0; k < 3; ++k) {
        o[k] = N.box[k * N.cap + x];
        o[4 + k] = N.box[(3 + k) * N.cap + x];
    }
    if (N.left[x] < 0) {
        const int32_t off = n - N.start[x] - N.len[x] + tri_offset;
        o[3] = ibits((off << 4) | (N.len[x] & 0xF));
    } else {
        o[3] = ibits(-1);
    }
    const int64_t nx = f + size[x];
    o[7] = ibits(nx < total ? static_cast<int32_t>(nx) : -1);
}

// Stack layout, BFS over internal nodes, one level at a time: rank the level's internal nodes,
// give them BFS indices and queue their children (left, right) in order.
__global__ void k_bfs_flags(Nodes N, const int32_t* lvl, int32_t count, uint32_t* flag) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) flag[i] = N.left[lvl[i]] >= 0 ? 1u : 0u;
}
__global__ void k_bfs_expand(Nodes N, const int32_t* lvl, int32_t count, const uint32_t* rank, int32_t bfs_base,
                             int32_t* bfs, int32_t* next) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int32_t x = lvl[i];
    if (N.left[x] < 0) return;
    const int32_t r = static_cast<int32_t>(rank[i]);
    bfs[x] = bfs_base + r;
    next[2 * r] = N.left[x];
    next[2 * r + 1] = N.right[x];
}

__global__ void k_stack_out(Nodes N, int32_t total, int32_t n, int32_t tri_offset, const int32_t* bfs,
                            float* __restrict__ F) {
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= total || N.left[x] < 0) return;
    float* o = F + static_cast<int64_t>(bfs[x]) * 16;
    const int32_t kids[2] = {N.left[x], N.right[x]};
    for (int s = 0; s < 2; ++s) {
        const int32_t c = kids[s];
        float* b = o + s * 8;
        for (int k = 0; k < 3; ++k) {
            b[k] = N.box[k * N.cap + c];
            b[4 + k] = N.box[(3 + k) * N.cap + c];
        }
        if (N.left[c] < 0) {
            const int32_t off = n - N.start[c] - N.len[c] + tri_offset;
            b[3] = ibits((off << 4) | (N.len[c] & 0xF));
            b[7] = 0.0f;
        } else {
            b[3] = ibits(-1);
            b[7] = ibits(bfs[c]);
        }
    }
}

inline unsigned blocks(int64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

// Sub-allocator over one device buffer: measure mode (base == nullptr) only adds up the aligned
// sizes, so the same carve sequence first sizes and then fills the context's build buffer.
struct Arena {
    char* base = nullptr;
    size_t used = 0, cap = 0;
    bool over = false;
    template <class T>
    T* get(int64_t count) {
        const size_t bytes = (static_cast<size_t>(std::max<int64_t>(count, 1)) * sizeof(T) + 255) & ~size_t(255);
        T* p = base ? reinterpret_cast<T*>(base + used) : nullptr;
        used += bytes;
        if (base && used > cap) over = true;
        return p;
    }
};

// Every device buffer of one build (tree-sized ones at the node capacity 2n + 1).
struct Buffers {
    float* verts;
    uint32_t* idx;
    int32_t* mesh;
    float* tb;
    int32_t *refs, *refs2;
    uint32_t *pred, *P, *sums;
    int32_t *ptr, *ptr2;
    int32_t *nstart, *nlen, *nleft, *nright, *nparent;
    float* nbox;
    unsigned long long* ckeys;
    int32_t *cnt, *large, *next, *small;
    unsigned *bin_cnt, *bin_kmin, *bin_kmax;
    int32_t* axis;
    float* border;
    int32_t *k_below, *mid, *fallback, *slot_info;
    Chunk* chunks;
    unsigned long long* rootkeys;
    // flattening
    int32_t *sorted, *size, *arrive, *anc, *anc2;
    int4* tris;
    int64_t *val, *val2, *walk;
    float* F;
    int32_t *draws, *first, *bfs, *lvl, *lvl2;
    uint32_t* flag;
};

void carve(Arena& a, Buffers& b, int64_t n, int64_t n_verts, bool mesh, int layout) {
    const int64_t cap = 2 * n + 1;
    const int64_t max_slots = n / (kSmall + 1) + 2;
    b.verts = a.get<float>(n_verts * 8);
    b.idx = a.get<uint32_t>(n * 3);
    b.mesh = mesh ? a.get<int32_t>(n) : nullptr;
    b.tb = a.get<float>(9 * n);
    b.refs = a.get<int32_t>(n);
    b.refs2 = a.get<int32_t>(n);
    b.pred = a.get<uint32_t>(n);
    b.P = a.get<uint32_t>(cap + 1);
    b.sums = a.get<uint32_t>(cap / kScanBlock + 2);
    b.ptr = a.get<int32_t>(n);
    b.ptr2 = a.get<int32_t>(n);
    b.nstart = a.get<int32_t>(cap);
    b.nlen = a.get<int32_t>(cap);
    b.nleft = a.get<int32_t>(cap);
    b.nright = a.get<int32_t>(cap);
    b.nparent = a.get<int32_t>(cap);
    b.nbox = a.get<float>(6 * cap);
    b.ckeys = a.get<unsigned long long>(6 * cap);
    b.cnt = a.get<int32_t>(16);
    b.large = a.get<int32_t>(max_slots);
    b.next = a.get<int32_t>(max_slots);
    b.small = a.get<int32_t>(n + 1);
    b.bin_cnt = a.get<unsigned>(max_slots * 3 * kBins);
    b.bin_kmin = a.get<unsigned>(max_slots * 3 * kBins * 3);
    b.bin_kmax = a.get<unsigned>(max_slots * 3 * kBins * 3);
    b.axis = a.get<int32_t>(max_slots);
    b.border = a.get<float>(max_slots);
    b.k_below = a.get<int32_t>(max_slots);
    b.mid = a.get<int32_t>(max_slots);
    b.fallback = a.get<int32_t>(max_slots);
    b.slot_info = a.get<int32_t>(2 * max_slots);
    b.chunks = a.get<Chunk>(n / kChunk + max_slots + 2);
    b.rootkeys = a.get<unsigned long long>(6);
    b.sorted = a.get<int32_t>(n);
    b.tris = a.get<int4>(n);
    b.size = a.get<int32_t>(cap);
    b.arrive = a.get<int32_t>(cap);
    b.val = a.get<int64_t>(cap);
    b.val2 = a.get<int64_t>(cap);
    b.anc = a.get<int32_t>(cap);
    b.anc2 = a.get<int32_t>(cap);
    b.F = a.get<float>(cap * (layout == 1 ? 8 : 16));
    if (layout == 1) {
        b.draws = a.get<int32_t>(cap / 2 + 1);
        b.first = a.get<int32_t>(cap);
        b.walk = a.get<int64_t>(cap);
    } else {
        b.bfs = a.get<int32_t>(cap);
        b.lvl = a.get<int32_t>(cap + 1);
        b.lvl2 = a.get<int32_t>(cap + 1);
        b.flag = a.get<uint32_t>(cap + 1);
    }
}

}  // namespace

// Exclusive scan helper: out[0..n] (out[n] = total) of in[0..n).
static cudaError_t scan_u32(const uint32_t* in, int64_t n, uint32_t* out, uint32_t* sums, cudaStream_t st) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    k_scan_blocks<<<static_cast<unsigned>(std::max<int64_t>(nb, 1)), kScanBlock, 0, st>>>(in, n, out, sums);
    k_scan_sums<<<1, kScanBlock, 0, st>>>(sums, nb);
    k_scan_add<<<static_cast<unsigned>(std::max<int64_t>(nb, 1)), kScanBlock, 0, st>>>(out, n, sums);
    return cudaGetLastError();
}

// GPU build of one object.  Returns RQ_OK and fills `out` like build_bvh, else a status with
// `why`.  Inputs are host arrays (the rq_build_bvh interface).  Device buffers come from one
// grow-only scratch buffer of the context, so repeated builds allocate nothing.
rq_status build_bvh_gpu(rq_ctx* ctx, const BuildInput& in, BuildOutput& out, std::string& why) {
    const auto t0 = std::chrono::steady_clock::now();
    const int64_t n = in.n_tris;
    if (!in.vert_records || !in.indices || n <= 0 || in.n_verts <= 0 || in.leaf_size < 1 || in.leaf_size > 15 ||
        (in.layout != 0 && in.layout != 1) || n + static_cast<int64_t>(in.tri_offset) >= (int64_t(1) << 27) ||
        (in.layout == 0 && n <= in.leaf_size)) {
        why = "invalid build input (leaf size 1..15, < 2^27 triangles, stack layout needs more triangles than "
              "one leaf)";
        return RQ_EINVAL;
    }
    for (int64_t i = 0; i < n * 3; ++i)
        if (static_cast<int64_t>(in.indices[i]) >= in.n_verts) {
            why = "vertex index out of range";
            return RQ_EINVAL;
        }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
        why = cudaGetErrorString(e);
        return RQ_ECUDA;
    }
    cudaStream_t st = ctx->stream;
    const int64_t cap = 2 * n + 1;
    const int64_t max_slots = n / (kSmall + 1) + 2;
    Buffers B{};
    {
        Arena m;
        carve(m, B, n, in.n_verts, in.mesh_ids != nullptr, in.layout);
        void* base = nullptr;
        rq_status s = scratch(ctx, rq::kSlotBuild, m.used, &base);
        if (s != RQ_OK) {
            why = "device allocation failed during GPU BVH build";
            return RQ_ENOMEM;
        }
        Arena a;
        a.base = static_cast<char*>(base);
        a.cap = m.used;
        carve(a, B, n, in.n_verts, in.mesh_ids != nullptr, in.layout);
        if (a.over) {
            why = "GPU BVH build: buffer layout mismatch";
            return RQ_EINVAL;
        }
    }
    float* d_verts = B.verts;
    uint32_t* d_idx = B.idx;
    int32_t* d_mesh = B.mesh;
    float* d_tb = B.tb;
    int32_t* d_refs = B.refs;
    int32_t* d_refs2 = B.refs2;
    uint32_t* d_pred = B.pred;
    uint32_t* d_P = B.P;
    uint32_t* d_sums = B.sums;
    int32_t* d_ptr = B.ptr;
    int32_t* d_ptr2 = B.ptr2;
    Nodes N{B.nstart, B.nlen, B.nleft, B.nright, B.nparent, B.nbox, cap};
    unsigned long long* d_ckeys = B.ckeys;
    int32_t* d_cnt = B.cnt;  // [0] nodes, [1] fails, [2] overflow, [3] next large, [4] small, [5] leaves
    int32_t* d_large = B.large;
    int32_t* d_next = B.next;
    int32_t* d_small = B.small;
    Level L{};
    L.bin_cnt = B.bin_cnt;
    L.bin_kmin = B.bin_kmin;
    L.bin_kmax = B.bin_kmax;
    L.axis = B.axis;
    L.border = B.border;
    L.k_below = B.k_below;
    L.mid = B.mid;
    L.fallback = B.fallback;
    int32_t* d_slot_info = B.slot_info;  // start, len per slot (for the host)
    Chunk* d_chunks = B.chunks;
    unsigned long long* d_rootkeys = B.rootkeys;
    (void)max_slots;
    auto fail_cuda = [&](cudaError_t err, const char* what) {
        why = std::string(what) + ": " + cudaGetErrorString(err);
        return RQ_ECUDA;
    };
#define GB_CHECK(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return fail_cuda(e_, #call); \
    } while (0)
    GB_CHECK(cudaMemcpyAsync(d_verts, in.vert_records, sizeof(float) * 8 * in.n_verts, cudaMemcpyHostToDevice, st));
    GB_CHECK(cudaMemcpyAsync(d_idx, in.indices, sizeof(uint32_t) * 3 * n, cudaMemcpyHostToDevice, st));
    if (d_mesh) GB_CHECK(cudaMemcpyAsync(d_mesh, in.mesh_ids, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    GB_CHECK(cudaMemsetAsync(d_cnt, 0, 16 * sizeof(int32_t), st));
    k_tri_bounds<<<blocks(n, 256), 256, 0, st>>>(d_verts, d_idx, n, d_tb, d_refs);
    const Tri T{d_tb, n};
    {
        const unsigned long long init[6] = {~0ull, ~0ull, ~0ull, 0ull, 0ull, 0ull};
        GB_CHECK(cudaMemcpyAsync(d_rootkeys, init, sizeof(init), cudaMemcpyHostToDevice, st));
        k_root_keys<<<blocks(n, 256), 256, 0, st>>>(T, d_rootkeys);
        k_root_decode<<<1, 32, 0, st>>>(T, d_rootkeys, N, 0, static_cast<int32_t>(n));
        GB_CHECK(cudaGetLastError());
    }
    int32_t node_count = 1;
    std::vector<int32_t> large_ids;  // current level's large nodes (host copy of ids)
    int32_t n_small = 0;
    if (n > kSmall) {
        large_ids.push_back(0);
    } else if (n > in.leaf_size) {
        const int32_t zero = 0;
        GB_CHECK(cudaMemcpyAsync(d_small, &zero, sizeof(int32_t), cudaMemcpyHostToDevice, st));
        n_small = 1;
    }
    std::vector<Chunk> chunks;
    std::vector<int32_t> info;
    int levels = 0;
    while (!large_ids.empty()) {
        if (++levels > kMaxLevels) {
            why = "GPU BVH build: too many levels of large nodes";
            return RQ_EBUDGET;
        }
        const int32_t slots = static_cast<int32_t>(large_ids.size());
        GB_CHECK(cudaMemcpyAsync(d_large, large_ids.data(), sizeof(int32_t) * slots, cudaMemcpyHostToDevice, st));
        // host copy of the level's ranges (chunk table)
        info.resize(2 * slots);
        {
            k_gather_info<<<blocks(slots, 128), 128, 0, st>>>(N, d_large, slots, d_slot_info);
            GB_CHECK(cudaMemcpyAsync(info.data(), d_slot_info, sizeof(int32_t) * 2 * slots, cudaMemcpyDeviceToHost, st));
            GB_CHECK(cudaStreamSynchronize(st));
            chunks.clear();
            int32_t max_len = 0;
            for (int32_t s = 0; s < slots; ++s) {
                const int32_t b0 = info[2 * s], ln = info[2 * s + 1];
                max_len = std::max(max_len, ln);
                for (int32_t b = b0; b < b0 + ln; b += kChunk)
                    chunks.push_back(Chunk{s, b, std::min(b + kChunk, b0 + ln)});
            }
            const int32_t nch = static_cast<int32_t>(chunks.size());
            GB_CHECK(cudaMemcpyAsync(d_chunks, chunks.data(), sizeof(Chunk) * nch, cudaMemcpyHostToDevice, st));
            L.node = d_large;
            L.n_slots = slots;
            GB_CHECK(cudaMemsetAsync(L.bin_cnt, 0, sizeof(unsigned) * slots * 3 * kBins, st));
            GB_CHECK(cudaMemsetAsync(L.bin_kmin, 0xFF, sizeof(unsigned) * slots * 3 * kBins * 3, st));
            GB_CHECK(cudaMemsetAsync(L.bin_kmax, 0, sizeof(unsigned) * slots * 3 * kBins * 3, st));
            k_bin_large<<<nch, 256, 0, st>>>(T, N, L, d_chunks, d_refs);
            k_split_large<<<slots, 32, 0, st>>>(N, L);
            GB_CHECK(cudaMemsetAsync(d_pred, 0, sizeof(uint32_t) * n, st));
            k_pred_large<<<nch, 256, 0, st>>>(T, N, L, d_chunks, d_refs, d_pred);
            GB_CHECK(scan_u32(d_pred, n, d_P, d_sums, st));
            k_split_counts<<<blocks(slots, 128), 128, 0, st>>>(N, L, d_P, d_cnt + 1);
            k_ptr_init<<<nch, 256, 0, st>>>(N, L, d_chunks, d_pred, d_P, d_ptr);
            int rounds = 1;
            while ((int64_t(1) << rounds) < max_len) ++rounds;
            for (int r = 0; r <= rounds; ++r) {
                k_ptr_jump<<<nch, 256, 0, st>>>(d_chunks, d_ptr, d_ptr2);
                std::swap(d_ptr, d_ptr2);
            }
            GB_CHECK(cudaMemcpyAsync(d_refs2, d_refs, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
            k_scatter<<<nch, 256, 0, st>>>(N, L, d_chunks, d_pred, d_P, d_ptr, d_refs, d_refs2);
            std::swap(d_refs, d_refs2);
            const int32_t base = node_count;
            node_count += 2 * slots;
            if (node_count + 1 > cap) {
                why = "GPU BVH build: node capacity exceeded";
                return RQ_EBUDGET;
            }
            GB_CHECK(cudaMemsetAsync(d_cnt + 3, 0, sizeof(int32_t), st));
            k_children<<<blocks(slots, 128), 128, 0, st>>>(N, L, base, in.leaf_size, d_next, d_cnt + 3,
                                                          d_small, d_cnt + 4, d_ckeys);
            k_child_keys<<<nch, 256, 0, st>>>(T, N, L, d_chunks, d_refs, d_ckeys);
            k_child_decode<<<blocks(2 * slots, 128), 128, 0, st>>>(T, N, base, 2 * slots, d_refs, d_ckeys);
            GB_CHECK(cudaGetLastError());
            int32_t n_next = 0;
            GB_CHECK(cudaMemcpyAsync(&n_next, d_cnt + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
            GB_CHECK(cudaStreamSynchronize(st));
            large_ids.resize(n_next);
            if (n_next) {
                GB_CHECK(cudaMemcpyAsync(large_ids.data(), d_next, sizeof(int32_t) * n_next, cudaMemcpyDeviceToHost, st));
                GB_CHECK(cudaStreamSynchronize(st));
            }
            // a stable level order (ids ascend with creation) keeps the schedule deterministic
            std::sort(large_ids.begin(), large_ids.end());
        }
    }
    {
        int32_t ns = 0;
        GB_CHECK(cudaMemcpyAsync(&ns, d_cnt + 4, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        GB_CHECK(cudaStreamSynchronize(st));
        n_small = std::max(n_small, ns);
    }
    GB_CHECK(cudaMemcpyAsync(d_cnt, &node_count, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    if (n_small > 0)
        k_small<<<blocks(n_small, kSmallWarps), 32 * kSmallWarps, 0, st>>>(T, N, d_small, n_small, d_refs,
                                                                        in.leaf_size, d_cnt, d_cnt + 1,
                                                    d_cnt + 2);
    GB_CHECK(cudaGetLastError());
    int32_t cnt_h[3] = {0, 0, 0};
    GB_CHECK(cudaMemcpyAsync(cnt_h, d_cnt, sizeof(cnt_h), cudaMemcpyDeviceToHost, st));
    GB_CHECK(cudaStreamSynchronize(st));
    if (cnt_h[2]) {
        why = "GPU BVH build: subtree stack or node capacity exceeded";
        return RQ_EBUDGET;
    }
    const int32_t total = cnt_h[0];
    out.split_fails = cnt_h[1];

    // ---- flatten
    int32_t* d_sorted = B.sorted;
    int4* d_tris = B.tris;
    int32_t* d_size = B.size;
    int32_t* d_arrive = B.arrive;
    int64_t* d_val = B.val;
    int64_t* d_val2 = B.val2;
    int32_t* d_anc = B.anc;
    int32_t* d_anc2 = B.anc2;
    float* d_F = B.F;
    GB_CHECK(cudaMemsetAsync(d_cnt + 5, 0, sizeof(int32_t), st));
    k_leaves<<<blocks(total, 256), 256, 0, st>>>(N, total, static_cast<int32_t>(n), d_refs, d_sorted, d_cnt + 5);
    k_tris_out<<<blocks(n, 256), 256, 0, st>>>(d_idx, d_mesh, n, d_sorted, d_tris);
    GB_CHECK(cudaMemsetAsync(d_arrive, 0, sizeof(int32_t) * total, st));
    k_sizes<<<blocks(total, 256), 256, 0, st>>>(N, total, d_size, d_arrive);
    GB_CHECK(cudaGetLastError());
    int rounds = 1;
    while ((int64_t(1) << rounds) < total) ++rounds;
    auto path_sums = [&](int64_t*& val, int32_t*& anc) -> cudaError_t {
        for (int r = 0; r <= rounds; ++r) {
            k_jump_sum<<<blocks(total, 256), 256, 0, st>>>(total, anc, val, d_anc2, d_val2);
            std::swap(anc, d_anc2);
            std::swap(val, d_val2);
        }
        return cudaGetLastError();
    };
    out.n_nodes = total;
    if (in.layout == 1) {
        // walk positions of internal nodes (for the swaps), then pre-order with swapped children
        int32_t n_internal = (total - 1) / 2;
        std::vector<int32_t> draws(std::max(n_internal, 1), 4);
        if (in.swap_children) {
            std::mt19937 rng(in.swap_seed);
            std::uniform_int_distribution<std::mt19937::result_type> dist(1, 4);
            for (int32_t i = 0; i < n_internal; ++i) draws[i] = static_cast<int32_t>(dist(rng));
        }
        int32_t* d_draws = B.draws;
        int32_t* d_first = B.first;
        int64_t* d_walk = B.walk;
        GB_CHECK(cudaMemcpyAsync(d_draws, draws.data(), sizeof(int32_t) * draws.size(), cudaMemcpyHostToDevice, st));
        int64_t* val = d_val;
        int32_t* anc = d_anc;
        k_walk_val<<<blocks(total, 256), 256, 0, st>>>(N, total, d_size, val, anc);
        GB_CHECK(path_sums(val, anc));
        GB_CHECK(cudaMemcpyAsync(d_walk, val, sizeof(int64_t) * total, cudaMemcpyDeviceToDevice, st));
        k_pre_val<<<blocks(total, 256), 256, 0, st>>>(N, total, d_size, d_walk, d_draws, in.swap_children ? 1 : 0,
                                                      val, anc, d_first);
        k_pre_val2<<<blocks(total, 256), 256, 0, st>>>(N, total, d_size, d_first, val);
        GB_CHECK(path_sums(val, anc));
        k_stackless_out<<<blocks(total, 256), 256, 0, st>>>(N, total, static_cast<int32_t>(n), in.tri_offset, val,
                                                            d_size, d_F);
        out.n_nodes_used = total;
        out.nodes.resize(static_cast<size_t>(total) * 8);
    } else {
        GB_CHECK(cudaMemsetAsync(d_F, 0, sizeof(float) * 16 * static_cast<int64_t>(total), st));
        int32_t* d_bfs = B.bfs;
        int32_t* d_lvl = B.lvl;
        int32_t* d_lvl2 = B.lvl2;
        uint32_t* d_flag = B.flag;
        const int32_t zero = 0;
        GB_CHECK(cudaMemcpyAsync(d_lvl, &zero, sizeof(int32_t), cudaMemcpyHostToDevice, st));
        int32_t count = 1, bfs_base = 0;
        for (int guard = 0; count > 0 && guard <= total; ++guard) {
            k_bfs_flags<<<blocks(count, 256), 256, 0, st>>>(N, d_lvl, count, d_flag);
            GB_CHECK(scan_u32(d_flag, count, d_P, d_sums, st));
            uint32_t internal = 0;
            GB_CHECK(cudaMemcpyAsync(&internal, d_P + count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            k_bfs_expand<<<blocks(count, 256), 256, 0, st>>>(N, d_lvl, count, d_P, bfs_base, d_bfs, d_lvl2);
            GB_CHECK(cudaStreamSynchronize(st));
            bfs_base += static_cast<int32_t>(internal);
            count = 2 * static_cast<int32_t>(internal);
            std::swap(d_lvl, d_lvl2);
        }
        k_stack_out<<<blocks(total, 256), 256, 0, st>>>(N, total, static_cast<int32_t>(n), in.tri_offset, d_bfs, d_F);
        out.n_nodes_used = bfs_base;
        out.nodes.resize(static_cast<size_t>(total) * 16);
    }
    GB_CHECK(cudaGetLastError());
    out.tris.resize(static_cast<size_t>(n) * 4);
    int32_t leaves = 0;
    GB_CHECK(cudaMemcpyAsync(out.nodes.data(), d_F, sizeof(float) * out.nodes.size(), cudaMemcpyDeviceToHost, st));
    GB_CHECK(cudaMemcpyAsync(out.tris.data(), d_tris, sizeof(int32_t) * 4 * n, cudaMemcpyDeviceToHost, st));
    GB_CHECK(cudaMemcpyAsync(&leaves, d_cnt + 5, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GB_CHECK(cudaStreamSynchronize(st));
#undef GB_CHECK
    out.leaf_count = leaves;
    out.max_depth = 0;
    out.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return RQ_OK;
}

}  // namespace rq
