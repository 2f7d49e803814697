// Differentiable depth + Lambert rendering: forward pass with a tape, closed-form adjoint per hit,
// deterministic reduction to vertices, and the BVH refit used after vertex updates.
//
// Derivatives (A, B, C the hit triangle's vertices, n = (B - A) x (C - A), d the ray direction,
// (wa, wb, wc) the barycentric weights of the hit, m = -sun_dir, s = -1 when dot(n, d) > 0 else 1):
//   t  = dot(n, A - o) / dot(n, d)            dt/dV_k = w_k n / dot(n, d)
//   f  = s dot(n, m) / |n|                    df/dV_k = E_k x g,  g = s (m - (n^.m) n^) / |n|
//   with E_A = B - C, E_B = C - A, E_C = A - B (dn = dV x E_k) and radiance = c lit max(f, 0).
// Reduction: per-pixel contributions are keyed by triangle, stably radix-sorted (pixel order is
// kept inside each triangle), and every vertex sums its triangles' segments in the fixed order of a
// vertex -> (triangle, corner) list.  Integer atomics build histograms only; no float atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "rq_bvh8_walk.cuh"
#include "rq_objects.h"
#include "rq_strict.cuh"

struct rq_tape {
    rq_ctx* ctx = nullptr;
    const rq_scene* sc = nullptr;
    const rq_ray* rays = nullptr;
    int64_t n = 0;
    rq_diff_params p{};
    float4* d_hits = nullptr;  // 2 x float4 per pixel: (t, wa, wb, wc), (tri bits, lit, 0, 0)
    float2* d_gimg = nullptr;  // dloss/d(depth, radiance)
    int64_t bytes = 0;
};

namespace rq {
namespace {

using strict::f3;

constexpr int kTile = 2048;  // radix sort elements per block (256 threads x 8)

struct DiffArgs {
    f3 m;  // -sun_dir
    float c;  // albedo * sun_color
    float w_depth, w_rad;
    int shadow;
    float shadow_offset;
    int bvh8;  // trace the BVH8q (same hits as the strict BVH2 walk)
};

DiffArgs to_args(const rq_diff_params& p) {
    DiffArgs a;
    a.m = {-p.sun_dir[0], -p.sun_dir[1], -p.sun_dir[2]};
    a.c = p.albedo * p.sun_color;
    a.w_depth = p.w_depth;
    a.w_rad = p.w_radiance;
    a.shadow = p.shadow_rays;
    a.shadow_offset = p.shadow_offset;
    a.bvh8 = p.layout == RQ_LAYOUT_BVH8Q ? 1 : 0;
    return a;
}

__device__ __forceinline__ f3 fsub(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 fcross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Forward: strict closest hit, geometric-normal Lambert, optional strict any-hit shadow ray; on the
// BVH8q (kBvh8) the walks give the same hits and occlusion (strict leaf test, conservative boxes).
template <bool kBvh8>
__global__ void k_diff_fwd(SceneView s, const rq_ray* __restrict__ rays, int64_t n,
                           const float2* __restrict__ target, DiffArgs a, float2* __restrict__ image,
                           float4* __restrict__ hits, float2* __restrict__ gimg,
                           float* __restrict__ loss_pp, unsigned* status_out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * i;
    const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    rq_hit h;
    int32_t tests = 0, visits = 0;
    unsigned status = 0;
    if (kBvh8) {
        bool occ;
        bvh8_ray<false>(s, r0, r1, 0, h, occ, visits, tests, status);
    } else {
        strict::scene_closest<false, true>(s, r0, r1, 0, h, tests);
    }
    float depth = 0.0f, rad = 0.0f, lit = 0.0f;
    float2 g = make_float2(0.0f, 0.0f);
    float l = 0.0f;
    if (h.t > 0.0f) {
        const int4 tr = __ldg(s.tris + h.tri);
        const f3 A = strict::vpos(s, tr.x), B = strict::vpos(s, tr.y), C = strict::vpos(s, tr.z);
        const f3 d = strict::xyz(r1);
        f3 nrm = fcross(fsub(B, A), fsub(C, A));
        const float ln = sqrtf(fdot(nrm, nrm));
        f3 N = {nrm.x / ln, nrm.y / ln, nrm.z / ln};
        if (fdot(N, d) > 0.0f) N = {-N.x, -N.y, -N.z};
        const float f = fdot(N, a.m);
        lit = 1.0f;
        if (a.shadow && f > 0.0f) {
            const f3 o = strict::xyz(r0);
            const f3 P = {o.x + d.x * h.t, o.y + d.y * h.t, o.z + d.z * h.t};
            const float4 s0 = make_float4(P.x + N.x * a.shadow_offset, P.y + N.y * a.shadow_offset,
                                          P.z + N.z * a.shadow_offset, 0.0f);
            const float4 s1 = make_float4(a.m.x, a.m.y, a.m.z, 1000000.0f);
            int32_t it = 0, te = 0;
            if (kBvh8) {
                rq_hit hs;
                bool occ = false;
                bvh8_ray<true>(s, s0, s1, 0, hs, occ, it, te, status);
                lit = occ ? 0.0f : 1.0f;
            } else {
                lit = strict::scene_any<false>(s, s0, s1, it, te) ? 0.0f : 1.0f;
            }
        }
        depth = h.t;
        rad = a.c * lit * fmaxf(f, 0.0f);
        const float2 T = target[i];
        const float ed = depth - T.x, er = rad - T.y;
        g = make_float2(2.0f * a.w_depth * ed, 2.0f * a.w_rad * er);
        l = a.w_depth * ed * ed + a.w_rad * er * er;
    }
    image[i] = make_float2(depth, rad);
    gimg[i] = g;
    loss_pp[i] = l;
    if (hits) {
        hits[2 * i] = make_float4(h.t, h.u, h.v, h.w);
        hits[2 * i + 1] = make_float4(__int_as_float(h.t > 0.0f ? h.tri : -1), lit, 0.0f, 0.0f);
    }
    if (status) atomicOr(status_out, status);
}

// Deterministic sum: each block sums a contiguous range in a fixed tree order.
__global__ void k_sum_blocks(const float* __restrict__ x, int64_t n, float* __restrict__ out) {
    __shared__ float sh[256];
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = static_cast<int64_t>(blockIdx.x) * per, b1 = b0 + per < n ? b0 + per : n;
    float acc = 0.0f;
    for (int64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) acc += x[k];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// Per-pixel gradient contributions to the hit triangle's corners (9 floats) + sort key.
__global__ void k_adj_pixel(SceneView s, const rq_ray* __restrict__ rays, int64_t n,
                            const float4* __restrict__ hits, const float2* __restrict__ gimg,
                            DiffArgs a, int32_t miss_key, float* __restrict__ contrib,
                            uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 h0 = hits[2 * i], h1 = hits[2 * i + 1];
    const int32_t tri = __float_as_int(h1.x);
    vals[i] = static_cast<uint32_t>(i);
    float* c = contrib + 9 * i;
    if (tri < 0) {
        keys[i] = static_cast<uint32_t>(miss_key);
        for (int k = 0; k < 9; ++k) c[k] = 0.0f;
        return;
    }
    keys[i] = static_cast<uint32_t>(tri);
    const int4 tr = __ldg(s.tris + tri);
    const f3 A = strict::vpos(s, tr.x), B = strict::vpos(s, tr.y), C = strict::vpos(s, tr.z);
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * i;
    const f3 d = strict::xyz(__ldg(pr + 1));
    const f3 nrm = fcross(fsub(B, A), fsub(C, A));
    const float ndotd = fdot(nrm, d);
    const float2 g = gimg[i];
    const float kt = g.x / ndotd;
    const float w[3] = {h0.y, h0.z, h0.w};
    f3 out[3];
    for (int k = 0; k < 3; ++k) out[k] = {kt * w[k] * nrm.x, kt * w[k] * nrm.y, kt * w[k] * nrm.z};
    const float ln = sqrtf(fdot(nrm, nrm));
    const f3 nh = {nrm.x / ln, nrm.y / ln, nrm.z / ln};
    const float sgn = ndotd > 0.0f ? -1.0f : 1.0f;
    const float f = sgn * fdot(nh, a.m);
    const float lit = h1.y;
    if (g.y != 0.0f && lit > 0.0f && f > 0.0f) {
        const float nm = fdot(nh, a.m);
        const float sc = sgn / ln;
        const f3 gg = {sc * (a.m.x - nm * nh.x), sc * (a.m.y - nm * nh.y), sc * (a.m.z - nm * nh.z)};
        const float kr = g.y * a.c * lit;
        const f3 E[3] = {fsub(B, C), fsub(C, A), fsub(A, B)};
        for (int k = 0; k < 3; ++k) {
            const f3 x = fcross(E[k], gg);
            out[k] = {out[k].x + kr * x.x, out[k].y + kr * x.y, out[k].z + kr * x.z};
        }
    }
    for (int k = 0; k < 3; ++k) {
        c[3 * k] = out[k].x;
        c[3 * k + 1] = out[k].y;
        c[3 * k + 2] = out[k].z;
    }
}

// ---- stable LSD radix sort of (key, value) pairs, 8 bits per pass -----------------------------

__global__ void __launch_bounds__(256) k_radix_hist(const uint32_t* __restrict__ keys, int64_t n,
                                                    int shift, uint32_t* __restrict__ hist, int nb) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kTile;
    for (int c = 0; c < kTile / 256; ++c) {
        const int64_t idx = base + c * 256 + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[static_cast<int64_t>(threadIdx.x) * nb + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m counts in one block (fixed order).
__global__ void __launch_bounds__(1024) k_scan_excl(uint32_t* __restrict__ x, int64_t m) {
    __shared__ uint32_t part[1024];
    const int64_t per = (m + 1023) / 1024;
    const int64_t b0 = threadIdx.x * per, b1 = b0 + per < m ? b0 + per : m;
    uint32_t s = 0;
    for (int64_t k = b0; k < b1; ++k) s += x[k];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int t = 0; t < 1024; ++t) {
            const uint32_t v = part[t];
            part[t] = run;
            run += v;
        }
    }
    __syncthreads();
    uint32_t run = part[threadIdx.x];
    for (int64_t k = b0; k < b1; ++k) {
        const uint32_t v = x[k];
        x[k] = run;
        run += v;
    }
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__global__ void __launch_bounds__(256) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin,
                                                       uint32_t* __restrict__ kout,
                                                       uint32_t* __restrict__ vout, int64_t n,
                                                       int shift, const uint32_t* __restrict__ off,
                                                       int nb) {
    __shared__ uint32_t running[256];
    __shared__ uint16_t wcount[8][256];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    running[threadIdx.x] = off[static_cast<int64_t>(threadIdx.x) * nb + blockIdx.x];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kTile;
    for (int c = 0; c < kTile / 256; ++c) {
        for (int w = 0; w < 8; ++w) wcount[w][threadIdx.x] = 0;
        __syncthreads();
        const int64_t idx = base + c * 256 + threadIdx.x;
        const bool valid = idx < n;
        const uint32_t key = valid ? kin[idx] : 0u;
        const uint32_t val = valid ? vin[idx] : 0u;
        const uint32_t digit = (key >> shift) & 0xFFu;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, valid ? digit : 256u + lane);
        const unsigned wrank = __popc(peers & lanemask_lt());
        if (valid && wrank == 0) wcount[warp][digit] = static_cast<uint16_t>(__popc(peers));
        __syncthreads();
        if (valid) {
            uint32_t r = running[digit] + wrank;
            for (unsigned w = 0; w < warp; ++w) r += wcount[w][digit];
            kout[r] = key;
            vout[r] = val;
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < 8; ++w) add += wcount[w][threadIdx.x];
        running[threadIdx.x] += add;
        __syncthreads();
    }
}

__global__ void k_seg_bounds(const uint32_t* __restrict__ keys, int64_t n, uint32_t n_keys,
                             uint32_t* __restrict__ start, uint32_t* __restrict__ end) {
    const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = keys[k];
    if (key >= n_keys) return;
    if (k == 0 || keys[k - 1] != key) start[key] = static_cast<uint32_t>(k);
    if (k == n - 1 || keys[k + 1] != key) end[key] = static_cast<uint32_t>(k + 1);
}

// Per vertex: sum of its corners' contributions, triangles in list order, pixels in sort order.
__global__ void k_vertex_gather(int64_t n_verts, const int32_t* __restrict__ adj_off,
                                const int32_t* __restrict__ adj, const uint32_t* __restrict__ start,
                                const uint32_t* __restrict__ end, const uint32_t* __restrict__ pix,
                                const float* __restrict__ contrib, float* __restrict__ grad) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= n_verts) return;
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    for (int32_t e = adj_off[v]; e < adj_off[v + 1]; ++e) {
        const int32_t t = adj[e] / 3, corner = adj[e] % 3;
        for (uint32_t k = start[t]; k < end[t]; ++k) {
            const float* c = contrib + 9 * static_cast<int64_t>(pix[k]) + 3 * corner;
            gx += c[0];
            gy += c[1];
            gz += c[2];
        }
    }
    grad[3 * v] = gx;
    grad[3 * v + 1] = gy;
    grad[3 * v + 2] = gz;
}

// ---- positions and refit -----------------------------------------------------------------

__global__ void k_set_positions(float4* __restrict__ verts, const float* __restrict__ xyz, int64_t n) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= n) return;
    float4 p = verts[2 * v];
    p.x = xyz[3 * v];
    p.y = xyz[3 * v + 1];
    p.z = xyz[3 * v + 2];
    verts[2 * v] = p;
}

// One level of a stack-layout BVH2: recompute both child boxes of each node (leaf: its triangles'
// vertices; internal: the union of the child node's two boxes, refitted one level deeper).
__global__ void k_refit_level(float4* __restrict__ nodes, const int4* __restrict__ tris,
                              const float4* __restrict__ verts, const int2* __restrict__ level,
                              int64_t count) {
    const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int2 e = level[k];  // (node, object node offset)
    float4* nd = nodes + 4 * static_cast<int64_t>(e.x);
    for (int side = 0; side < 2; ++side) {
        float4 mn = nd[2 * side], mx = nd[2 * side + 1];
        const int32_t kind = __float_as_int(mn.w);
        float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        if (kind != -1) {
            const int32_t st = kind >> 4, len = kind & 0xF;
            for (int32_t t = st; t < st + len; ++t) {
                const int4 tr = tris[t];
                const int32_t vi[3] = {tr.x, tr.y, tr.z};
                for (int q = 0; q < 3; ++q) {
                    const float4 p = verts[2 * static_cast<int64_t>(vi[q])];
                    lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
                    hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
                }
            }
            if (len == 0) continue;
        } else {
            const float4* cn = nodes + 4 * static_cast<int64_t>(__float_as_int(mx.w) + e.y);
            const float4 a0 = cn[0], a1 = cn[1], b0 = cn[2], b1 = cn[3];
            lo[0] = fminf(a0.x, b0.x); lo[1] = fminf(a0.y, b0.y); lo[2] = fminf(a0.z, b0.z);
            hi[0] = fmaxf(a1.x, b1.x); hi[1] = fmaxf(a1.y, b1.y); hi[2] = fmaxf(a1.z, b1.z);
        }
        mn.x = lo[0]; mn.y = lo[1]; mn.z = lo[2];
        mx.x = hi[0]; mx.y = hi[1]; mx.z = hi[2];
        nd[2 * side] = mn;
        nd[2 * side + 1] = mx;
    }
}

inline unsigned grid(int64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

// Refit plan (levels bottom-up) and vertex adjacency, built once per scene on the host.
rq_status prepare_scene(rq_ctx* ctx, rq_scene* sc) {
    if (sc->layout != RQ_LAYOUT_BVH2_STACK)
        return fail(ctx, RQ_ENOTSUP, "refit and adjoint need a stack-layout scene");
    if (!sc->refit_ready) {
        std::vector<std::vector<std::pair<int32_t, int32_t>>> levels;
        std::vector<std::pair<int32_t, int32_t>> seen;
        for (const rq_entity& e : sc->h_ents) {
            const std::pair<int32_t, int32_t> r{e.node_offset, e.node_count};
            if (std::find(seen.begin(), seen.end(), r) != seen.end()) continue;
            seen.push_back(r);
            std::vector<std::pair<int32_t, int32_t>> cur{{0, 0}};  // (relative node, depth)
            std::vector<uint8_t> visited(e.node_count, 0);
            while (!cur.empty()) {
                const auto [j, dpt] = cur.back();
                cur.pop_back();
                if (j < 0 || j >= e.node_count || visited[j])
                    return fail(ctx, RQ_EINVAL, "BVH is not a tree");
                visited[j] = 1;
                if (static_cast<int>(levels.size()) <= dpt) levels.resize(dpt + 1);
                levels[dpt].push_back({e.node_offset + j, e.node_offset});
                const float* nd = sc->h_nodes.data() + static_cast<int64_t>(e.node_offset + j) * 16;
                for (int s = 0; s < 2; ++s) {
                    int32_t kind, link;
                    std::memcpy(&kind, nd + s * 8 + 3, 4);
                    std::memcpy(&link, nd + s * 8 + 7, 4);
                    if (kind == -1) cur.push_back({link, dpt + 1});
                }
            }
        }
        std::vector<int2> flat;
        sc->refit_level_off.assign(1, 0);
        for (int L = static_cast<int>(levels.size()) - 1; L >= 0; --L) {
            for (const auto& x : levels[L]) flat.push_back(make_int2(x.first, x.second));
            sc->refit_level_off.push_back(static_cast<int64_t>(flat.size()));
        }
        if (sc->d_refit) cudaFree(sc->d_refit);
        sc->d_refit = nullptr;
        if (cudaMalloc(&sc->d_refit, sizeof(int2) * std::max<size_t>(1, flat.size())) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "refit plan allocation failed");
        RQ_CUDA(ctx, cudaMemcpy(sc->d_refit, flat.data(), sizeof(int2) * flat.size(), cudaMemcpyHostToDevice));
        sc->refit_ready = true;
    }
    if (!sc->adj_ready) {
        const int64_t nv = sc->n_verts, nt = sc->n_tris;
        std::vector<int32_t> off(nv + 1, 0), adj(3 * nt);
        for (int64_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k) ++off[sc->h_tris[4 * t + k] + 1];
        for (int64_t v = 0; v < nv; ++v) off[v + 1] += off[v];
        std::vector<int32_t> fill(off.begin(), off.end() - 1);
        for (int64_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k) adj[fill[sc->h_tris[4 * t + k]]++] = static_cast<int32_t>(3 * t + k);
        if (sc->d_adj_off) cudaFree(sc->d_adj_off);
        if (sc->d_adj) cudaFree(sc->d_adj);
        sc->d_adj_off = sc->d_adj = nullptr;
        if (cudaMalloc(&sc->d_adj_off, sizeof(int32_t) * (nv + 1)) != cudaSuccess ||
            cudaMalloc(&sc->d_adj, sizeof(int32_t) * std::max<int64_t>(1, 3 * nt)) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "adjacency allocation failed");
        RQ_CUDA(ctx, cudaMemcpy(sc->d_adj_off, off.data(), sizeof(int32_t) * (nv + 1), cudaMemcpyHostToDevice));
        RQ_CUDA(ctx, cudaMemcpy(sc->d_adj, adj.data(), sizeof(int32_t) * 3 * nt, cudaMemcpyHostToDevice));
        sc->adj_ready = true;
    }
    return RQ_OK;
}

rq_status check_diff(rq_ctx* ctx, const rq_scene* sc, const rq_diff_params* p) {
    if (!p) return fail(ctx, RQ_EINVAL, "NULL diff params");
    if (!sc->view.all_identity) return fail(ctx, RQ_ENOTSUP, "the adjoint needs identity entities");
    if (p->layout != 0 && p->layout != RQ_LAYOUT_BVH8Q && p->layout != sc->layout)
        return fail(ctx, RQ_EINVAL, "diff params: layout must be 0, the scene's BVH2 layout or RQ_LAYOUT_BVH8Q");
    if (p->layout == RQ_LAYOUT_BVH8Q && !sc->bvh8)
        return fail(ctx, RQ_ENOTSUP, "BVH8 not built: call rq_scene_build_bvh8");
    if (sc->n_tris >= (int64_t(1) << 30)) return fail(ctx, RQ_EINVAL, "too many triangles");
    return RQ_OK;
}

rq_status forward(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays, int64_t n, const float* target,
                  const DiffArgs& a, float* image, float4* hits, float2* gimg, double* loss,
                  cudaStream_t st) {
    void* d_lpp = nullptr;
    void* d_part = nullptr;
    rq_status s;
    if ((s = scratch(ctx, rq::kSlotLossPerPixel, sizeof(float) * n, &d_lpp)) != RQ_OK ||
        (s = scratch(ctx, rq::kSlotLossPartials, sizeof(float) * 256, &d_part)) != RQ_OK)
        return s;
    if (a.bvh8)
        k_diff_fwd<true><<<grid(n, 128), 128, 0, st>>>(sc->view, rays, n, reinterpret_cast<const float2*>(target),
                                                        a, reinterpret_cast<float2*>(image), hits, gimg,
                                                        static_cast<float*>(d_lpp), status_word(ctx));
    else
        k_diff_fwd<false><<<grid(n, 128), 128, 0, st>>>(sc->view, rays, n, reinterpret_cast<const float2*>(target),
                                                         a, reinterpret_cast<float2*>(image), hits, gimg,
                                                         static_cast<float*>(d_lpp), status_word(ctx));
    RQ_CUDA(ctx, cudaGetLastError());
    if (loss) {
        k_sum_blocks<<<256, 256, 0, st>>>(static_cast<float*>(d_lpp), n, static_cast<float*>(d_part));
        float part[256];
        RQ_CUDA(ctx, cudaMemcpyAsync(part, d_part, sizeof(part), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
        double tot = 0.0;
        for (int b = 0; b < 256; ++b) tot += part[b];
        *loss = tot;
    }
    return RQ_OK;
}

}  // namespace
}  // namespace rq

using rq::fail;

extern "C" {

rq_status rq_scene_update_positions(rq_scene* sc, const float* xyz, void* stream) {
    if (!sc || !xyz) return fail(sc ? sc->ctx : nullptr, RQ_EINVAL, "NULL argument");
    rq_ctx* ctx = sc->ctx;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    rq_status s = rq::prepare_scene(ctx, sc);
    if (s != RQ_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rq::k_set_positions<<<rq::grid(sc->n_verts, 256), 256, 0, st>>>(sc->d_verts, xyz, sc->n_verts);
    RQ_CUDA(ctx, cudaGetLastError());
    for (size_t L = 0; L + 1 < sc->refit_level_off.size(); ++L) {
        const int64_t b = sc->refit_level_off[L], e = sc->refit_level_off[L + 1];
        if (e > b)
            rq::k_refit_level<<<rq::grid(e - b, 128), 128, 0, st>>>(sc->d_nodes, sc->d_tris, sc->d_verts,
                                                                    sc->d_refit + b, e - b);
    }
    RQ_CUDA(ctx, rq::launch_tri_fast(sc->d_tris, sc->n_tris, sc->d_verts, sc->d_tri_fast, st));
    RQ_CUDA(ctx, cudaGetLastError());
    if ((s = rq::refit_bvh8(sc, st)) != RQ_OK) return s;  // quantised boxes refitted, topology kept
    sc->view.tlas = nullptr;   // the top-level boxes are not refitted: every entity is walked until
                               // the entities or the BVH8 are set again
    sc->host_stale = true;     // host copies of vertices / nodes are refreshed on demand
    return RQ_OK;
}

rq_status rq_fwd(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays, int64_t n, const float* target2,
                 const rq_diff_params* p, float* image2, double* loss, rq_tape** tape, void* stream) {
    if (!ctx || !sc || !tape || n <= 0 || !rays || !target2 || !image2)
        return fail(ctx, RQ_EINVAL, "bad arguments");
    *tape = nullptr;
    rq_status s = rq::check_diff(ctx, sc, p);
    if (s != RQ_OK) return s;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    auto* t = new (std::nothrow) rq_tape;
    if (!t) return fail(ctx, RQ_ENOMEM, "tape allocation failed");
    t->ctx = ctx;
    t->sc = sc;
    t->rays = rays;
    t->n = n;
    t->p = *p;
    if (cudaMalloc(&t->d_gimg, sizeof(float2) * n) != cudaSuccess ||
        (!p->recompute && cudaMalloc(&t->d_hits, 2 * sizeof(float4) * n) != cudaSuccess)) {
        rq_tape_free(t);
        return fail(ctx, RQ_ENOMEM, "tape buffers");
    }
    t->bytes = static_cast<int64_t>(sizeof(float2) * n + (p->recompute ? 0 : 2 * sizeof(float4) * n));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void* hits = t->d_hits;
    if (p->recompute && (s = rq::scratch(ctx, rq::kSlotTapeHits, 2 * sizeof(float4) * n, &hits)) != RQ_OK) {
        rq_tape_free(t);
        return s;
    }
    s = rq::forward(ctx, sc, rays, n, target2, rq::to_args(*p), image2, static_cast<float4*>(hits),
                    t->d_gimg, loss, st);
    if (s != RQ_OK) {
        rq_tape_free(t);
        return s;
    }
    *tape = t;
    return RQ_OK;
}

rq_status rq_bwd(rq_ctx* ctx, rq_tape* t, float* grad, void* stream) {
    if (!ctx || !t || !grad) return fail(ctx, RQ_EINVAL, "bad arguments");
    rq_scene* sc = const_cast<rq_scene*>(t->sc);
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    rq_status s = rq::prepare_scene(ctx, sc);
    if (s != RQ_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = t->n;
    const rq::DiffArgs a = rq::to_args(t->p);
    float4* hits = t->d_hits;
    if (t->p.recompute) {  // re-trace: hits only (image and dloss/dimage are already known)
        void* h = nullptr;
        void *img = nullptr, *g2 = nullptr, *tg = nullptr;
        if ((s = rq::scratch(ctx, rq::kSlotTapeHits, 2 * sizeof(float4) * n, &h)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotTapeImage, sizeof(float2) * n, &img)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotTapeGrad, sizeof(float2) * n, &g2)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotTapeTarget, sizeof(float2) * n, &tg)) != RQ_OK)
            return s;
        RQ_CUDA(ctx, cudaMemsetAsync(tg, 0, sizeof(float2) * n, st));
        if ((s = rq::forward(ctx, sc, t->rays, n, static_cast<float*>(tg), a, static_cast<float*>(img),
                             static_cast<float4*>(h), static_cast<float2*>(g2), nullptr, st)) != RQ_OK)
            return s;
        hits = static_cast<float4*>(h);
    }
    const int64_t nb = (n + rq::kTile - 1) / rq::kTile;
    void *contrib, *ka, *va, *kb, *vb, *hist, *segs, *sege;
    if ((s = rq::scratch(ctx, rq::kSlotAdjContrib, 9 * sizeof(float) * n, &contrib)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotAdjKeysA, 4 * n, &ka)) != RQ_OK || (s = rq::scratch(ctx, rq::kSlotAdjValsA, 4 * n, &va)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotAdjKeysB, 4 * n, &kb)) != RQ_OK || (s = rq::scratch(ctx, rq::kSlotAdjValsB, 4 * n, &vb)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotAdjHist, 4 * 256 * nb, &hist)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotAdjSegStart, 4 * (sc->n_tris + 1), &segs)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotAdjSegEnd, 4 * (sc->n_tris + 1), &sege)) != RQ_OK)
        return s;
    const int32_t miss_key = static_cast<int32_t>(sc->n_tris);
    rq::k_adj_pixel<<<rq::grid(n, 128), 128, 0, st>>>(sc->view, t->rays, n, hits, t->d_gimg, a, miss_key,
                                                       static_cast<float*>(contrib),
                                                       static_cast<uint32_t*>(ka), static_cast<uint32_t*>(va));
    RQ_CUDA(ctx, cudaGetLastError());
    int bits = 1;
    while ((int64_t(1) << bits) <= miss_key) ++bits;
    uint32_t *kin = static_cast<uint32_t*>(ka), *vin = static_cast<uint32_t*>(va);
    uint32_t *kout = static_cast<uint32_t*>(kb), *vout = static_cast<uint32_t*>(vb);
    for (int shift = 0; shift < bits; shift += 8) {
        rq::k_radix_hist<<<static_cast<unsigned>(nb), 256, 0, st>>>(kin, n, shift,
                                                                    static_cast<uint32_t*>(hist),
                                                                    static_cast<int>(nb));
        rq::k_scan_excl<<<1, 1024, 0, st>>>(static_cast<uint32_t*>(hist), 256 * nb);
        rq::k_radix_scatter<<<static_cast<unsigned>(nb), 256, 0, st>>>(
            kin, vin, kout, vout, n, shift, static_cast<uint32_t*>(hist), static_cast<int>(nb));
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    RQ_CUDA(ctx, cudaMemsetAsync(segs, 0, 4 * (sc->n_tris + 1), st));
    RQ_CUDA(ctx, cudaMemsetAsync(sege, 0, 4 * (sc->n_tris + 1), st));
    rq::k_seg_bounds<<<rq::grid(n, 256), 256, 0, st>>>(kin, n, static_cast<uint32_t>(sc->n_tris),
                                                       static_cast<uint32_t*>(segs),
                                                       static_cast<uint32_t*>(sege));
    rq::k_vertex_gather<<<rq::grid(sc->n_verts, 128), 128, 0, st>>>(
        sc->n_verts, sc->d_adj_off, sc->d_adj, static_cast<uint32_t*>(segs), static_cast<uint32_t*>(sege),
        vin, static_cast<float*>(contrib), grad);
    RQ_CUDA(ctx, cudaGetLastError());
    return RQ_OK;
}

rq_status rq_tape_free(rq_tape* t) {
    if (!t) return RQ_OK;
    if (t->ctx) cudaSetDevice(t->ctx->device);
    if (t->d_hits) cudaFree(t->d_hits);
    if (t->d_gimg) cudaFree(t->d_gimg);
    delete t;
    return RQ_OK;
}

rq_status rq_tape_bytes(const rq_tape* t, int64_t* bytes) {
    if (!t || !bytes) return fail(nullptr, RQ_EINVAL, "NULL argument");
    *bytes = t->bytes;
    return RQ_OK;
}

}  // extern "C"
