// Diffuse-GI / RTAO pass: secondary ray generation, shading and per-pixel accumulation, plus the
// C ABI entry points that drive the whole pass (rq_gi_frame).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "rq_gi.cuh"
#include "rq_persistent.cuh"
#include "rq_objects.h"

namespace rq {
namespace {

using strict::f3;

struct GiArgs {
    int32_t spp;
    uint32_t seed;
    float origin_offset;
    float ray_tmax;
    int32_t normal_mode;
    float shadow_offset;
    f3 sun_dir, sun_color, sky;
    int32_t bounces;
};

// Output pixels of a GI pass: 4 floats, or 4 binary16 values (rq_gi_params.pixel_format, the
// reference's rgba16f output image) each rounded to nearest, ties to even.
struct PixelOut {
    void* base;
    bool half;
    __device__ __forceinline__ void put(int64_t i, float4 v) const {
        if (half) {
            const __half2 lo = __halves2half2(__float2half_rn(v.x), __float2half_rn(v.y));
            const __half2 hi = __halves2half2(__float2half_rn(v.z), __float2half_rn(v.w));
            uint2 w;
            w.x = *reinterpret_cast<const uint32_t*>(&lo);
            w.y = *reinterpret_cast<const uint32_t*>(&hi);
            static_cast<uint2*>(base)[i] = w;
        } else {
            static_cast<float4*>(base)[i] = v;
        }
    }
};

// Origin offset of the bounce rays (HitPosition + iNormal * 0.02, DiffuseTrace.glsl:518).
constexpr float kBounceOffset = 0.02f;
// A bounce that misses sees 2.2 x the skymap (DiffuseTrace.glsl:523), the first bounce 2.0 x
// (:490); the sky parameter holds the first bounce's radiance.
constexpr float kBounceSky = 1.1f;

GiArgs to_args(const rq_gi_params& p) {
    GiArgs a;
    a.spp = p.spp;
    a.seed = p.seed;
    a.origin_offset = p.origin_offset;
    a.ray_tmax = p.ray_tmax;
    a.normal_mode = p.normal_mode;
    a.shadow_offset = p.shadow_offset;
    a.sun_dir = {p.sun_dir[0], p.sun_dir[1], p.sun_dir[2]};
    a.sun_color = {p.sun_color[0], p.sun_color[1], p.sun_color[2]};
    a.sky = {p.sky_color[0], p.sky_color[1], p.sky_color[2]};
    a.bounces = p.bounces;
    return a;
}

__device__ __forceinline__ void put_ray(rq_ray* out, int64_t j, f3 o, float tmin, f3 d, float tmax) {
    float4* p = reinterpret_cast<float4*>(out) + 2 * j;
    p[0] = make_float4(o.x, o.y, o.z, tmin);
    p[1] = make_float4(d.x, d.y, d.z, tmax);
}

__device__ __forceinline__ void get_hit(const rq_hit* hits, int64_t i, float4& a, int4& b) {
    const float4* p = reinterpret_cast<const float4*>(hits) + 2 * i;
    a = __ldg(p);
    const float4 q = __ldg(p + 1);
    b = make_int4(__float_as_int(q.x), __float_as_int(q.y), __float_as_int(q.z), __float_as_int(q.w));
}

// One thread per secondary ray j = i*spp + k (DiffuseTrace.glsl:439-446, 486-488).
__global__ void k_gi_raygen(SceneView s, const rq_ray* __restrict__ prim,
                            const rq_hit* __restrict__ hits, int64_t n, GiArgs a,
                            rq_ray* __restrict__ out, unsigned long long* active) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = n * a.spp;
    bool act = false;
    if (j < total) {
        const int64_t i = j / a.spp;
        float4 h0;
        int4 h1;
        get_hit(hits, i, h0, h1);
        if (h0.x > 0.0f) {
            const float4* pr = reinterpret_cast<const float4*>(prim) + 2 * i;
            const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
            const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
            const f3 P = strict::add(ro, strict::muls(rd, h0.x));
            f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
            if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
            const uint32_t rid = static_cast<uint32_t>(j);
            const float u0 = gi::u01(gi::sample_key(a.seed, rid, 0u));
            const float u1 = gi::u01(gi::sample_key(a.seed, rid, 1u));
            const f3 dir = gi::cos_weighted_hemisphere(N, u0, u1);
            const f3 org = strict::add(P, strict::muls(N, a.origin_offset));
            put_ray(out, j, org, 0.0f, dir, a.ray_tmax);
            act = true;
        } else {
            put_ray(out, j, f3{0.0f, 0.0f, 0.0f}, 0.0f, f3{0.0f, 0.0f, 1.0f}, -1.0f);
        }
    }
    if (active) {
        const unsigned m = __ballot_sync(0xFFFFFFFFu, act);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(active, static_cast<unsigned long long>(__popc(m)));
    }
}

__global__ void k_shadow_raygen(SceneView s, const rq_ray* __restrict__ rays,
                                const rq_hit* __restrict__ hits, int64_t n, GiArgs a,
                                rq_ray* __restrict__ out, unsigned long long* active) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool act = false;
    if (j < n) {
        float4 h0;
        int4 h1;
        get_hit(hits, j, h0, h1);
        const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * j;
        const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
        if (h0.x > 0.0f && r1.w > r0.w) {
            const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
            const f3 P = strict::add(ro, strict::muls(rd, h0.x));
            f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
            if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
            const f3 org = strict::add(P, strict::muls(N, a.shadow_offset));
            put_ray(out, j, org, 0.0f, strict::neg(a.sun_dir), 1000000.0f);
            act = true;
        } else {
            put_ray(out, j, f3{0.0f, 0.0f, 0.0f}, 0.0f, f3{0.0f, 0.0f, 1.0f}, -1.0f);
        }
    }
    if (active) {
        const unsigned m = __ballot_sync(0xFFFFFFFFu, act);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(active, static_cast<unsigned long long>(__popc(m)));
    }
}

// Secondary ray j of the GI pass (same arithmetic as k_gi_raygen); false when the primary missed.
__device__ __forceinline__ bool gi_ray(const SceneView& s, const rq_ray* __restrict__ prim,
                                       const rq_hit* __restrict__ hits, int64_t j, const GiArgs& a,
                                       f3& org, f3& dir) {
    const int64_t i = j / a.spp;
    float4 h0;
    int4 h1;
    get_hit(hits, i, h0, h1);
    if (!(h0.x > 0.0f)) return false;
    const float4* pr = reinterpret_cast<const float4*>(prim) + 2 * i;
    const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
    const f3 P = strict::add(ro, strict::muls(rd, h0.x));
    f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
    if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
    const uint32_t rid = static_cast<uint32_t>(j);
    const float u0 = gi::u01(gi::sample_key(a.seed, rid, 0u));
    const float u1 = gi::u01(gi::sample_key(a.seed, rid, 1u));
    dir = gi::cos_weighted_hemisphere(N, u0, u1);
    org = strict::add(P, strict::muls(N, a.origin_offset));
    return true;
}

__device__ __forceinline__ unsigned octant(const f3& d) {
    return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
}

// Pass 1 of the octant-binned compaction: counts active rays per direction octant.
__global__ void __launch_bounds__(256) k_gi_octant_count(SceneView s, const rq_ray* __restrict__ prim,
                                                         const rq_hit* __restrict__ hits, int64_t n,
                                                         GiArgs a, unsigned long long* counts) {
    __shared__ unsigned c[8];
    if (threadIdx.x < 8) c[threadIdx.x] = 0;
    __syncthreads();
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < n * a.spp) {
        f3 org, dir;
        if (gi_ray(s, prim, hits, j, a, org, dir)) atomicAdd(&c[octant(dir)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 8 && c[threadIdx.x])
        atomicAdd(counts + threadIdx.x, static_cast<unsigned long long>(c[threadIdx.x]));
}

// Pass 2: writes each active ray into its octant's region (regions in octant order, starting at
// the exclusive prefix of the counts; cursors[o] advances per block), with the slot map comp_of.
__global__ void __launch_bounds__(256) k_gi_octant_scatter(
    SceneView s, const rq_ray* __restrict__ prim, const rq_hit* __restrict__ hits, int64_t n, GiArgs a,
    const unsigned long long* counts, unsigned long long* cursors, rq_ray* __restrict__ out,
    int32_t* __restrict__ comp_of, unsigned long long* total) {
    __shared__ unsigned c[8];
    __shared__ unsigned long long base[8];
    if (threadIdx.x < 8) c[threadIdx.x] = 0;
    __syncthreads();
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    f3 org{0.0f, 0.0f, 0.0f}, dir{0.0f, 0.0f, 1.0f};
    bool act = false;
    unsigned o = 0, rank = 0;
    if (j < n * a.spp) {
        act = gi_ray(s, prim, hits, j, a, org, dir);
        if (act) {
            o = octant(dir);
            rank = atomicAdd(&c[o], 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        unsigned long long pre = 0;
        for (unsigned k = 0; k < threadIdx.x; ++k) pre += counts[k];
        base[threadIdx.x] = c[threadIdx.x]
                                ? pre + atomicAdd(cursors + threadIdx.x, static_cast<unsigned long long>(c[threadIdx.x]))
                                : 0ull;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            unsigned long long t = 0;
            for (int k = 0; k < 8; ++k) t += counts[k];
            *total = t;
        }
    }
    __syncthreads();
    if (j < n * a.spp) {
        if (act) {
            const int64_t cidx = static_cast<int64_t>(base[o] + rank);
            put_ray(out, cidx, org, 0.0f, dir, a.ray_tmax);
            comp_of[j] = static_cast<int32_t>(cidx);
        } else {
            comp_of[j] = -1;
        }
    }
}

// Compacting variant of k_gi_raygen: active secondary rays are appended to `out` (block-aggregated
// atomic, so only the order of blocks varies between runs), with comp_of[j] = the compact index
// of slot j's ray (or -1 for an inactive slot).  Results are scattered back by slot, so
// per-pixel sums keep their sample order; only the assignment of rays to threads changes.
__global__ void __launch_bounds__(256) k_gi_raygen_compact(
    SceneView s, const rq_ray* __restrict__ prim, const rq_hit* __restrict__ hits, int64_t n,
    GiArgs a, rq_ray* __restrict__ out, int32_t* __restrict__ comp_of, unsigned long long* count) {
    __shared__ unsigned warp_count[8];
    __shared__ unsigned long long block_base;
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = n * a.spp;
    bool act = false;
    f3 org{0.0f, 0.0f, 0.0f}, dir{0.0f, 0.0f, 1.0f};
    if (j < total) {
        const int64_t i = j / a.spp;
        float4 h0;
        int4 h1;
        get_hit(hits, i, h0, h1);
        if (h0.x > 0.0f) {
            const float4* pr = reinterpret_cast<const float4*>(prim) + 2 * i;
            const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
            const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
            const f3 P = strict::add(ro, strict::muls(rd, h0.x));
            f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
            if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
            const uint32_t rid = static_cast<uint32_t>(j);
            const float u0 = gi::u01(gi::sample_key(a.seed, rid, 0u));
            const float u1 = gi::u01(gi::sample_key(a.seed, rid, 1u));
            dir = gi::cos_weighted_hemisphere(N, u0, u1);
            org = strict::add(P, strict::muls(N, a.origin_offset));
            act = true;
        }
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, act);
    if (lane == 0) warp_count[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned tot = 0;
        for (unsigned w = 0; w < blockDim.x / 32; ++w) {
            const unsigned c = warp_count[w];
            warp_count[w] = tot;
            tot += c;
        }
        block_base = tot ? atomicAdd(count, static_cast<unsigned long long>(tot)) : 0ull;
    }
    __syncthreads();
    if (j < total) {
        if (act) {
            const int64_t c = static_cast<int64_t>(block_base) + warp_count[warp] +
                              __popc(m & ((1u << lane) - 1u));
            put_ray(out, c, org, 0.0f, dir, a.ray_tmax);
            comp_of[j] = static_cast<int32_t>(c);
        } else {
            comp_of[j] = -1;
        }
    }
}

// Whether a pass traces its secondary rays compacted: always without a live count, else when the
// fraction of primary rays with a hit is below the threshold.
__device__ __forceinline__ bool compact_rays(const unsigned long long* live, int64_t n, float compact_below) {
    if (!live) return true;
    return __fdiv_rn(static_cast<float>(*live), static_cast<float>(n)) < compact_below;
}

// Per-pixel form of k_gi_raygen_compact: one thread per primary ray i computes the hit point and
// faced normal once and writes the spp secondary rays of slots j = i*spp + k.  Compaction is
// block-aggregated and pixel-major within the block, the order k_gi_raygen_compact gives, with the
// same slot map; every value is computed with the same functions.  With a live count (the primary
// hits, counted by k_count_live) at or above the compaction threshold the rays stay in place
// instead: slot j holds sample j (an inactive ray for a pixel without a hit), the slot map is the
// identity and *count = n * spp, so the secondary launch covers every slot.
__global__ void __launch_bounds__(256) k_gi_raygen_pixel(
    SceneView s, const rq_ray* __restrict__ prim, const rq_hit* __restrict__ hits, int64_t n,
    GiArgs a, rq_ray* __restrict__ out, int32_t* __restrict__ comp_of, unsigned long long* count,
    int32_t* __restrict__ samp_of, const unsigned long long* __restrict__ live, float compact_below) {
    __shared__ unsigned warp_hits[8];
    __shared__ unsigned long long block_base;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    float4 h0 = make_float4(-1.0f, 0.0f, 0.0f, 0.0f);
    int4 h1 = make_int4(-1, -1, -1, 0);
    if (i < n) get_hit(hits, i, h0, h1);
    const bool hit = i < n && h0.x > 0.0f;
    if (!compact_rays(live, n, compact_below)) {  // in place
        if (i == 0) *count = static_cast<unsigned long long>(n) * a.spp;
        if (i >= n) return;
        if (!hit) {
            for (int k = 0; k < a.spp; ++k) {
                put_ray(out, i * a.spp + k, f3{0.0f, 0.0f, 0.0f}, 0.0f, f3{0.0f, 0.0f, 1.0f}, -1.0f);
                comp_of[i * a.spp + k] = -1;
            }
            return;
        }
        const float4* pr = reinterpret_cast<const float4*>(prim) + 2 * i;
        const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
        const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
        const f3 P = strict::add(ro, strict::muls(rd, h0.x));
        f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
        if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
        const f3 org = strict::add(P, strict::muls(N, a.origin_offset));
        for (int k = 0; k < a.spp; ++k) {
            const int64_t j = i * a.spp + k;
            const uint32_t rid = static_cast<uint32_t>(j);
            const float u0 = gi::u01(gi::sample_key(a.seed, rid, 0u));
            const float u1 = gi::u01(gi::sample_key(a.seed, rid, 1u));
            put_ray(out, j, org, 0.0f, gi::cos_weighted_hemisphere(N, u0, u1), a.ray_tmax);
            comp_of[j] = static_cast<int32_t>(j);
        }
        return;
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, hit);
    if (lane == 0) warp_hits[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned tot = 0;
        for (unsigned w = 0; w < blockDim.x / 32; ++w) {
            const unsigned c = warp_hits[w];
            warp_hits[w] = tot;
            tot += c;
        }
        block_base = tot ? atomicAdd(count, static_cast<unsigned long long>(tot) * a.spp) : 0ull;
    }
    __syncthreads();
    if (i >= n) return;
    if (!hit) {
        for (int k = 0; k < a.spp; ++k) comp_of[i * a.spp + k] = -1;
        return;
    }
    const int64_t c0 = static_cast<int64_t>(block_base) +
                       static_cast<int64_t>(warp_hits[warp] + __popc(m & persist::lanemask_lt())) * a.spp;
    const float4* pr = reinterpret_cast<const float4*>(prim) + 2 * i;
    const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
    const f3 P = strict::add(ro, strict::muls(rd, h0.x));
    f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
    if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
    const f3 org = strict::add(P, strict::muls(N, a.origin_offset));
    for (int k = 0; k < a.spp; ++k) {
        const int64_t j = i * a.spp + k;
        const uint32_t rid = static_cast<uint32_t>(j);
        const float u0 = gi::u01(gi::sample_key(a.seed, rid, 0u));
        const float u1 = gi::u01(gi::sample_key(a.seed, rid, 1u));
        const f3 dir = gi::cos_weighted_hemisphere(N, u0, u1);
        put_ray(out, c0 + k, org, 0.0f, dir, a.ray_tmax);
        comp_of[j] = static_cast<int32_t>(c0 + k);
        if (samp_of) samp_of[c0 + k] = static_cast<int32_t>(j);
    }
}

// Shadow rays for the first *count compact secondary hits.
__global__ void k_shadow_raygen_c(SceneView s, const rq_ray* __restrict__ rays,
                                  const rq_hit* __restrict__ hits, int64_t n_max, GiArgs a,
                                  rq_ray* __restrict__ out, const unsigned long long* count,
                                  unsigned long long* active) {
    const int64_t n = static_cast<int64_t>(*count) < n_max ? static_cast<int64_t>(*count) : n_max;
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool act = false;
    if (j < n) {
        float4 h0;
        int4 h1;
        get_hit(hits, j, h0, h1);
        const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * j;
        const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
        if (h0.x > 0.0f && r1.w > r0.w) {
            const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
            const f3 P = strict::add(ro, strict::muls(rd, h0.x));
            f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
            if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
            const f3 org = strict::add(P, strict::muls(N, a.shadow_offset));
            put_ray(out, j, org, 0.0f, strict::neg(a.sun_dir), 1000000.0f);
            act = true;
        } else {
            put_ray(out, j, f3{0.0f, 0.0f, 0.0f}, 0.0f, f3{0.0f, 0.0f, 1.0f}, -1.0f);
        }
    }
    if (active) {
        const unsigned m = __ballot_sync(0xFFFFFFFFu, act);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(active, static_cast<unsigned long long>(__popc(m)));
    }
}

// Radiance and AO of one secondary hit (GetDirect, DiffuseTrace.glsl:368-372; emissive :491;
// AO :494): h0 = (t, u, v, w), h1 = (tri, mesh, entity), rd the ray direction, l the sun's
// visibility.  A miss returns the sky.
__device__ __forceinline__ float4 shade_one(const SceneView& s, const Materials& mat, const GiArgs& a, const f3 rd,
                                            const float4 h0, const int4 h1, float l) {
    if (!(h0.x > 0.0f)) return make_float4(a.sky.x, a.sky.y, a.sky.z, 1.0f);
    f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
    if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
    const f3 alb = gi::hit_albedo(s, mat, h0, h1);
    const float em = __int_as_float(s.ents[h1.z].data[0]);
    const float ndl = strict::gmin(strict::gmax(strict::dot(N, strict::neg(a.sun_dir)), 0.0f), 1.0f);
    const f3 direct = strict::muls(strict::muls(strict::mul(alb, a.sun_color), l), ndl);
    const f3 rad = strict::add(direct, strict::muls(alb, em));
    const float ao = powf(strict::gmin(strict::gmax(__fdiv_rn(h0.x, 2.4f), 0.0f), 1.0f), 1.23f);
    return make_float4(rad.x, rad.y, rad.z, ao);
}

// Shading per slot from compact rays / hits / visibility (comp_of[j] < 0: inactive slot).
__global__ void k_shade_c(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                          const int32_t* __restrict__ comp_of, int64_t m,
                          const uint8_t* __restrict__ occl, int query, const Materials mat, GiArgs a,
                          float4* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int32_t c = comp_of[j];
    if (c < 0) {
        out[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    if (query == 1) {  // AO: visibility of the compact any-hit ray
        out[j] = make_float4(0.0f, 0.0f, 0.0f, occl[c] ? 0.0f : 1.0f);
        return;
    }
    float4 h0;
    int4 h1;
    get_hit(hits, c, h0, h1);
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * static_cast<int64_t>(c);
    const f3 rd = strict::xyz(__ldg(pr + 1));
    const float l = occl ? (occl[c] ? 0.0f : 1.0f) : 1.0f;
    out[j] = shade_one(s, mat, a, rd, h0, h1, l);
}

// k_shade_c and k_accumulate in one pass, one thread per pixel: the spp samples are shaded with
// shade_one and summed in sample order, so the pixel is bit-identical to the two-kernel form.
__global__ void k_shade_accumulate(SceneView s, const rq_ray* __restrict__ rays,
                                   const rq_hit* __restrict__ hits, const int32_t* __restrict__ comp_of,
                                   int64_t n, const uint8_t* __restrict__ occl, int query,
                                   const Materials mat, GiArgs a,
                                   const PixelOut pixels) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int k = 0; k < a.spp; ++k) {
        const int32_t c = __ldg(comp_of + i * a.spp + k);
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (c >= 0) {
            if (query == 1) {
                v.w = occl[c] ? 0.0f : 1.0f;
            } else {
                float4 h0;
                int4 h1;
                get_hit(hits, c, h0, h1);
                const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * static_cast<int64_t>(c);
                const f3 rd = strict::xyz(__ldg(pr + 1));
                const float l = occl ? (occl[c] ? 0.0f : 1.0f) : 1.0f;
                v = shade_one(s, mat, a, rd, h0, h1, l);
            }
        }
        acc.x = __fadd_rn(acc.x, v.x);
        acc.y = __fadd_rn(acc.y, v.y);
        acc.z = __fadd_rn(acc.z, v.z);
        acc.w = __fadd_rn(acc.w, v.w);
    }
    const float inv = __fdiv_rn(1.0f, static_cast<float>(a.spp));
    pixels.put(i, make_float4(__fmul_rn(acc.x, inv), __fmul_rn(acc.y, inv), __fmul_rn(acc.z, inv),
                              __fmul_rn(acc.w, inv)));
}

// ---- RT second-bounce loop (DiffuseTrace.glsl:502-536), per compact GI slot c ----------------
// rad[c]: the slot's radiance (rgb) and AO (w); thr[c]: the path throughput (rgb), w = 1 while
// the path continues.

// First bounce: the GI hit's shading, and its albedo as the throughput (Throughput = Albedo.xyz).
__global__ void k_bounce_init(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                              const uint8_t* __restrict__ occl, const unsigned long long* count, int64_t n_max,
                              const Materials mat, GiArgs a,
                              float4* __restrict__ rad, float4* __restrict__ thr, float4* __restrict__ bnc) {
    const int64_t n = static_cast<int64_t>(*count) < n_max ? static_cast<int64_t>(*count) : n_max;
    const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
    bnc[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // Bounced = vec3(0.0f) (:499)
    float4 h0;
    int4 h1;
    get_hit(hits, c, h0, h1);
    const f3 rd = strict::xyz(__ldg(reinterpret_cast<const float4*>(rays) + 2 * c + 1));
    const float l = occl ? (occl[c] ? 0.0f : 1.0f) : 1.0f;
    rad[c] = shade_one(s, mat, a, rd, h0, h1, l);
    if (h0.x > 0.0f) {
        const f3 alb = gi::hit_albedo(s, mat, h0, h1);
        thr[c] = make_float4(alb.x, alb.y, alb.z, 1.0f);
    } else {
        thr[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// Bounce b's rays from the previous segment's hits, compacted: segment k of the previous bounce
// belongs to GI slot prev_slot[k] (k itself for the GI segment); the live paths (throughput
// w > 0) get consecutive entries of out / out_slot in warp-aggregated order.  Origin P + N * 0.02,
// a cosine direction about N from sample samp_of[slot], dimensions 2 + 2b and 3 + 2b.
__global__ void k_bounce_raygen(SceneView s, const rq_ray* __restrict__ prev_rays, const rq_hit* __restrict__ prev_hits,
                                const int32_t* __restrict__ prev_slot, const unsigned long long* prev_count,
                                int64_t n_max, const float4* __restrict__ thr, const int32_t* __restrict__ samp_of,
                                GiArgs a, int bounce, rq_ray* __restrict__ out, int32_t* __restrict__ out_slot,
                                unsigned long long* out_count, unsigned long long* active) {
    const int64_t n = static_cast<int64_t>(*prev_count) < n_max ? static_cast<int64_t>(*prev_count) : n_max;
    const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int32_t c = -1;
    bool alive = false;
    if (k < n) {
        c = prev_slot ? prev_slot[k] : static_cast<int32_t>(k);
        alive = thr[c].w > 0.0f;
    }
    const unsigned lane = threadIdx.x & 31u;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, alive);
    unsigned long long base = 0;
    if (lane == 0 && m) {
        base = atomicAdd(out_count, static_cast<unsigned long long>(__popc(m)));
        if (active) atomicAdd(active, static_cast<unsigned long long>(__popc(m)));
    }
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (!alive) return;
    const int64_t j = static_cast<int64_t>(base) + __popc(m & persist::lanemask_lt());
    float4 h0;
    int4 h1;
    get_hit(prev_hits, k, h0, h1);
    const float4* pr = reinterpret_cast<const float4*>(prev_rays) + 2 * k;
    const f3 ro = strict::xyz(__ldg(pr)), rd = strict::xyz(__ldg(pr + 1));
    const f3 P = strict::add(ro, strict::muls(rd, h0.x));
    f3 N = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, a.normal_mode);
    if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
    const uint32_t rid = static_cast<uint32_t>(samp_of[c]);
    const float u0 = gi::u01(gi::sample_key(a.seed, rid, 2u + 2u * bounce));
    const float u1 = gi::u01(gi::sample_key(a.seed, rid, 3u + 2u * bounce));
    const f3 dir = gi::cos_weighted_hemisphere(N, u0, u1);
    put_ray(out, j, strict::add(P, strict::muls(N, kBounceOffset)), 0.0f, dir, a.ray_tmax);
    out_slot[j] = c;
}

// Bounce shading of compact segment k (GI slot slot[k]): Bounced += (GetDirect + emissive) *
// throughput, throughput *= albedo (:524, :530); a miss adds 1.1 x sky x throughput (nothing under
// ref_miss, as the reference) and ends the path.  Bounced joins the slot's radiance once, after the
// last bounce (FinalRadiance += Bounced, :535), in k_gather_accumulate.
__global__ void k_bounce_shade(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                               const uint8_t* __restrict__ occl, const int32_t* __restrict__ slot,
                               const unsigned long long* count, int64_t n_max, const Materials mat, GiArgs a,
                               int ref_miss, float4* __restrict__ bnc, float4* __restrict__ thr,
                               unsigned long long* hit_count) {
    const int64_t n = static_cast<int64_t>(*count) < n_max ? static_cast<int64_t>(*count) : n_max;
    const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool hit = false;
    if (k < n) {
        const int32_t c = slot[k];
        float4 T = thr[c];
        float4 h0;
        int4 h1;
        get_hit(hits, k, h0, h1);
        float4 R = bnc[c];
        if (h0.x > 0.0f) {
            const f3 rd = strict::xyz(__ldg(reinterpret_cast<const float4*>(rays) + 2 * k + 1));
            const float l = occl ? (occl[k] ? 0.0f : 1.0f) : 1.0f;
            const float4 v = shade_one(s, mat, a, rd, h0, h1, l);
            R.x = __fadd_rn(R.x, __fmul_rn(v.x, T.x));
            R.y = __fadd_rn(R.y, __fmul_rn(v.y, T.y));
            R.z = __fadd_rn(R.z, __fmul_rn(v.z, T.z));
            const f3 alb = gi::hit_albedo(s, mat, h0, h1);
            T = make_float4(__fmul_rn(T.x, alb.x), __fmul_rn(T.y, alb.y), __fmul_rn(T.z, alb.z), 1.0f);
            hit = true;
        } else {
            if (!ref_miss) {
                R.x = __fadd_rn(R.x, __fmul_rn(__fmul_rn(a.sky.x, kBounceSky), T.x));
                R.y = __fadd_rn(R.y, __fmul_rn(__fmul_rn(a.sky.y, kBounceSky), T.y));
                R.z = __fadd_rn(R.z, __fmul_rn(__fmul_rn(a.sky.z, kBounceSky), T.z));
            }
            T.w = 0.0f;
        }
        bnc[c] = R;
        thr[c] = T;
    }
    if (hit_count) {
        const unsigned m = __ballot_sync(0xFFFFFFFFu, hit);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(hit_count, static_cast<unsigned long long>(__popc(m)));
    }
}

// Per-pixel mean of the slots' radiance (summed in sample order; inactive samples add 0), each
// slot's radiance being its first hit's plus the bounces' (FinalRadiance += Bounced).
__global__ void k_gather_accumulate(const float4* __restrict__ rad, const float4* __restrict__ bnc,
                                    const int32_t* __restrict__ comp_of, int64_t n, int32_t spp,
                                    const PixelOut pixels) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int k = 0; k < spp; ++k) {
        const int32_t c = __ldg(comp_of + i * spp + k);
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (c >= 0) {
            v = __ldg(rad + c);
            const float4 b = __ldg(bnc + c);
            v.x = __fadd_rn(v.x, b.x);
            v.y = __fadd_rn(v.y, b.y);
            v.z = __fadd_rn(v.z, b.z);
        }
        acc.x = __fadd_rn(acc.x, v.x);
        acc.y = __fadd_rn(acc.y, v.y);
        acc.z = __fadd_rn(acc.z, v.z);
        acc.w = __fadd_rn(acc.w, v.w);
    }
    const float inv = __fdiv_rn(1.0f, static_cast<float>(spp));
    pixels.put(i, make_float4(__fmul_rn(acc.x, inv), __fmul_rn(acc.y, inv), __fmul_rn(acc.z, inv),
                              __fmul_rn(acc.w, inv)));
}

__global__ void k_count_hits_c(const rq_hit* __restrict__ hits, int64_t n_max,
                               const unsigned long long* count, unsigned long long* cnt) {
    const int64_t n = static_cast<int64_t>(*count) < n_max ? static_cast<int64_t>(*count) : n_max;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool h = i < n && __ldg(reinterpret_cast<const float*>(hits) + 8 * i) > 0.0f;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, h);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(cnt, static_cast<unsigned long long>(__popc(m)));
}

__global__ void k_count_bytes_c(const uint8_t* __restrict__ b, int64_t n_max,
                                const unsigned long long* count, unsigned long long* cnt) {
    const int64_t n = static_cast<int64_t>(*count) < n_max ? static_cast<int64_t>(*count) : n_max;
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool h = i < n && b[i] != 0;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, h);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(cnt, static_cast<unsigned long long>(__popc(m)));
}

// GetDirect (DiffuseTrace.glsl:368-372) + emissive (:491) + AO (:494).
__global__ void k_shade(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                        int64_t n, const uint8_t* __restrict__ lit, int lit_is_occlusion,
                        const Materials mat, GiArgs a,
                        float4* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * j;
    const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    if (!(r1.w > r0.w)) {
        out[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    float4 h0;
    int4 h1;
    get_hit(hits, j, h0, h1);
    // lit[j] = 1 means the sun is visible; an occlusion buffer (1 = blocked) is read inverted.
    const float l = lit ? ((lit[j] != 0) != (lit_is_occlusion != 0) ? 1.0f : 0.0f) : 1.0f;
    out[j] = shade_one(s, mat, a, strict::xyz(r1), h0, h1, l);
}

// Per-pixel mean over the spp secondary samples (summed in sample order).
__global__ void k_accumulate(const float4* __restrict__ shaded, int64_t n, int32_t spp,
                             const PixelOut pixels) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int k = 0; k < spp; ++k) {
        const float4 v = __ldg(shaded + i * spp + k);
        acc.x = __fadd_rn(acc.x, v.x);
        acc.y = __fadd_rn(acc.y, v.y);
        acc.z = __fadd_rn(acc.z, v.z);
        acc.w = __fadd_rn(acc.w, v.w);
    }
    const float inv = __fdiv_rn(1.0f, static_cast<float>(spp));
    pixels.put(i, make_float4(__fmul_rn(acc.x, inv), __fmul_rn(acc.y, inv), __fmul_rn(acc.z, inv),
                              __fmul_rn(acc.w, inv)));
}

__global__ void k_count_hits(const rq_hit* __restrict__ hits, int64_t n, unsigned long long* cnt) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool h = i < n && __ldg(reinterpret_cast<const float*>(hits) + 8 * i) > 0.0f;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, h);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(cnt, static_cast<unsigned long long>(__popc(m)));
}


inline unsigned grid(int64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

rq_status check_params(rq_ctx* ctx, const rq_gi_params* p) {
    if (!p) return fail(ctx, RQ_EINVAL, "NULL gi params");
    if (p->spp < 1 || p->spp > 1024) return fail(ctx, RQ_EINVAL, "spp must be 1..1024");
    if (p->normal_mode != 0 && p->normal_mode != 1) return fail(ctx, RQ_EINVAL, "bad normal_mode");
    if (p->query != 0 && p->query != 1) return fail(ctx, RQ_EINVAL, "bad query kind");
    if (p->bounces < 0 || p->bounces > 8) return fail(ctx, RQ_EINVAL, "bounces must be 0..8");
    if (p->pixel_format != RQ_PIXELS_RGBA32F && p->pixel_format != RQ_PIXELS_RGBA16F)
        return fail(ctx, RQ_EINVAL, "bad pixel_format");
    return RQ_OK;
}

}  // namespace

// Adds the active secondary ray count of a pass to the frame statistics: the compact count, or
// live x spp when the rays stayed in place.
__global__ void k_add_count(unsigned long long* dst, const unsigned long long* src,
                            const unsigned long long* live, int64_t n, int32_t spp, float compact_below) {
    *dst += compact_rays(live, n, compact_below) ? *src : *live * static_cast<unsigned long long>(spp);
}

// One GI pass over n primary rays on stream st, in three phases: (1) primary closest hits and
// secondary ray generation, (2) one secondary traversal over all compact rays (+ shadow rays),
// (3) shading and the per-pixel mean.  Device buffers: prim and pixels4.  With host buffers
// (h_prim / h_pix non-null, prim / pixels4 then device staging of n rays / pixels), the rays are
// copied in first, and phase 3 runs in chunks of kGiHostChunk pixels whose pixels are copied out
// on pipe[1] while the next chunk is shaded.  (Copying the rays in chunks overlapped with phase 1
// was measured slower on GB300: the primary traversal slowed several-fold while the host-to-device
// copies ran.)  With `stats`, the ray counts are added to the context's frame counters (cleared by
// the caller).
rq_status gi_pass(rq_ctx* ctx, const rq_scene* sc, const QueryConfig& q, const rq_gi_params& p,
                  const rq_ray* prim, int64_t n, void* pixels4, cudaStream_t st, bool stats,
                  const rq_ray* h_prim, void* h_pix, GiArena& arena) {
    rq_status s;
    const int64_t m = n * p.spp;
    void *d_phit = nullptr, *d_sec = nullptr, *d_shit = nullptr, *d_occ = nullptr, *d_shade = nullptr,
         *d_shadow = nullptr, *d_comp = nullptr;
    if ((s = arena.get(rq::kSlotPrimaryHits, sizeof(rq_hit) * n, &d_phit)) != RQ_OK ||
        (s = arena.get(rq::kSlotRays, sizeof(rq_ray) * m, &d_sec)) != RQ_OK ||
        (s = arena.get(rq::kSlotHits, sizeof(rq_hit) * m, &d_shit)) != RQ_OK ||
        (s = arena.get(rq::kSlotOccluded, m, &d_occ)) != RQ_OK ||
        (s = arena.get(rq::kSlotCompactOf, 4 * m, &d_comp)) != RQ_OK)
        return s;
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(ctx->counters);
    unsigned long long* count = arena.count();  // compact (active) secondary rays
    RQ_CUDA(ctx, cudaMemsetAsync(count, 0, sizeof(unsigned long long), st));
    const GiArgs a = to_args(p);
    rq_hit* phit = static_cast<rq_hit*>(d_phit);
    rq_ray* sec = static_cast<rq_ray*>(d_sec);
    rq_hit* shit = static_cast<rq_hit*>(d_shit);
    uint8_t* occ = static_cast<uint8_t*>(d_occ);
    int32_t* comp_of = static_cast<int32_t*>(d_comp);
    const int64_t chunk = h_pix ? kGiHostChunk : n;
    const int64_t pix_bytes = p.pixel_format == RQ_PIXELS_RGBA16F ? 8 : 16;
    auto px = [&](int64_t off) {
        return PixelOut{static_cast<char*>(pixels4) + off * pix_bytes, pix_bytes == 8};
    };
    // Camera rays are coherent and short (a few node visits): the one-thread-per-ray form of the
    // tuned launch shape beats the persistent ray queue there, which pays per-ray hand-over costs.
    QueryConfig qp = q;
    qp.variant_closest = non_persistent_variant(q.variant_closest);
    // RT second-bounce loop: per compact slot its sample index, radiance and path throughput
    const bool bounce = p.query == 0 && p.bounces > 0;
    int32_t* samp_of = nullptr;
    float4 *rad = nullptr, *thr = nullptr, *bnc = nullptr;
    if (bounce) {
        void *d_samp = nullptr, *d_rad = nullptr, *d_thr = nullptr;
        void* d_bnc = nullptr;
        if ((s = arena.get(rq::kSlotSampleOf, 4 * m, &d_samp)) != RQ_OK || (s = arena.get(rq::kSlotRadiance, 16 * m, &d_rad)) != RQ_OK ||
            (s = arena.get(rq::kSlotThroughput, 16 * m, &d_thr)) != RQ_OK || (s = arena.get(rq::kSlotBounced, 16 * m, &d_bnc)) != RQ_OK)
            return s;
        samp_of = static_cast<int32_t*>(d_samp);
        rad = static_cast<float4*>(d_rad);
        thr = static_cast<float4*>(d_thr);
        bnc = static_cast<float4*>(d_bnc);
    }
    // phase 1.  Host rays in pinned memory on the BVH8 layout: the primary launch reads them over
    // the host link itself and stores the device copy the later kernels read, so the transfer
    // overlaps the traversal; other host rays are copied in first.
    SceneView pv = sc->view;
    const rq_ray* src = prim;
    if (h_prim && q.layout == RQ_LAYOUT_BVH8Q) {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, h_prim) == cudaSuccess && at.type == cudaMemoryTypeHost &&
            at.devicePointer != nullptr) {
            src = static_cast<const rq_ray*>(at.devicePointer);
            pv.ray_copy = const_cast<rq_ray*>(prim);
        } else {
            (void)cudaGetLastError();  // not registered with CUDA: copy it in
        }
    }
    if (h_prim && src == prim)
        RQ_CUDA(ctx, cudaMemcpyAsync(const_cast<rq_ray*>(prim), h_prim, sizeof(rq_ray) * n,
                                     cudaMemcpyHostToDevice, st));
    RQ_CUDA(ctx, launch_closest(pv, qp, src, n, phit, arena.queue(0), st));
    if (stats) k_count_hits<<<grid(n, 256), 256, 0, st>>>(phit, n, cnt + 0);
    // Compaction threshold: the per-pixel form keeps the rays in place when the fraction of primary
    // rays with a hit is at or above it (counted on the device: no host round trip); the bounce
    // loop, octant binning and the per-sample form always compact.
    const float compact_below = p.compact_below > 0.0f ? p.compact_below : sc->gi_compact_below;
    const unsigned long long* live = nullptr;
    if (compact_below <= 1.0f && !bounce && !p.sort_rays && !p.unfused) {
        unsigned long long* lw = arena.live();
        RQ_CUDA(ctx, cudaMemsetAsync(lw, 0, sizeof(unsigned long long), st));
        k_count_hits<<<grid(n, 256), 256, 0, st>>>(phit, n, lw);
        live = lw;
    }
    if ((!p.sort_rays && !p.unfused) || bounce) {
        k_gi_raygen_pixel<<<grid(n, 256), 256, 0, st>>>(sc->view, prim, phit, n, a, sec, comp_of, count,
                                                        samp_of, live, compact_below);
    } else if (p.sort_rays) {
        void* d_oct = nullptr;
        if ((s = arena.get(rq::kSlotOctants, 16 * sizeof(unsigned long long), &d_oct)) != RQ_OK) return s;
        unsigned long long* counts = static_cast<unsigned long long*>(d_oct);
        RQ_CUDA(ctx, cudaMemsetAsync(counts, 0, 16 * sizeof(unsigned long long), st));
        k_gi_octant_count<<<grid(m, 256), 256, 0, st>>>(sc->view, prim, phit, n, a, counts);
        k_gi_octant_scatter<<<grid(m, 256), 256, 0, st>>>(sc->view, prim, phit, n, a, counts, counts + 8, sec,
                                                          comp_of, count);
    } else if (p.unfused) {
        k_gi_raygen_compact<<<grid(m, 256), 256, 0, st>>>(sc->view, prim, phit, n, a, sec, comp_of, count);
    }
    RQ_CUDA(ctx, cudaGetLastError());
    if (stats) k_add_count<<<1, 1, 0, st>>>(cnt + 5, count, live, n, p.spp, compact_below);
    // phase 2
    SceneView cv = sc->view;  // secondary launches cover only the compact prefix
    cv.ray_count = count;
    const uint8_t* vis = nullptr;
    if (p.query == 1) {
        RQ_CUDA(ctx, launch_anyhit(cv, q, sec, m, occ, arena.queue(1), st));
        if (stats) k_count_bytes_c<<<grid(m, 256), 256, 0, st>>>(occ, m, count, cnt + 2);
        vis = occ;
    } else {
        RQ_CUDA(ctx, launch_closest(cv, q, sec, m, shit, arena.queue(1), st));
        if (stats) k_count_hits_c<<<grid(m, 256), 256, 0, st>>>(shit, m, count, cnt + 2);
        if (p.shadow_rays) {
            if ((s = arena.get(rq::kSlotShadowRays, sizeof(rq_ray) * m, &d_shadow)) != RQ_OK) return s;
            rq_ray* sh = static_cast<rq_ray*>(d_shadow);
            k_shadow_raygen_c<<<grid(m, 256), 256, 0, st>>>(sc->view, sec, shit, m, a, sh, count,
                                                            stats ? cnt + 3 : nullptr);
            RQ_CUDA(ctx, cudaGetLastError());
            RQ_CUDA(ctx, launch_anyhit(cv, q, sh, m, occ, arena.queue(2), st));
            if (stats) k_count_bytes_c<<<grid(m, 256), 256, 0, st>>>(occ, m, count, cnt + 4);
            vis = occ;
        }
    }
    if (bounce) {
        // Live paths are compacted every bounce: the rays ping-pong between a scratch buffer and
        // the (no longer needed) GI rays, the hits reuse the GI hit buffer, and per segment the
        // GI slot it belongs to is kept.
        void *d_bray = nullptr, *d_sa = nullptr, *d_sb = nullptr, *d_bc = nullptr;
        if ((s = arena.get(rq::kSlotBounceRays, sizeof(rq_ray) * m, &d_bray)) != RQ_OK ||
            (s = arena.get(rq::kSlotBounceSlotA, 4 * m, &d_sa)) != RQ_OK || (s = arena.get(rq::kSlotBounceSlotB, 4 * m, &d_sb)) != RQ_OK ||
            (s = arena.get(rq::kSlotBounceCounts, 8 * sizeof(unsigned long long) + 8 * p.bounces, &d_bc)) != RQ_OK)
            return s;
        unsigned long long* bcount = static_cast<unsigned long long*>(d_bc);
        RQ_CUDA(ctx, cudaMemsetAsync(bcount, 0, sizeof(unsigned long long) * p.bounces, st));
        k_bounce_init<<<grid(m, 256), 256, 0, st>>>(sc->view, sec, shit, vis, count, m, materials_of(sc), a, rad, thr,
                                                    bnc);
        RQ_CUDA(ctx, cudaGetLastError());
        QueryConfig qb = q;  // bounces use IntersectRay, not the ignore-transparent variant
        qb.flags &= ~RQ_FLAG_IGNORE_TRANSPARENT;
        rq_ray* ray_buf[2] = {static_cast<rq_ray*>(d_bray), sec};
        int32_t* slot_buf[2] = {static_cast<int32_t*>(d_sa), static_cast<int32_t*>(d_sb)};
        const rq_ray* prev_rays = sec;
        const int32_t* prev_slot = nullptr;
        const unsigned long long* prev_count = count;
        for (int b = 0; b < p.bounces; ++b) {
            rq_ray* brays = ray_buf[b & 1];
            int32_t* bslot = slot_buf[b & 1];
            unsigned long long* bc = bcount + b;
            k_bounce_raygen<<<grid(m, 256), 256, 0, st>>>(sc->view, prev_rays, shit, prev_slot, prev_count, m, thr,
                                                          samp_of, a, b, brays, bslot, bc, stats ? cnt + 6 : nullptr);
            RQ_CUDA(ctx, cudaGetLastError());
            SceneView bv = sc->view;
            bv.ray_count = bc;
            RQ_CUDA(ctx, launch_closest(bv, qb, brays, m, shit, arena.queue(1), st));
            const uint8_t* bvis = nullptr;
            if (p.shadow_rays) {
                if ((s = arena.get(rq::kSlotShadowRays, sizeof(rq_ray) * m, &d_shadow)) != RQ_OK) return s;
                rq_ray* sh = static_cast<rq_ray*>(d_shadow);
                k_shadow_raygen_c<<<grid(m, 256), 256, 0, st>>>(sc->view, brays, shit, m, a, sh, bc, nullptr);
                RQ_CUDA(ctx, cudaGetLastError());
                RQ_CUDA(ctx, launch_anyhit(bv, qb, sh, m, occ, arena.queue(2), st));
                bvis = occ;
            }
            k_bounce_shade<<<grid(m, 256), 256, 0, st>>>(sc->view, brays, shit, bvis, bslot, bc, m, materials_of(sc), a,
                                                         (q.flags & RQ_FLAG_REF_COMPAT) ? 1 : 0, bnc, thr,
                                                         stats ? cnt + 7 : nullptr);
            RQ_CUDA(ctx, cudaGetLastError());
            prev_rays = brays;
            prev_slot = bslot;
            prev_count = bc;
        }
    }
    // phase 3
    float4* shade = nullptr;
    if (p.unfused && !bounce) {  // per-sample shading into a scratch buffer, then the per-pixel mean
        if ((s = arena.get(rq::kSlotShaded, 16 * m, &d_shade)) != RQ_OK) return s;
        shade = static_cast<float4*>(d_shade);
        k_shade_c<<<grid(m, 256), 256, 0, st>>>(sc->view, sec, shit, comp_of, m, vis, p.query, materials_of(sc), a, shade);
    }
    for (int64_t off = 0; off < n; off += chunk) {
        const int64_t c = std::min(chunk, n - off);
        if (bounce)
            k_gather_accumulate<<<grid(c, 256), 256, 0, st>>>(rad, bnc, comp_of + off * p.spp, c, p.spp, px(off));
        else if (p.unfused)
            k_accumulate<<<grid(c, 256), 256, 0, st>>>(shade + off * p.spp, c, p.spp, px(off));
        else
            k_shade_accumulate<<<grid(c, 256), 256, 0, st>>>(sc->view, sec, shit, comp_of + off * p.spp, c, vis,
                                                             p.query, materials_of(sc), a, px(off));
        RQ_CUDA(ctx, cudaGetLastError());
        if (h_pix) {
            RQ_CUDA(ctx, cudaEventRecord(ctx->ev, st));
            RQ_CUDA(ctx, cudaStreamWaitEvent(ctx->pipe[1], ctx->ev, 0));
            RQ_CUDA(ctx, cudaMemcpyAsync(static_cast<char*>(h_pix) + off * pix_bytes, px(off).base, pix_bytes * c,
                                         cudaMemcpyDeviceToHost, ctx->pipe[1]));
        }
    }
    if (h_pix) {
        RQ_CUDA(ctx, cudaEventRecord(ctx->ev, ctx->pipe[1]));
        RQ_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev, 0));
    }
    return RQ_OK;
}

}  // namespace rq

using rq::fail;

extern "C" {

rq_status rq_scene_set_materials(rq_scene* sc, const float* albedo_rgb, int32_t n_meshes) {
    if (!sc || n_meshes < 0 || (n_meshes > 0 && !albedo_rgb))
        return fail(sc ? sc->ctx : nullptr, RQ_EINVAL, "bad material arguments");
    rq_ctx* ctx = sc->ctx;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    if (sc->d_albedo) cudaFree(sc->d_albedo);
    sc->d_albedo = nullptr;
    sc->n_albedo = 0;
    if (n_meshes == 0) return RQ_OK;
    if (cudaMalloc(&sc->d_albedo, sizeof(float) * 3 * n_meshes) != cudaSuccess)
        return fail(ctx, RQ_ENOMEM, "material buffer allocation failed");
    RQ_CUDA(ctx, cudaMemcpy(sc->d_albedo, albedo_rgb, sizeof(float) * 3 * n_meshes,
                            cudaMemcpyHostToDevice));
    sc->n_albedo = n_meshes;
    return RQ_OK;
}

rq_status rq_scene_set_textures(rq_scene* sc, const rq_texture* textures, int32_t n_textures,
                                const int32_t* mesh_texture, int32_t n_meshes) {
    if (!sc || n_textures < 0 || n_meshes < 0 || (n_textures > 0 && !textures) || (n_meshes > 0 && !mesh_texture))
        return fail(sc ? sc->ctx : nullptr, RQ_EINVAL, "bad texture arguments");
    rq_ctx* ctx = sc->ctx;
    std::vector<int4> desc(n_textures);
    int64_t total = 0;
    for (int32_t t = 0; t < n_textures; ++t) {
        const rq_texture& x = textures[t];
        if (x.width < 1 || x.height < 1 || x.width > 65536 || x.height > 65536 || !x.rgba8 ||
            (x.srgb != 0 && x.srgb != 1) || (x.wrap != 0 && x.wrap != 1))
            return fail(ctx, RQ_EINVAL, "texture " + std::to_string(t) + ": bad size, data, srgb or wrap");
        desc[t] = make_int4(static_cast<int32_t>(total), x.width, x.height, x.srgb | (x.wrap << 1));
        total += static_cast<int64_t>(x.width) * x.height;
        if (total >= (int64_t(1) << 31)) return fail(ctx, RQ_EINVAL, "more than 2^31 texels");
    }
    for (int32_t m = 0; m < n_meshes; ++m)
        if (mesh_texture[m] < -1 || mesh_texture[m] >= n_textures)
            return fail(ctx, RQ_EINVAL, "mesh " + std::to_string(m) + ": texture index out of range");
    std::vector<uint32_t> texels(static_cast<size_t>(total));
    for (int32_t t = 0; t < n_textures; ++t) {
        const uint8_t* p = textures[t].rgba8;
        const int64_t nt = static_cast<int64_t>(textures[t].width) * textures[t].height;
        for (int64_t k = 0; k < nt; ++k)
            texels[desc[t].x + k] = uint32_t(p[4 * k]) | (uint32_t(p[4 * k + 1]) << 8) |
                                    (uint32_t(p[4 * k + 2]) << 16) | (uint32_t(p[4 * k + 3]) << 24);
    }
    float lut[256];  // IEC 61966-2-1 decoding of byte / 255, in double, rounded once
    for (int c = 0; c < 256; ++c) {
        const double x = c / 255.0;
        lut[c] = static_cast<float>(x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4));
    }
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    RQ_CUDA(ctx, cudaDeviceSynchronize());  // no kernel may still read the old arrays
    for (void* q : {static_cast<void*>(sc->d_mesh_tex), static_cast<void*>(sc->d_tex),
                    static_cast<void*>(sc->d_texels), static_cast<void*>(sc->d_srgb)})
        if (q) cudaFree(q);
    sc->d_mesh_tex = nullptr;
    sc->d_tex = nullptr;
    sc->d_texels = nullptr;
    sc->d_srgb = nullptr;
    sc->n_mesh_tex = 0;
    sc->tex_bytes = 0;
    if (n_meshes == 0) return RQ_OK;
    const size_t mb = 4 * static_cast<size_t>(n_meshes), db = 16 * std::max<size_t>(1, desc.size()),
                 tb = 4 * std::max<size_t>(1, texels.size());
    if (cudaMalloc(&sc->d_mesh_tex, mb) != cudaSuccess || cudaMalloc(&sc->d_tex, db) != cudaSuccess ||
        cudaMalloc(&sc->d_texels, tb) != cudaSuccess || cudaMalloc(&sc->d_srgb, sizeof(lut)) != cudaSuccess)
        return fail(ctx, RQ_ENOMEM, "texture allocation failed");
    RQ_CUDA(ctx, cudaMemcpy(sc->d_mesh_tex, mesh_texture, mb, cudaMemcpyHostToDevice));
    if (!desc.empty()) RQ_CUDA(ctx, cudaMemcpy(sc->d_tex, desc.data(), 16 * desc.size(), cudaMemcpyHostToDevice));
    if (!texels.empty())
        RQ_CUDA(ctx, cudaMemcpy(sc->d_texels, texels.data(), 4 * texels.size(), cudaMemcpyHostToDevice));
    RQ_CUDA(ctx, cudaMemcpy(sc->d_srgb, lut, sizeof(lut), cudaMemcpyHostToDevice));
    sc->n_mesh_tex = n_meshes;
    sc->tex_bytes = static_cast<int64_t>(mb + db + tb + sizeof(lut));
    return RQ_OK;
}

rq_status rq_gi_raygen(rq_ctx* ctx, const rq_scene* sc, const rq_ray* primary, const rq_hit* hits,
                       int64_t n, const rq_gi_params* p, rq_ray* out, void* stream) {
    if (!ctx || !sc || n < 0 || (n > 0 && (!primary || !hits || !out)))
        return fail(ctx, RQ_EINVAL, "bad arguments");
    rq_status s = rq::check_params(ctx, p);
    if (s != RQ_OK || n == 0) return s;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = the default stream
    const int64_t total = n * p->spp;
    rq::k_gi_raygen<<<rq::grid(total, 256), 256, 0, st>>>(sc->view, primary, hits, n, rq::to_args(*p),
                                                          out, nullptr);
    RQ_CUDA(ctx, cudaGetLastError());
    return RQ_OK;
}

rq_status rq_shadow_raygen(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays, const rq_hit* hits,
                           int64_t n, const rq_gi_params* p, rq_ray* out, void* stream) {
    if (!ctx || !sc || n < 0 || (n > 0 && (!rays || !hits || !out)))
        return fail(ctx, RQ_EINVAL, "bad arguments");
    rq_status s = rq::check_params(ctx, p);
    if (s != RQ_OK || n == 0) return s;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = the default stream
    rq::k_shadow_raygen<<<rq::grid(n, 256), 256, 0, st>>>(sc->view, rays, hits, n, rq::to_args(*p),
                                                          out, nullptr);
    RQ_CUDA(ctx, cudaGetLastError());
    return RQ_OK;
}

rq_status rq_shade(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays, const rq_hit* hits,
                   int64_t n, const uint8_t* lit, const rq_gi_params* p, float* out4, void* stream) {
    if (!ctx || !sc || n < 0 || (n > 0 && (!rays || !hits || !out4)))
        return fail(ctx, RQ_EINVAL, "bad arguments");
    rq_status s = rq::check_params(ctx, p);
    if (s != RQ_OK || n == 0) return s;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = the default stream
    rq::k_shade<<<rq::grid(n, 256), 256, 0, st>>>(sc->view, rays, hits, n, lit, 0, rq::materials_of(sc),
                                                  rq::to_args(*p),
                                                  reinterpret_cast<float4*>(out4));
    RQ_CUDA(ctx, cudaGetLastError());
    return RQ_OK;
}

rq_status rq_gi_autotune(rq_ctx* ctx, rq_scene* sc, const rq_ray* primary, int64_t n, const rq_gi_params* p,
                         const rq_opts* opts, float* pixels4, rq_gi_tune* out) {
    if (!ctx || !sc || !out || n <= 0 || !primary || !pixels4) return fail(ctx, RQ_EINVAL, "bad arguments");
    rq_status s = rq::check_params(ctx, p);
    if (s != RQ_OK) return s;
    rq::QueryConfig q{};
    if ((s = rq::resolve_query(ctx, sc, opts, q)) != RQ_OK) return s;
    if (q.flags & RQ_FLAG_HOST_BUFFERS) return fail(ctx, RQ_EINVAL, "rq_gi_autotune takes device buffers");
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    rq::CtxGiArena arena(ctx);
    cudaEvent_t a, b;
    RQ_CUDA(ctx, cudaEventCreate(&a));
    RQ_CUDA(ctx, cudaEventCreate(&b));
    float ms[2] = {1e30f, 1e30f};
    unsigned long long live = 0;
    for (int form = 0; form < 2; ++form) {  // 0: always compact, 1: in place
        rq_gi_params pp = *p;
        pp.bounces = 0;
        pp.sort_rays = 0;
        pp.unfused = 0;
        pp.compact_below = form == 0 ? 2.0f : 1e-30f;
        for (int rep = 0; rep < 4; ++rep) {
            RQ_CUDA(ctx, cudaEventRecord(a, st));
            if ((s = rq::gi_pass(ctx, sc, q, pp, primary, n, pixels4, st, false, nullptr, nullptr, arena)) != RQ_OK)
                return s;
            RQ_CUDA(ctx, cudaEventRecord(b, st));
            RQ_CUDA(ctx, cudaEventSynchronize(b));
            float t = 0.0f;
            RQ_CUDA(ctx, cudaEventElapsedTime(&t, a, b));
            if (rep > 0) ms[form] = std::min(ms[form], t);
        }
        if (form == 1) RQ_CUDA(ctx, cudaMemcpy(&live, arena.live(), sizeof(live), cudaMemcpyDeviceToHost));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    out->live_fraction = static_cast<float>(static_cast<double>(live) / static_cast<double>(n));
    out->ms_compact = ms[0];
    out->ms_in_place = ms[1];
    sc->gi_compact_below = ms[1] < ms[0] ? std::max(out->live_fraction, 1e-30f) : 2.0f;
    out->compact_below = sc->gi_compact_below;
    return RQ_OK;
}

rq_status rq_gi_frame(rq_ctx* ctx, const rq_scene* sc, const rq_ray* primary, int64_t n,
                      const rq_gi_params* p, const rq_opts* opts, float* pixels4,
                      rq_frame_stats* stats, void* stream) {
    if (!ctx || !sc || n < 0 || (n > 0 && (!primary || !pixels4)))
        return fail(ctx, RQ_EINVAL, "bad arguments");
    rq_status s = rq::check_params(ctx, p);
    if (s != RQ_OK) return s;
    rq::QueryConfig q{};
    if ((s = rq::resolve_query(ctx, sc, opts, q)) != RQ_OK) return s;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = the default stream
    const bool host = (q.flags & RQ_FLAG_HOST_BUFFERS) != 0;
    q.flags &= ~RQ_FLAG_HOST_BUFFERS;
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(ctx->counters);
    if (stats) RQ_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8 * sizeof(unsigned long long), st));
    rq::CtxGiArena arena(ctx);
    if (!host) {
        if ((s = rq::gi_pass(ctx, sc, q, *p, primary, n, pixels4, st, stats != nullptr, nullptr, nullptr, arena)) !=
            RQ_OK)
            return s;
    } else {
        void *d_prim = nullptr, *d_pix = nullptr;
        if ((s = rq::scratch(ctx, rq::kSlotStageRays, sizeof(rq_ray) * n, &d_prim)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotStageOut, 16 * n, &d_pix)) != RQ_OK)
            return s;
        if ((s = rq::gi_pass(ctx, sc, q, *p, static_cast<const rq_ray*>(d_prim), n, d_pix, st, stats != nullptr,
                             primary, pixels4, arena)) != RQ_OK)
            return s;
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
    if (stats) {
        unsigned long long c[8];
        RQ_CUDA(ctx, cudaMemcpyAsync(c, cnt, sizeof(c), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
        stats->primary_rays = n;
        stats->primary_hits = static_cast<int64_t>(c[0]);
        stats->secondary_rays = static_cast<int64_t>(c[5]);
        stats->secondary_hits = static_cast<int64_t>(c[2]);
        stats->shadow_rays = static_cast<int64_t>(c[3]);
        stats->shadow_occluded = static_cast<int64_t>(c[4]);
        stats->bounce_rays = static_cast<int64_t>(c[6]);
        stats->bounce_hits = static_cast<int64_t>(c[7]);
    }
    return RQ_OK;
}

}  // extern "C"
