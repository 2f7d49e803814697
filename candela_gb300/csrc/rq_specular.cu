// Specular reflection pass: the world-trace path of the reference's SpecularTrace.glsl
// (:485-596), one reflection ray per pixel from the primary hit, traced by the engine's
// closest-hit launch, lit by SampleLighting (:420-425) or the sky (:435-437).
#include <cuda_runtime.h>

#include <cstring>

#include "rq_gi.cuh"
#include "rq_objects.h"

namespace rq {
namespace {

using strict::f3;

struct SpecArgs {
    uint32_t seed;
    float roughness, ray_tmax;
    int32_t normal_mode;
    float shadow_offset;
    f3 sun_dir, sun_color, sky, ambient;
};

SpecArgs spec_args(const rq_specular_params& p) {
    SpecArgs a;
    a.seed = p.seed;
    a.roughness = p.roughness;
    a.ray_tmax = p.ray_tmax;
    a.normal_mode = p.normal_mode;
    a.shadow_offset = p.shadow_offset;
    a.sun_dir = {p.sun_dir[0], p.sun_dir[1], p.sun_dir[2]};
    a.sun_color = {p.sun_color[0], p.sun_color[1], p.sun_color[2]};
    a.sky = {p.sky_color[0], p.sky_color[1], p.sky_color[2]};
    a.ambient = {p.ambient[0], p.ambient[1], p.ambient[2]};
    return a;
}

// GLSL mix(x, y, a) = x * (1 - a) + y * a.
__device__ __forceinline__ float mixf(float x, float y, float a) {
    return __fadd_rn(__fmul_rn(x, __fsub_rn(1.0f, a)), __fmul_rn(y, a));
}

__device__ __forceinline__ void put(rq_ray* out, int64_t i, f3 o, f3 d, float tmax) {
    float4* p = reinterpret_cast<float4*>(out) + 2 * i;
    p[0] = make_float4(o.x, o.y, o.z, 0.0f);
    p[1] = make_float4(d.x, d.y, d.z, tmax);
}

// Reflection ray of pixel i (SpecularTrace.glsl:505-513, StochasticReflectionDirection :102-135).
__global__ void k_spec_raygen(SceneView s, const rq_ray* __restrict__ prim, const rq_hit* __restrict__ hits,
                              int64_t n, SpecArgs a, rq_ray* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* hp = reinterpret_cast<const float4*>(hits) + 2 * i;
    const float4 h0 = __ldg(hp), h1f = __ldg(hp + 1);
    if (!(h0.x > 0.0f)) {
        put(out, i, f3{0.0f, 0.0f, 0.0f}, f3{0.0f, 0.0f, 1.0f}, -1.0f);
        return;
    }
    const float4* pr = reinterpret_cast<const float4*>(prim) + 2 * i;
    const f3 ro = strict::xyz(__ldg(pr)), rd = strict::xyz(__ldg(pr + 1));
    const f3 P = strict::add(ro, strict::muls(rd, h0.x));
    f3 N = gi::hit_normal(s, __float_as_int(h1f.x), h0.y, h0.z, h0.w, a.normal_mode);
    if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
    const f3 I = gi::normalize(strict::sub(P, ro));
    const float r = __fmul_rn(a.roughness, 0.9f);
    f3 dir;
    if (r < 0.01f) {
        dir = gi::reflect(I, N);
    } else {
        f3 micro = N;
        const uint32_t rid = static_cast<uint32_t>(i);
        for (uint32_t k = 0; k < 12; ++k) {
            const float x0 = __fmul_rn(gi::u01(gi::sample_key(a.seed, rid, 2u * k)), 0.8f);
            const float x1 = __fmul_rn(gi::u01(gi::sample_key(a.seed, rid, 2u * k + 1u)), 0.7f);
            const f3 smp = gi::sample_ggx(N, r, x0, x1);
            if (strict::dot(smp, N) > 0.001f) {
                micro = smp;
                break;
            }
        }
        dir = gi::reflect(I, micro);
    }
    const float off = mixf(0.05f, 0.1f, strict::gmin(strict::gmax(__fmul_rn(a.roughness, 1.4f), 0.0f), 1.0f));
    put(out, i, strict::add(P, strict::muls(N, off)), dir, a.ray_tmax);
}

// Shadow ray toward the sun from the reflection hit of pixel i (inactive without a hit).
__global__ void k_spec_shadow(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                              int64_t n, SpecArgs a, rq_ray* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* hp = reinterpret_cast<const float4*>(hits) + 2 * i;
    const float4 h0 = __ldg(hp), h1f = __ldg(hp + 1);
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * i;
    const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    if (!(h0.x > 0.0f) || !(r1.w > r0.w)) {
        put(out, i, f3{0.0f, 0.0f, 0.0f}, f3{0.0f, 0.0f, 1.0f}, -1.0f);
        return;
    }
    const f3 ro = strict::xyz(r0), rd = strict::xyz(r1);
    const f3 P = strict::add(ro, strict::muls(rd, h0.x));
    f3 N = gi::hit_normal(s, __float_as_int(h1f.x), h0.y, h0.z, h0.w, a.normal_mode);
    if (strict::dot(N, rd) > 0.0001f) N = strict::neg(N);
    put(out, i, strict::add(P, strict::muls(N, a.shadow_offset)), strict::neg(a.sun_dir), 1000000.0f);
}

__device__ __forceinline__ bool finite3(f3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }

// SampleLighting (:420-425) + emissive, or the sky; IsValid, clamp to [0, 6], t / 48 (:588-596).
__global__ void k_spec_shade(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                             const uint8_t* __restrict__ occl, int64_t n, const Materials mat, SpecArgs a,
                             float4* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* pr = reinterpret_cast<const float4*>(rays) + 2 * i;
    const float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    if (!(r1.w > r0.w)) {  // the primary ray missed
        out[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float4* hp = reinterpret_cast<const float4*>(hits) + 2 * i;
    const float4 h0 = __ldg(hp), h1f = __ldg(hp + 1);
    const int4 h1 = make_int4(__float_as_int(h1f.x), __float_as_int(h1f.y), __float_as_int(h1f.z), 0);
    float t = h0.x;
    f3 rad;
    if (h0.x > 0.0f) {
        const f3 alb = gi::hit_albedo(s, mat, h0, h1);
        const float em = __int_as_float(s.ents[h1.z].data[0]);
        const float l = occl ? (occl[i] ? 0.0f : 1.0f) : 1.0f;
        const f3 direct = strict::muls(strict::mul(alb, a.sun_color), l);
        const f3 indirect = strict::mul(strict::muls(alb, 2.0f), a.ambient);
        rad = strict::add(strict::add(direct, indirect), strict::muls(alb, em));
    } else {
        rad = strict::muls(a.sky, mixf(1.4f, 2.65f, a.roughness));
    }
    if (!finite3(rad)) {
        rad = {0.0f, 0.0f, 0.0f};
        t = -1.0f;
    }
    rad = {strict::gmin(strict::gmax(rad.x, 0.0f), 6.0f), strict::gmin(strict::gmax(rad.y, 0.0f), 6.0f),
           strict::gmin(strict::gmax(rad.z, 0.0f), 6.0f)};
    out[i] = make_float4(rad.x, rad.y, rad.z, __fdiv_rn(t, 48.0f));
}

inline unsigned grid(int64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace
}  // namespace rq

using rq::fail;

extern "C" {

rq_status rq_specular_frame(rq_ctx* ctx, const rq_scene* sc, const rq_ray* primary, int64_t n,
                            const rq_specular_params* p, const rq_opts* opts, float* out4, void* stream) {
    if (!ctx || !sc || !p || n < 0 || (n > 0 && (!primary || !out4))) return fail(ctx, RQ_EINVAL, "bad arguments");
    if (p->normal_mode != 0 && p->normal_mode != 1) return fail(ctx, RQ_EINVAL, "bad normal_mode");
    rq::QueryConfig q{};
    rq_status s;
    if ((s = rq::resolve_query(ctx, sc, opts, q)) != RQ_OK) return s;
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool host = (q.flags & RQ_FLAG_HOST_BUFFERS) != 0;
    q.flags &= ~RQ_FLAG_HOST_BUFFERS;
    void *d_prim = nullptr, *d_out = nullptr, *d_phit = nullptr, *d_ray = nullptr, *d_hit = nullptr,
         *d_sh = nullptr, *d_occ = nullptr;
    // scratch: the GI pass's slots (a specular pass never overlaps one on the same context)
    if ((s = rq::scratch(ctx, rq::kSlotPrimaryHits, sizeof(rq_hit) * n, &d_phit)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotRays, sizeof(rq_ray) * n, &d_ray)) != RQ_OK ||
        (s = rq::scratch(ctx, rq::kSlotHits, sizeof(rq_hit) * n, &d_hit)) != RQ_OK)
        return s;
    const rq_ray* prim = primary;
    float4* out = reinterpret_cast<float4*>(out4);
    if (host) {
        if ((s = rq::scratch(ctx, rq::kSlotStageRays, sizeof(rq_ray) * n, &d_prim)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotStageOut, 16 * n, &d_out)) != RQ_OK)
            return s;
        RQ_CUDA(ctx, cudaMemcpyAsync(d_prim, primary, sizeof(rq_ray) * n, cudaMemcpyHostToDevice, st));
        prim = static_cast<const rq_ray*>(d_prim);
        out = static_cast<float4*>(d_out);
    }
    const rq::SpecArgs a = rq::spec_args(*p);
    rq_hit* phit = static_cast<rq_hit*>(d_phit);
    rq_ray* ray = static_cast<rq_ray*>(d_ray);
    rq_hit* hit = static_cast<rq_hit*>(d_hit);
    rq::QueryConfig qp = q;  // camera rays: one thread per ray (as in the GI pass)
    qp.variant_closest = rq::non_persistent_variant(q.variant_closest);
    RQ_CUDA(ctx, rq::launch_closest(sc->view, qp, prim, n, phit, rq::queue_counter(ctx, 0), st));
    rq::k_spec_raygen<<<rq::grid(n, 256), 256, 0, st>>>(sc->view, prim, phit, n, a, ray);
    RQ_CUDA(ctx, cudaGetLastError());
    RQ_CUDA(ctx, rq::launch_closest(sc->view, q, ray, n, hit, rq::queue_counter(ctx, 1), st));
    const uint8_t* vis = nullptr;
    if (p->shadow_rays) {
        if ((s = rq::scratch(ctx, rq::kSlotShadowRays, sizeof(rq_ray) * n, &d_sh)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotOccluded, n, &d_occ)) != RQ_OK)
            return s;
        rq::k_spec_shadow<<<rq::grid(n, 256), 256, 0, st>>>(sc->view, ray, hit, n, a, static_cast<rq_ray*>(d_sh));
        RQ_CUDA(ctx, cudaGetLastError());
        RQ_CUDA(ctx, rq::launch_anyhit(sc->view, q, static_cast<rq_ray*>(d_sh), n, static_cast<uint8_t*>(d_occ),
                                       rq::queue_counter(ctx, 2), st));
        vis = static_cast<uint8_t*>(d_occ);
    }
    rq::k_spec_shade<<<rq::grid(n, 256), 256, 0, st>>>(sc->view, ray, hit, vis, n, rq::materials_of(sc), a, out);
    RQ_CUDA(ctx, cudaGetLastError());
    if (host) {
        RQ_CUDA(ctx, cudaMemcpyAsync(out4, out, 16 * n, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return RQ_OK;
}

}  // extern "C"
