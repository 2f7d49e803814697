// Per-hit surface attributes: the reference's GetData (TraverseBVHStack.glsl:422-455), which the
// IntersectRay overloads that return Albedo, Normal and Alpha (:458-502, stackless
// TraverseBVHStackless.glsl the same) run after IntersectScene.  rq_hit_attribs evaluates it over
// hit records; rq_closest_attribs is the closest-hit query followed by it.
//
// Per hit, with the statements in the shader's order (explicit round-to-nearest arithmetic, so the
// values equal the CPU restatement's bit for bit): a miss (t < 0 or mesh < 0) gives Normal = -1,
// Albedo = 0, Emissivity = 0; a hit gives the normalised barycentric mix of the three vertices'
// half-packed normals, the mesh's albedo texture sampled at the interpolated half-packed UV when it
// has one (and t > 0) or else its ModelColor, and the hit entity's emissive and alpha words.
#include <cuda_runtime.h>

#include "rq_gi.cuh"
#include "rq_objects.h"

namespace rq {
namespace {

__global__ void __launch_bounds__(256) k_hit_attribs(SceneView s, Materials mat, const rq_hit* __restrict__ hits,
                                                     int64_t n, rq_hit_attrib* __restrict__ out) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float4* hp = reinterpret_cast<const float4*>(hits) + 2 * j;
    const float4 h0 = __ldg(hp);
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(hp + 1));
    float4 o0, o1;
    if (h0.x < 0.0f || h1.y < 0) {
        o0 = make_float4(-1.0f, -1.0f, -1.0f, 0.0f);
        o1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    } else {
        const strict::f3 nrm = gi::hit_normal(s, h1.x, h0.y, h0.z, h0.w, 0);
        const strict::f3 alb = gi::hit_albedo(s, mat, h0, h1);
        float emissive = 0.0f, alpha = 1.0f;
        if (h1.z >= 0 && h1.z < s.n_ents) {
            emissive = __int_as_float(__ldg(&s.ents[h1.z].data[0]));
            alpha = __int_as_float(__ldg(&s.ents[h1.z].data[1]));
        }
        o0 = make_float4(nrm.x, nrm.y, nrm.z, alpha);
        o1 = make_float4(alb.x, alb.y, alb.z, emissive);
    }
    float4* op = reinterpret_cast<float4*>(out) + 2 * j;
    op[0] = o0;
    op[1] = o1;
}

inline unsigned grid256(int64_t n) { return static_cast<unsigned>((n + 255) / 256); }

}  // namespace
}  // namespace rq

using rq::fail;

extern "C" {

rq_status rq_hit_attribs(rq_ctx* ctx, const rq_scene* sc, const rq_hit* hits, int64_t n, rq_hit_attrib* out,
                         const rq_opts* opts, void* stream) {
    if (!ctx || !sc) return fail(ctx, RQ_EINVAL, "NULL context or scene");
    if (n < 0 || (n > 0 && (!hits || !out))) return fail(ctx, RQ_EINVAL, "bad hit/attribute arrays");
    if (sc->ctx != ctx) return fail(ctx, RQ_EINVAL, "scene belongs to another context");
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool host = opts && (opts->flags & RQ_FLAG_HOST_BUFFERS);
    const rq_hit* d_hits = hits;
    rq_hit_attrib* d_out = out;
    if (host) {
        void *a = nullptr, *b = nullptr;
        rq_status s;
        if ((s = rq::scratch(ctx, rq::kSlotPrimaryHits, sizeof(rq_hit) * n, &a)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotStageOut, sizeof(rq_hit_attrib) * n, &b)) != RQ_OK)
            return s;
        RQ_CUDA(ctx, cudaMemcpyAsync(a, hits, sizeof(rq_hit) * n, cudaMemcpyHostToDevice, st));
        d_hits = static_cast<const rq_hit*>(a);
        d_out = static_cast<rq_hit_attrib*>(b);
    }
    rq::k_hit_attribs<<<rq::grid256(n), 256, 0, st>>>(sc->view, rq::materials_of(sc), d_hits, n, d_out);
    RQ_CUDA(ctx, cudaGetLastError());
    if (host) {
        RQ_CUDA(ctx, cudaMemcpyAsync(out, d_out, sizeof(rq_hit_attrib) * n, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return RQ_OK;
}

rq_status rq_closest_attribs(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays, int64_t n, rq_hit* hits,
                             rq_hit_attrib* attribs, const rq_opts* opts, void* stream) {
    if (!ctx || !sc) return fail(ctx, RQ_EINVAL, "NULL context or scene");
    if (n < 0 || (n > 0 && (!rays || !hits || !attribs))) return fail(ctx, RQ_EINVAL, "bad ray/hit/attribute arrays");
    if (sc->ctx != ctx) return fail(ctx, RQ_EINVAL, "scene belongs to another context");
    rq::QueryConfig q{};
    rq_status s = rq::resolve_query(ctx, sc, opts, q);
    if (s != RQ_OK) return s;
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool host = (q.flags & RQ_FLAG_HOST_BUFFERS) != 0;
    q.flags &= ~RQ_FLAG_HOST_BUFFERS;
    const rq_ray* d_rays = rays;
    rq_hit* d_hits = hits;
    rq_hit_attrib* d_att = attribs;
    if (host) {
        void *a = nullptr, *b = nullptr, *c = nullptr;
        if ((s = rq::scratch(ctx, rq::kSlotStageRays, sizeof(rq_ray) * n, &a)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotPrimaryHits, sizeof(rq_hit) * n, &b)) != RQ_OK ||
            (s = rq::scratch(ctx, rq::kSlotStageOut, sizeof(rq_hit_attrib) * n, &c)) != RQ_OK)
            return s;
        RQ_CUDA(ctx, cudaMemcpyAsync(a, rays, sizeof(rq_ray) * n, cudaMemcpyHostToDevice, st));
        d_rays = static_cast<const rq_ray*>(a);
        d_hits = static_cast<rq_hit*>(b);
        d_att = static_cast<rq_hit_attrib*>(c);
    }
    RQ_CUDA(ctx, rq::launch_closest(sc->view, q, d_rays, n, d_hits, rq::queue_counter(ctx, 0), st));
    rq::k_hit_attribs<<<rq::grid256(n), 256, 0, st>>>(sc->view, rq::materials_of(sc), d_hits, n, d_att);
    RQ_CUDA(ctx, cudaGetLastError());
    if (host) {
        RQ_CUDA(ctx, cudaMemcpyAsync(hits, d_hits, sizeof(rq_hit) * n, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaMemcpyAsync(attribs, d_att, sizeof(rq_hit_attrib) * n, cudaMemcpyDeviceToHost, st));
        RQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return RQ_OK;
}

}  // extern "C"
