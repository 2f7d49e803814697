// FP64 recomputation of winning hits (the only double-precision code on the GPU).
#include <cuda_runtime.h>

#include <cmath>

#include "rq_objects.h"

namespace rq {
namespace {

struct d3 {
    double x, y, z;
};
__device__ __forceinline__ d3 dsub(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 dcross(d3 a, d3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 dxform(const float* m, d3 v, double w) {
    return {double(m[0]) * v.x + double(m[4]) * v.y + double(m[8]) * v.z + double(m[12]) * w,
            double(m[1]) * v.x + double(m[5]) * v.y + double(m[9]) * v.z + double(m[13]) * w,
            double(m[2]) * v.x + double(m[6]) * v.y + double(m[10]) * v.z + double(m[14]) * w};
}

__global__ void k_verify(SceneView s, const rq_ray* __restrict__ rays, const rq_hit* __restrict__ hits,
                         int64_t n, float* __restrict__ err) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* hp = reinterpret_cast<const float4*>(hits) + 2 * i;
    const float4 h0 = hp[0], h1 = hp[1];
    const int32_t tri = __float_as_int(h1.x), ent = __float_as_int(h1.z);
    const float nanf_ = __int_as_float(0x7FC00000);
    err[2 * i] = nanf_;
    err[2 * i + 1] = nanf_;
    if (!(h0.x > 0.0f) || tri < 0 || tri >= s.n_tris || ent < 0 || ent >= s.n_ents) return;
    const float4* rp = reinterpret_cast<const float4*>(rays) + 2 * i;
    const float4 r0 = rp[0], r1 = rp[1];
    const rq_entity& e = s.ents[ent];
    const d3 o = dxform(e.inverse, {r0.x, r0.y, r0.z}, 1.0);
    const d3 d = dxform(e.inverse, {r1.x, r1.y, r1.z}, 0.0);
    const int4 tr = s.tris[tri];
    const float4 A = s.verts[2 * static_cast<int64_t>(tr.x)], B = s.verts[2 * static_cast<int64_t>(tr.y)];
    const float4 C = s.verts[2 * static_cast<int64_t>(tr.z)];
    const d3 a = {A.x, A.y, A.z}, b = {B.x, B.y, B.z}, c = {C.x, C.y, C.z};
    const d3 e1 = dsub(b, a), e2 = dsub(c, a);
    const d3 p = dcross(d, e2);
    const double det = ddot(e1, p);
    if (det == 0.0) return;
    const double id = 1.0 / det;
    const d3 tv = dsub(o, a);
    const double u = ddot(tv, p) * id;
    const d3 q = dcross(tv, e1);
    const double v = ddot(d, q) * id;
    const double t = ddot(e2, q) * id;
    if (!(t > 0.0)) return;
    const double wa = 1.0 - u - v;
    err[2 * i] = static_cast<float>(fabs(double(h0.x) - t) / t);
    const double db = fmax(fabs(double(h0.y) - wa), fmax(fabs(double(h0.z) - u), fabs(double(h0.w) - v)));
    err[2 * i + 1] = static_cast<float>(db);
}

}  // namespace
}  // namespace rq

extern "C" rq_status rq_verify_hits(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays,
                                    const rq_hit* hits, int64_t n, float* err2, void* stream) {
    if (!ctx || !sc || n < 0 || (n > 0 && (!rays || !hits || !err2)))
        return rq::fail(ctx, RQ_EINVAL, "bad arguments");
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    rq::k_verify<<<static_cast<unsigned>((n + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        sc->view, rays, hits, n, err2);
    RQ_CUDA(ctx, cudaGetLastError());
    return RQ_OK;
}
