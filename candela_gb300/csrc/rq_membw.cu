// rq_measure_read_gbs: a read-bandwidth probe for the roofline denominators of the traversal
// kernels.  No counterpart in the reference.
//
// The traversal kernels read a scene that fits the L2 (the 1.31M-triangle scene is about 90 MB of
// BVH8 nodes and triangle records against 129 MB of L2), so their memory roof is the L2's read
// bandwidth, not HBM's.  This probe measures it the way the kernels read: 16-byte loads that bypass
// L1 (ld.global.cg), from every SM, over a buffer of the caller's size, re-read `reps` times
// back to back.  With a buffer well under the L2 size every read after the first pass is an L2
// hit; with one well above it the same probe measures HBM.
#include <cuda_runtime.h>

#include "rq_objects.h"

namespace {

// `passes` grid-stride reads of n16 16-byte words (each pass starts at a different rotation so that
// a thread does not re-read its own words from L1); the XOR of what was read is stored only when it
// equals a value the data cannot produce, so the loads stay live without a store per thread.
__global__ void __launch_bounds__(512) k_read(const uint4* __restrict__ buf, int64_t n16, int passes,
                                              unsigned* __restrict__ sink) {
    uint32_t acc = 0;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    for (int p = 0; p < passes; ++p) {
        int64_t i = t;
        const int64_t rot = (static_cast<int64_t>(p) * 7919 * 32) % n16;
        for (; i + 3 * stride < n16; i += 4 * stride) {
            int64_t j0 = i + rot, j1 = i + stride + rot, j2 = i + 2 * stride + rot, j3 = i + 3 * stride + rot;
            j0 -= j0 >= n16 ? n16 : 0;
            j1 -= j1 >= n16 ? n16 : 0;
            j2 -= j2 >= n16 ? n16 : 0;
            j3 -= j3 >= n16 ? n16 : 0;
            const uint4 a = __ldcg(buf + j0), b = __ldcg(buf + j1), c = __ldcg(buf + j2), d = __ldcg(buf + j3);
            acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
        }
        for (; i < n16; i += stride) {
            int64_t j = i + rot;
            j -= j >= n16 ? n16 : 0;
            const uint4 a = __ldcg(buf + j);
            acc ^= a.x ^ a.y ^ a.z ^ a.w;
        }
    }
    if (acc == 0x9E3779B9u) atomicAdd(sink, 1u);
}

__global__ void k_fill(uint4* buf, int64_t n16) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n16; i += stride)
        buf[i] = make_uint4(static_cast<uint32_t>(i), static_cast<uint32_t>(i >> 32), 0x01234567u, 0x89ABCDEFu);
}

}  // namespace

extern "C" {

rq_status rq_measure_read_gbs(rq_ctx* ctx, int64_t bytes, int32_t reps, double* gbs) {
    if (!ctx || !gbs || bytes < (1 << 20) || reps < 1 || reps > 100000)
        return rq::fail(ctx, RQ_EINVAL, "bad arguments (bytes >= 1 MiB, 1 <= reps <= 100000)");
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    int sms = 0;
    RQ_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int64_t n16 = bytes / 16;
    void* buf = nullptr;
    unsigned* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&buf, n16 * 16);
    if (e != cudaSuccess) return rq::fail(ctx, RQ_ENOMEM, "read probe: buffer allocation failed");
    cudaStream_t st = ctx->stream;
    float ms = 0.0f;
    if ((e = cudaMalloc(&sink, sizeof(unsigned))) == cudaSuccess &&
        (e = cudaEventCreate(&e0)) == cudaSuccess && (e = cudaEventCreate(&e1)) == cudaSuccess) {
        const unsigned grid = static_cast<unsigned>(sms) * 4;  // 4 blocks of 512 threads per SM
        k_fill<<<grid, 512, 0, st>>>(static_cast<uint4*>(buf), n16);
        k_read<<<grid, 512, 0, st>>>(static_cast<const uint4*>(buf), n16, 3, sink);  // warm-up
        // many passes per launch, so that launch gaps do not count against the bandwidth
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps; r += 50)
            k_read<<<grid, 512, 0, st>>>(static_cast<const uint4*>(buf), n16, reps - r < 50 ? reps - r : 50, sink);
        cudaEventRecord(e1, st);
        if ((e = cudaEventSynchronize(e1)) == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    cudaFree(buf);
    if (e != cudaSuccess) return rq::cuda_fail(ctx, e, "read probe");
    *gbs = static_cast<double>(n16) * 16.0 * reps / (static_cast<double>(ms) * 1e-3) / 1e9;
    return RQ_OK;
}

}  // extern "C"
