// rq_gi_frame_noalloc: the diffuse-GI / RTAO pass with its intermediate buffers in a fixed,
// library-owned device array instead of memory allocated per call.
//
// Who needs it: callers that must not allocate device memory while they render.  cudaMalloc can
// synchronise the whole device and can fail under memory pressure, so a frame loop that has to
// keep its timing, or a host application that owns every device byte through its own allocator
// and forbids plugins from calling cudaMalloc, cannot use rq_gi_frame, which grows its scratch
// buffers on demand.  This entry point allocates nothing: the scene must already be uploaded and
// the caller passes device buffers for the primary rays and the pixels.
//
// The scratch is one file-scope __device__ array of RQ_NOALLOC_MAX_RAYS-sized slices
// (~9.1 MiB).  Every GPU that loads librq.so holds it until the process exits.  Host code cannot
// use the array's name as a device address (it names a host-side stand-in), so the device address
// is fetched with cudaGetSymbolAddress, once per device, by the first call made on that device
// (with that device current) and cached.  Every call shares the array and it keeps the previous
// call's contents; each call writes every byte it later reads, so nothing needs clearing, but
// calls whose work overlaps on the GPU (other streams or host threads) race on it.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "rq_objects.h"

namespace {

constexpr int64_t kMaxRays = RQ_NOALLOC_MAX_RAYS;

// Slices of the scratch array, each 256-byte aligned.
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kPrimHitsOff = 0;
constexpr size_t kSecOff = kPrimHitsOff + align256(sizeof(rq_hit) * kMaxRays);
constexpr size_t kSecHitsOff = kSecOff + align256(sizeof(rq_ray) * kMaxRays);
constexpr size_t kShadowOff = kSecHitsOff + align256(sizeof(rq_hit) * kMaxRays);
constexpr size_t kShadedOff = kShadowOff + align256(sizeof(rq_ray) * kMaxRays);
constexpr size_t kOccOff = kShadedOff + align256(16 * kMaxRays);
constexpr size_t kScratchBytes = kOccOff + align256(kMaxRays);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on first use).
rq_status scratch_address(rq_ctx* ctx, int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices)
        return rq::fail(ctx, RQ_EINVAL, "device index beyond the no-alloc address table");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return rq::cuda_fail(ctx, e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_addr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_addr[device]);
    return RQ_OK;
}

}  // namespace

extern "C" {

rq_status rq_gi_frame_noalloc(rq_ctx* ctx, const rq_scene* sc, const rq_ray* primary, int64_t n,
                              const rq_gi_params* p, const rq_opts* opts, float* pixels4,
                              void* stream) {
    if (!ctx || !sc || !p || n < 0 || (n > 0 && (!primary || !pixels4)))
        return rq::fail(ctx, RQ_EINVAL, "bad arguments");
    if (p->spp < 1 || p->spp > 1024 || (p->query != 0 && p->query != 1) ||
        (p->normal_mode != 0 && p->normal_mode != 1))
        return rq::fail(ctx, RQ_EINVAL, "bad gi params");
    if (p->bounces != 0) return rq::fail(ctx, RQ_EINVAL, "the no-alloc GI pass has no further bounces");
    if (n > kMaxRays || n * p->spp > kMaxRays) {
        char msg[160];
        std::snprintf(msg, sizeof(msg),
                      "no-alloc GI pass: %lld pixels x %d spp exceeds the fixed scratch capacity of "
                      "%lld rays (RQ_NOALLOC_MAX_RAYS)",
                      static_cast<long long>(n), p->spp, static_cast<long long>(kMaxRays));
        return rq::fail(ctx, RQ_EINVAL, msg);
    }
    if (opts && (opts->flags & RQ_FLAG_HOST_BUFFERS))
        return rq::fail(ctx, RQ_EINVAL, "no-alloc GI pass takes device buffers only");
    rq::QueryConfig q{};
    rq_status s = rq::resolve_query(ctx, sc, opts, q);
    if (s != RQ_OK) return s;
    q.counters = nullptr;
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned char* base = nullptr;
    if ((s = scratch_address(ctx, ctx->device, &base)) != RQ_OK) return s;
    rq::GiBuffers b;
    b.primary_hits = reinterpret_cast<rq_hit*>(base + kPrimHitsOff);
    b.secondary = reinterpret_cast<rq_ray*>(base + kSecOff);
    b.secondary_hits = reinterpret_cast<rq_hit*>(base + kSecHitsOff);
    b.shadow = reinterpret_cast<rq_ray*>(base + kShadowOff);
    b.shaded = reinterpret_cast<float4*>(base + kShadedOff);
    b.occluded = base + kOccOff;
    RQ_CUDA(ctx, rq::gi_pass_on_buffers(sc->view, q, *p, rq::materials_of(sc), primary, n, b,
                                        pixels4, static_cast<cudaStream_t>(stream)));
    return RQ_OK;
}

}  // extern "C"
