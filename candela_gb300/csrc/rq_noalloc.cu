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
// It runs the same pass as rq_gi_frame (gi_pass in rq_gi.cu: the per-pixel fused ray generation
// and shading kernels, the autotuned launch variants, the persistent ray queue), only with every
// intermediate buffer and device counter carved from one file-scope __device__ array sized for
// RQ_NOALLOC_MAX_RAYS rays (about 8.3 MiB).  So its pixels are the pixels rq_gi_frame gives for the
// same arguments, bit for bit.
//
// The array's device address: host code cannot use the array's name as a device address (it names
// a host-side stand-in), so rq_create fetches the address with cudaGetSymbolAddress, with the
// context's device current, and keeps it in the context (noalloc_resolve below).  That call is also
// what makes the CUDA runtime load this file's module, which reserves the array on that device (CUDA
// loads modules lazily by default): so the array is reserved when the first context is created on a
// device, not inside a frame, and stays reserved until the process exits.  A context created after a
// cudaDeviceReset resolves the address again.
//
// Every call shares the array and it keeps the previous call's contents.  Each call writes every
// byte it later reads (the ray counters included), so nothing needs clearing, but calls whose work
// overlaps on the GPU (other streams or host threads) race on it.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "rq_objects.h"

namespace {

constexpr int64_t kMaxRays = RQ_NOALLOC_MAX_RAYS;

// Slices of the scratch array, each 256-byte aligned: primary hits (n), secondary rays and hits,
// shadow rays, occlusion bytes and compact-slot indices (n * spp each), and the device counters.
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kPrimHitsOff = 0;
constexpr size_t kSecOff = kPrimHitsOff + align256(sizeof(rq_hit) * kMaxRays);
constexpr size_t kSecHitsOff = kSecOff + align256(sizeof(rq_ray) * kMaxRays);
constexpr size_t kShadowOff = kSecHitsOff + align256(sizeof(rq_hit) * kMaxRays);
constexpr size_t kOccOff = kShadowOff + align256(sizeof(rq_ray) * kMaxRays);
constexpr size_t kCompOff = kOccOff + align256(kMaxRays);
constexpr size_t kCountersOff = kCompOff + align256(sizeof(int32_t) * kMaxRays);
constexpr size_t kScratchBytes = kCountersOff + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The fixed array as the GI pass's arena: each slot the fused pass uses maps to its slice; any
// other slot (octant binning, the unfused kernels, the bounce loop) is refused.
struct FixedArena final : rq::GiArena {
    rq_ctx* ctx;
    unsigned char* base;
    FixedArena(rq_ctx* c, unsigned char* b) : ctx(c), base(b) {}
    rq_status get(int slot, size_t bytes, void** out) override {
        size_t off = 0, cap = 0;
        switch (slot) {
            case rq::kSlotPrimaryHits: off = kPrimHitsOff, cap = sizeof(rq_hit) * kMaxRays; break;
            case rq::kSlotRays: off = kSecOff, cap = sizeof(rq_ray) * kMaxRays; break;
            case rq::kSlotHits: off = kSecHitsOff, cap = sizeof(rq_hit) * kMaxRays; break;
            case rq::kSlotShadowRays: off = kShadowOff, cap = sizeof(rq_ray) * kMaxRays; break;
            case rq::kSlotOccluded: off = kOccOff, cap = kMaxRays; break;
            case rq::kSlotCompactOf: off = kCompOff, cap = sizeof(int32_t) * kMaxRays; break;
            default: return rq::fail(ctx, RQ_ENOTSUP, "no-alloc GI pass: no fixed slice for this buffer");
        }
        if (bytes > cap) return rq::fail(ctx, RQ_EINVAL, "no-alloc GI pass: buffer beyond its fixed slice");
        *out = base + off;
        return RQ_OK;
    }
    unsigned long long* count() override {
        return reinterpret_cast<unsigned long long*>(base + kCountersOff);
    }
    unsigned long long* queue(int k) override {
        return reinterpret_cast<unsigned long long*>(base + kCountersOff) + 1 + k;
    }
    unsigned long long* live() override { return reinterpret_cast<unsigned long long*>(base + kCountersOff) + 4; }
};

}  // namespace

namespace rq {

// Called by rq_create with the context's device current: the device address of the fixed array
// (and so the module load that reserves it).  A failure is kept in the context and reported by
// rq_gi_frame_noalloc; the rest of the library does not depend on it.
void noalloc_resolve(rq_ctx* ctx) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        ctx->noalloc_base = nullptr;
        ctx->noalloc_error = std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e);
        return;
    }
    ctx->noalloc_base = p;
    ctx->noalloc_error.clear();
}

}  // namespace rq

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
    if (!ctx->noalloc_base)
        return rq::fail(ctx, RQ_ECUDA, "no-alloc scratch unavailable on this context: " + ctx->noalloc_error);
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    // sort_rays and unfused only rearrange the kernels (the pixels are the same); they need
    // buffers the fixed array does not hold, so the pass always runs the default fused form
    rq_gi_params pp = *p;
    pp.sort_rays = 0;
    pp.unfused = 0;
    FixedArena arena(ctx, static_cast<unsigned char*>(ctx->noalloc_base));
    return rq::gi_pass(ctx, sc, q, pp, primary, n, pixels4,
                       static_cast<cudaStream_t>(stream), false, nullptr, nullptr, arena);
}

}  // extern "C"
