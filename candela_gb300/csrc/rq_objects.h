// Library-internal object definitions shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/rq.h"
#include "bvh_build.h"
#include "rq_internal.h"

namespace rq {

// Grow-only device scratch buffers of a context (rq_ctx::scratch), one per purpose.  Calls that run
// one after another on the context's streams reuse them; each slot has one owner per kind of call,
// so that two kinds of work that may overlap on the GPU never share bytes.
enum ScratchSlot : int {
    kSlotStageRays = 0,      // host-buffer passes: primary rays staged on the device
    kSlotPrimaryHits = 1,    // GI / specular passes: primary hits
    kSlotRays = 2,           // secondary, reflection or probe rays
    kSlotHits = 3,           // their hits
    kSlotOccluded = 4,       // any-hit results of a pass
    kSlotShaded = 5,         // per-sample shading (unfused GI pass)
    kSlotStageOut = 6,       // host-buffer passes: pixels staged on the device; probe raw radiance
    kSlotShadowRays = 7,
    kSlotSampleOf = 8,       // GI bounce loop: sample index per compact slot
    kSlotTuneOut = 9,        // rq_autotune output
    kSlotRadiance = 10,      // GI bounce loop: first-hit radiance per slot
    kSlotCompactOf = 11,     // GI pass: compact slot of every sample
    kSlotBuild = 12,         // GPU BVH build arena
    kSlotCollideBoxes = 13,
    kSlotCollideOut = 14,
    kSlotThroughput = 15,    // GI bounce loop: path throughput per slot
    kSlotLossPerPixel = 16,  // rq_fwd / rq_bwd (16..29)
    kSlotLossPartials = 17,
    kSlotTapeHits = 18,
    kSlotTapeImage = 19,
    kSlotTapeGrad = 20,
    kSlotTapeTarget = 21,
    kSlotAdjContrib = 22,
    kSlotAdjKeysA = 23,
    kSlotAdjValsA = 24,
    kSlotAdjKeysB = 25,
    kSlotAdjValsB = 26,
    kSlotAdjHist = 27,
    kSlotAdjSegStart = 28,
    kSlotAdjSegEnd = 29,
    kSlotBatchDesc = 30,     // rq_batch descriptor table
    kSlotOctants = 31,       // GI pass with octant binning
    kSlotBounceRays = 32,    // GI bounce loop (32..35)
    kSlotBounceSlotA = 33,
    kSlotBounceSlotB = 34,
    kSlotBounceCounts = 35,
    kSlotProbeStageSh = 36,  // rq_probe_update on host buffers (36..39)
    kSlotProbeStageRaw = 37,
    kSlotProbeStageMap = 38,
    kSlotProbeStageOutSh = 39,
    kSlotBounced = 40,       // GI bounce loop: Bounced radiance per slot
    kNumScratchSlots = 41
};

}  // namespace rq

constexpr int kScratchSlots = rq::kNumScratchSlots;

struct rq_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;       // default stream of the context
    cudaStream_t pipe[2] = {nullptr, nullptr};  // host-buffer staging pipeline
    cudaEvent_t ev = nullptr;
    void* stage_in[2] = {nullptr, nullptr};
    void* stage_out[2] = {nullptr, nullptr};
    size_t stage_in_bytes[2] = {0, 0};
    size_t stage_out_bytes[2] = {0, 0};
    int* counters = nullptr;  // device work counters for persistent kernels (64 ints)
    void* scratch[kScratchSlots] = {};
    size_t scratch_bytes[kScratchSlots] = {};
    // device address of rq_gi_frame_noalloc's fixed array on this context's device (resolved by
    // rq_create), or null with the reason in noalloc_error
    void* noalloc_base = nullptr;
    std::string noalloc_error;
    std::string err;
};

struct rq_bvh {
    rq::BuildOutput out;
    int32_t layout = RQ_LAYOUT_BVH2_STACK;
};

struct rq_scene {
    rq_ctx* ctx = nullptr;
    int32_t layout = RQ_LAYOUT_BVH2_STACK;
    std::vector<float> h_nodes;  // host copy, used to validate entity lists
    int64_t n_nodes = 0, n_tris = 0, n_verts = 0;
    float4* d_nodes = nullptr;
    int4* d_tris = nullptr;
    float4* d_verts = nullptr;
    rq_entity* d_ents = nullptr;
    int32_t n_ents = 0;
    int32_t ents_cap = 0;
    int64_t bytes = 0;
    rq::SceneView view{};
    float4* d_tri_fast = nullptr;  // fast-mode triangle records (3 x float4 per triangle)
    float* d_albedo = nullptr;  // 3 floats per mesh id
    int32_t n_albedo = 0;
    // albedo textures (rq_scene_set_textures)
    int32_t* d_mesh_tex = nullptr;
    int32_t n_mesh_tex = 0;
    int4* d_tex = nullptr;
    uint32_t* d_texels = nullptr;
    float* d_srgb = nullptr;
    int64_t tex_bytes = 0;
    // host copies (validation and derived layouts)
    std::vector<int32_t> h_tris;
    std::vector<float> h_verts;
    std::vector<rq_entity> h_ents;
    // BVH8 with quantised boxes (built on request)
    bool bvh8 = false;
    uint4* d_b8nodes = nullptr;
    float4* d_b8tris = nullptr;
    int32_t* d_b8roots = nullptr;
    int32_t b8roots_cap = 0;
    int64_t b8_nodes = 0, b8_tris = 0, b8_bytes = 0;
    double b8_build_ms = 0.0;
    std::vector<int32_t> h_b8roots;  // per entity: BVH8 root (-1: none)
    std::vector<double> b8_bounds;   // per entity: object-space bounds its BVH8 root can box-test
    // BVH8 refit plan (rq_refit8.cu): node indices level by level from the roots down, the level
    // offsets, and a per-node FP32 box (6 floats) written during a refit; b8_bounds is recomputed
    // from the device roots after a refit
    int32_t* d_b8_order = nullptr;
    std::vector<int64_t> b8_level_off;
    float* d_b8box = nullptr;
    bool b8_bounds_stale = false;
    // top level over the entities (tlas.h); rebuilt with the entities and the BVH8
    float4* d_tlas = nullptr;
    int4* d_tlas_pre = nullptr;
    int64_t tlas_bytes = 0;
    int32_t tlas_nodes = 0, tlas_cullable = 0;
    // refit plan (node, object offset) bottom-up by level, and vertex -> (triangle, corner) lists
    bool refit_ready = false, adj_ready = false, host_stale = false;
    std::vector<int64_t> refit_level_off;
    int2* d_refit = nullptr;
    int32_t* d_adj_off = nullptr;
    int32_t* d_adj = nullptr;
    // autotuned launch variant per [layout][query kind] (-1 = default)
    int8_t tuned[4][2] = {{-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}};
    // GI compaction threshold used when rq_gi_params.compact_below is 0 (rq_gi_autotune); above 1 =
    // always compact
    float gi_compact_below = 2.0f;
};

namespace rq {

inline Materials materials_of(const rq_scene* sc) {
    return Materials{sc->d_albedo, sc->n_albedo, sc->n_mesh_tex, sc->d_mesh_tex, sc->d_tex, sc->d_texels,
                     sc->d_srgb};
}

rq_status fail(rq_ctx* ctx, rq_status s, const std::string& msg);
// Rebuilds the top level over the scene's entities (none below kTlasMinEntities entities).
rq_status rebuild_tlas(rq_scene* sc);
// Copies device-updated node and vertex buffers back to the host copies (and recomputes the BVH8
// root bounds after a BVH8 refit).
rq_status refresh_host(rq_scene* sc);
// Refits the scene's BVH8 to the current device vertex positions, topology kept (rq_refit8.cu).
rq_status refit_bvh8(rq_scene* sc, cudaStream_t st);
// Object-space bounds of each entity's BVH8 root children from host copies of the root nodes.
void bvh8_root_bounds(rq_scene* sc, const std::vector<uint32_t>& root_nodes);
rq_status cuda_fail(rq_ctx* ctx, cudaError_t e, const char* what);
// Resolves rq_opts (NULL = defaults) against the scene into a kernel configuration.
rq_status resolve_query(rq_ctx* ctx, const rq_scene* sc, const rq_opts* o, QueryConfig& q);
// Query work counters (2 x u64) inside the context's counter block.
inline unsigned long long* work_counters(rq_ctx* ctx) {
    return reinterpret_cast<unsigned long long*>(ctx->counters) + 8;
}
// Device counter of compact (active) secondary rays in a GI pass.
inline unsigned long long* frame_counter(rq_ctx* ctx) {
    return reinterpret_cast<unsigned long long*>(ctx->counters) + 12;
}
// Pixels per chunk of the shading phase of a GI frame on host buffers (each chunk's pixels are
// copied out while the next chunk is shaded).
constexpr int64_t kGiHostChunk = int64_t(1) << 18;
// Device status bits of the kernels (atomicOr), read by rq_device_status.
inline unsigned* status_word(rq_ctx* ctx) { return reinterpret_cast<unsigned*>(ctx->counters) + 30; }
// Ray-queue counter k (0..15) of the persistent kernels, inside the context's counter block.
inline unsigned long long* queue_counter(rq_ctx* ctx, int k) {
    return reinterpret_cast<unsigned long long*>(ctx->counters) + 16 + k;
}
// GPU build of one object's BVH2 (bvh_build_gpu.cu): the buffers build_bvh produces, from host
// input arrays, on the context's device.  RQ_OK, or a status with `why` set.
rq_status build_bvh_gpu(rq_ctx* ctx, const BuildInput& in, BuildOutput& out, std::string& why);
// BVH8 group-stack depths selectable by rq_opts.stack_depth (0 = the default).
constexpr int kBvh8Depths[3] = {48, 32, 24};
inline int bvh8_depth(int index) { return kBvh8Depths[(index >= 0 && index < 3) ? index : 0]; }
// The index of opts->stack_depth in kBvh8Depths (0 for 0 or NULL opts); RQ_EINVAL for any other depth.
rq_status depth_index_of(rq_ctx* ctx, const rq_opts* o, int& index);
// Status bit a BVH8 walk raises when its group stack overflows (bvh8::kStatusStackOverflow).
constexpr unsigned kStatusOverflowBit = 1u;

// Grow-only device scratch buffer of the context (slot < kScratchSlots).
rq_status scratch(rq_ctx* ctx, int slot, size_t bytes, void** out);

// Where a GI pass takes its intermediate buffers and its device counters: the context's grow-only
// scratch slots (rq_gi_frame), or fixed slices of a library array (rq_gi_frame_noalloc).
struct GiArena {
    virtual ~GiArena() = default;
    // A device buffer of at least `bytes` for `slot` (a ScratchSlot).
    virtual rq_status get(int slot, size_t bytes, void** out) = 0;
    // The device word that counts the pass's compact (active) secondary rays.
    virtual unsigned long long* count() = 0;
    // Ray-queue counter k (0..2) of the persistent traversal launches.
    virtual unsigned long long* queue(int k) = 0;
    // The device word that counts the primary rays with a hit (the compaction decision).
    virtual unsigned long long* live() = 0;
};
struct CtxGiArena final : GiArena {
    rq_ctx* ctx;
    explicit CtxGiArena(rq_ctx* c) : ctx(c) {}
    rq_status get(int slot, size_t bytes, void** out) override { return scratch(ctx, slot, bytes, out); }
    unsigned long long* count() override { return frame_counter(ctx); }
    unsigned long long* queue(int k) override { return queue_counter(ctx, k); }
    unsigned long long* live() override { return reinterpret_cast<unsigned long long*>(ctx->counters) + 13; }
};

// Resolves the device address of rq_gi_frame_noalloc's fixed array for the context (rq_noalloc.cu);
// called by rq_create with the context's device current.
void noalloc_resolve(rq_ctx* ctx);

// One GI / RTAO pass over n primary rays on stream st (rq_gi.cu): primary closest hits, secondary
// ray generation, the secondary traversal (+ shadow rays), shading and the per-pixel mean, with
// every intermediate buffer taken from `arena`.  h_prim / h_pix: host buffers (prim / pixels4 are
// then device staging buffers).  stats: add the ray counts to the context's frame counters.
rq_status gi_pass(rq_ctx* ctx, const rq_scene* sc, const QueryConfig& q, const rq_gi_params& p,
                  const rq_ray* prim, int64_t n, void* pixels4, cudaStream_t st, bool stats,
                  const rq_ray* h_prim, void* h_pix, GiArena& arena);

}  // namespace rq

#define RQ_CUDA(ctx, call)                                            \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return rq::cuda_fail((ctx), e_, #call); \
    } while (0)
