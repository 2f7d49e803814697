// Internal types shared by the host API (rq_api.cu) and the kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/rq.h"

namespace rq {

// Device view of an uploaded scene.  All buffers keep the reference byte layouts; derived
// layouts (compact triangle records, BVH8) are added next to them.
struct SceneView {
    const float4* nodes;      // stack: 4 float4 per node; stackless: 2 float4 per node
    int64_t n_nodes;
    const int4* tris;         // {i0, i1, i2, mesh}
    int64_t n_tris;
    const float4* verts;      // 2 float4 per vertex; .xyz of the first = position
    int64_t n_verts;
    const rq_entity* ents;
    int32_t n_ents;
    int32_t layout;           // RQ_LAYOUT_BVH2_STACK / RQ_LAYOUT_BVH2_STACKLESS
    int32_t all_identity;     // every entity's inverse matrix is exactly the identity
    int32_t pad;
    // BVH8 with quantised child boxes (rq_scene_build_bvh8): nodes (5 x uint4), triangle records
    // (4 x float4), BVH8 root per entity (-1: none).
    const uint4* b8_nodes;
    const float4* b8_tris;
    const int32_t* b8_roots;
    // Fast-mode triangle records in reference triangle order: {v0, mesh}, {e1, 0}, {e2, 0}.
    const float4* tri_fast;
    // Optional device-side ray count: when set, a launch over n rays processes only the first
    // min(n, *ray_count) (used for compacted secondary rays whose count is known on the device).
    const unsigned long long* ray_count;
    // Top level over the entities (tlas.h; NULL = walk every entity): pre-order nodes (2 x float4),
    // per-entity prefix counts (int4), per-ray margin factor.
    const float4* tlas;
    const int4* tlas_pre;
    float tlas_margin;
    int32_t tlas_pad;
    // Optional copy target of the rays (BVH8 one-thread-per-ray launches): each ray loaded is also
    // stored here, so a launch that reads rays from pinned host memory leaves a device copy for the
    // kernels after it.
    rq_ray* ray_copy;
};

// Per-mesh surface data of the shading kernels: ModelColor per mesh id, and optional albedo
// textures (rq_scene_set_textures): per mesh a texture index (-1: ModelColor), per texture
// {first texel, width, height, flags (1 = sRGB colour channels, 2 = clamp to edge)}, RGBA8 texels,
// and the sRGB decoding table of the 256 byte values.
struct Materials {
    const float* albedo;
    int32_t n_albedo;
    int32_t n_mesh_tex;
    const int32_t* mesh_tex;
    const int4* tex;
    const uint32_t* texels;
    const float* srgb;
};

// The view a query runs on: RQ_FLAG_ENTITY_LOOP walks every entity in turn.
inline SceneView entity_view(const SceneView& s, int flags) {
    SceneView v = s;
    if (flags & RQ_FLAG_ENTITY_LOOP) v.tlas = nullptr;
    return v;
}

// Query configuration resolved by the host API.
struct QueryConfig {
    int32_t layout;
    int32_t mode;
    int32_t tie_lower;   // 1 = lower-index rule
    int32_t flags;
    int32_t block;
    unsigned long long* counters;  // non-null: accumulate node visits / triangle tests here
    unsigned* status;              // device status bits (stack overflow, iteration budget)
    int32_t variant_closest;       // index into kLaunchVariants (-1 = default)
    int32_t variant_any;
};

// Compiled launch variants of the traversal kernels: threads per block, minimum resident blocks
// per SM (the register cap follows from it), the persistent ray-queue form, and the BVH8 group-stack
// depth (0 = the default, 48; the BVH2 walks keep the reference's 64-entry stack whatever it says).
struct LaunchVariant {
    int32_t block, min_blocks, persistent, depth;
};
constexpr int kNumLaunchVariants = 10;
extern const LaunchVariant kLaunchVariants[kNumLaunchVariants];
// The one-thread-per-ray variant with the same block size and occupancy target as variant v
// (v itself when it is not persistent).
int non_persistent_variant(int v);

// Fast-mode triangle records from the triangle and vertex buffers (rq_kernels.cu).
cudaError_t launch_tri_fast(const int4* tris, int64_t n_tris, const float4* verts, float4* out,
                            cudaStream_t st);

// Kernel launchers (rq_kernels.cu).  Return cudaGetLastError() after the launch.
// `queue` (nullable) is a device ray counter for the persistent kernels; without one (or with
// RQ_FLAG_NO_PERSISTENT) one thread runs per ray.
cudaError_t launch_closest(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                           rq_hit* hits, unsigned long long* queue, cudaStream_t st);
cudaError_t launch_anyhit(const SceneView& s, const QueryConfig& q, const rq_ray* rays, int64_t n,
                          uint8_t* occluded, unsigned long long* queue, cudaStream_t st);

// One query of a batch (device descriptor).
struct QueryDesc {
    SceneView s;
    const rq_ray* rays;
    rq_hit* hits;
    uint8_t* occ;
    int64_t n;
    int64_t base;   // first global work index of this query
    int32_t kind;   // 0 = closest, 1 = any
    int32_t flags;
    int32_t tie_lower;
    int32_t pad;
};
constexpr int kMaxBatchQueries = 1024;
// Batch launch variants (block, min blocks per SM) and layout families.
constexpr int kNumBatchVariants = 4;
extern const LaunchVariant kBatchVariants[kNumBatchVariants];
enum BatchFamily { kFamilyBvh8 = 0, kFamilyStrict = 1, kFamilyFast = 2 };
// BVH8 group-stack depths of the batch kernel (index into bvh8::kStackDepths: 48, 32, 24).
constexpr int kNumBatchDepths = 3;
// One persistent launch over every query (rq_kernels.cu).  queue is zeroed by the caller.
// depth_index selects the BVH8 family's group-stack depth.
// total_c >= 0 (BVH8 family, no scene with a top level, the closest-hit queries' descriptors first
// with total_c rays in all): the lane-refill kernel, which takes two queue counters (queue[0],
// queue[1]); otherwise the one-ray-per-thread kernel (one counter).
cudaError_t launch_batch(const QueryDesc* d_desc, int nq, int64_t total, int family, int variant,
                         unsigned long long* queue, unsigned* status, cudaStream_t st, int depth_index = 0,
                         int64_t total_c = -1);

}  // namespace rq
