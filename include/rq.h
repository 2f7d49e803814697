/* rq.h — C ABI of the GB300 ray-query engine (librq.so).
 *
 * A drop-in for the ray-query path of the Candela renderer (swr06/Candela): the SAH BVH
 * constructor, its flattened node / triangle / vertex buffers and the closest-hit / any-hit ray
 * API.  Every entry point names the reference interface it replaces.  Plain C types only: no
 * CUDA, C++ or torch types cross this boundary; `stream` arguments are cudaStream_t passed as
 * void* (NULL = the CUDA default stream, as everywhere in the CUDA runtime).
 *
 * Conventions
 *  - Every call returns rq_status.  On failure rq_last_error(ctx) holds a message.
 *  - Buffers are device pointers unless RQ_FLAG_HOST_BUFFERS is set in rq_opts.flags, in which
 *    case the library stages them through device memory itself (copies inside the call).
 *  - Calls are ordered on the given stream; results are ready when the stream is synchronised.
 *    With RQ_FLAG_HOST_BUFFERS the call synchronises before returning.
 *  - One rq_ctx per host thread.  One GPU per context.  There is no CPU fallback: a context can
 *    only be created on a CUDA device.
 *  - Queries through one context share its device work counters: do not run them concurrently
 *    on different streams (use one context per concurrent stream).
 */
#ifndef RQ_H_
#define RQ_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RQ_ABI_VERSION 3

typedef enum rq_status {
    RQ_OK = 0,
    RQ_EINVAL = 1,   /* bad argument or malformed buffer (the reference throws C strings) */
    RQ_ENOMEM = 2,   /* device or host allocation failed */
    RQ_ECUDA = 3,    /* CUDA runtime error */
    RQ_EBUDGET = 4,  /* a device loop ran out of its iteration budget (see rq_opts) */
    RQ_ENOTSUP = 5,  /* combination not supported (e.g. BVH8 query before rq_scene_build_bvh8) */
    RQ_ESTATE = 6    /* object used in the wrong state */
} rq_status;

/* ---- Buffer formats (byte-compatible with the reference) -------------------------------- */

/* Candela::Vertex, Source/Core/Utils/Vertex.h:7-12 (32 bytes).  Traversal reads position.xyz;
 * shading reads the half2x16-packed normal in normal_tangent_data[0..1] (UnpackNormal,
 * Shaders/Intersectors/Include/TraverseBVHStack.glsl:417-420). */
typedef struct rq_vertex {
    float position[4];
    uint32_t normal_tangent_data[3];
    uint32_t texcoords;
} rq_vertex;

/* BVH::Triangle, Source/Core/BVH/BVHConstructor.h:78-83: {i0, i1, i2, mesh id} (16 bytes). */
typedef struct rq_triangle {
    int32_t packed[4];
} rq_triangle;

/* BVH::FBounds / FlattenedStackNode, BVHConstructor.h:61-76 (64 bytes).  min[3] holds the child
 * kind as int bits: -1 = internal, else (first triangle << 4) | count.  max[3] holds the child's
 * node index (relative to the object's first node) for internal children. */
typedef struct rq_fbounds {
    float min[4];
    float max[4];
} rq_fbounds;
typedef struct rq_node_stack {
    rq_fbounds left, right;
} rq_node_stack;

/* BVH::FlattenedNode, BVHConstructor.h:66-70 (32 bytes): DFS pre-order, min[3] = leaf data or
 * -1, max[3] = escape link (-1 ends the walk). */
typedef struct rq_node_stackless {
    float min[4];
    float max[4];
} rq_node_stackless;

/* Candela::BVHEntity, Source/Core/BVH/Intersector.h:43-49 (192 bytes).  Matrices are glm
 * column-major.  data[0] = emissive amount (float bits), data[1] = alpha (float bits). */
typedef struct rq_entity {
    float model[16];
    float inverse[16];
    int32_t node_offset;
    int32_t node_count;
    int32_t data[14];
} rq_entity;

/* A ray (32 bytes).  The reference's IntersectRay(origin, direction) uses tmin = 0 and a scene
 * TMax of 1000000.0 (TraverseBVHStack.glsl:331); rays with !(tmax > tmin) are inactive. */
typedef struct rq_ray {
    float origin[3];
    float tmin;
    float dir[3];
    float tmax;
} rq_ray;

/* Closest-hit result (32 bytes): the reference's TUVW = (t, u, v, w) with u + v + w = 1 and u
 * weighting vertex i0 (ComputeBarycentrics, TraverseBVHStack.glsl:150-166), plus the mesh id,
 * global triangle index and entity index.  A miss is t = u = v = w = -1, tri = mesh = entity =
 * -1.  iters = BVH nodes visited, summed over entities (the last entity's under
 * RQ_FLAG_REF_COMPAT). */
typedef struct rq_hit {
    float t, u, v, w;
    int32_t tri, mesh, entity, iters;
} rq_hit;

typedef enum rq_layout {
    RQ_LAYOUT_DEFAULT = 0,         /* the scene's own layout */
    RQ_LAYOUT_BVH2_STACK = 1,      /* FlattenedStackNode, stack traversal */
    RQ_LAYOUT_BVH2_STACKLESS = 2,  /* FlattenedNode, skip-link traversal */
    RQ_LAYOUT_BVH8Q = 3            /* 8-wide BVH with 8-bit quantised child boxes (derived) */
} rq_layout;

typedef enum rq_mode {
    RQ_MODE_STRICT = 0,  /* reference arithmetic: no FMA, IEEE division, GLSL min/max,
                            reference traversal order: bit-exact with the CPU restatement */
    RQ_MODE_FAST = 1     /* FMA, reciprocal-multiply slab test, compact triangle records */
} rq_mode;

typedef enum rq_tie {
    RQ_TIE_LOWER_INDEX = 0, /* equal t: the lower triangle index wins (order independent) */
    RQ_TIE_FIRST_FOUND = 1  /* equal t: the first hit found in traversal order wins (reference) */
} rq_tie;

enum {
    RQ_FLAG_REF_COMPAT = 1,          /* reproduce IntersectScene's `TriangleIdx > 0` test
                                        (TraverseBVHStack.glsl:351): a hit on triangle 0 is
                                        reported with t = u = v = w = -1; and its Iters, which
                                        is the last walked entity's count (one `out int Iters`
                                        serves every walk, :337-349) instead of the sum (BVH2
                                        strict and fast walks; BVH8 iters count BVH8 nodes) */
    RQ_FLAG_IGNORE_TRANSPARENT = 2,  /* IntersectSceneIgnoreTransparent: skip entities with
                                        alpha < 0.99 (TraverseBVHStack.glsl:368-413) */
    RQ_FLAG_HOST_BUFFERS = 4,        /* ray/hit pointers are host memory */
    RQ_FLAG_NO_PERSISTENT = 8,       /* one thread per ray instead of the persistent kernel */
    RQ_FLAG_COUNT = 16,              /* accumulate node visits and triangle tests into the
                                        context's work counters (rq_counters_read) */
    RQ_FLAG_ENTITY_LOOP = 32         /* walk every entity in turn (the reference's loop) instead
                                        of skipping the ones the top-level BVH rules out; same
                                        results either way (for BVH8 closest hits, same hits
                                        with a different iters: see rq_tlas_info) */
};

typedef struct rq_opts {
    int32_t layout;      /* rq_layout */
    int32_t mode;        /* rq_mode */
    int32_t tie;         /* rq_tie */
    int32_t flags;       /* RQ_FLAG_* */
    /* Launch variant: (block_size, min_blocks, persistent) must name one of the compiled variants
     * listed by rq_autotune; all zero = the variant rq_autotune picked for this scene, layout and
     * query kind, else the default (128 threads, one thread per ray). */
    int32_t block_size;
    int32_t min_blocks;  /* minimum resident blocks per SM the kernel was compiled for */
    int32_t persistent;  /* 1 = persistent ray-queue kernel (strict mode, every layout) */
    int32_t stack_depth; /* BVH8 group-stack entries per lane of that variant: 0 (= 48), 32 or 24; a
                            walk that would go deeper raises status bit 0 (rq_device_status) and
                            returns the best hit found so far */
} rq_opts;

/* ---- Context ---------------------------------------------------------------------------- */

typedef struct rq_ctx rq_ctx;

int rq_abi_version(void);
const char* rq_status_string(rq_status s);

/* Creates a context on CUDA device `device`.  Fails with RQ_ECUDA when no device is present. */
rq_status rq_create(int device, rq_ctx** out);
rq_status rq_destroy(rq_ctx* ctx);
const char* rq_last_error(const rq_ctx* ctx);

/* Work counters accumulated by queries run with RQ_FLAG_COUNT (the reference has only a
 * per-ray iteration count, TraverseBVHStack.glsl:319).  Synchronises the context's stream.
 * reset != 0 zeroes them after reading. */
typedef struct rq_counters {
    int64_t node_visits;
    int64_t triangle_tests;
} rq_counters;
rq_status rq_counters_read(rq_ctx* ctx, rq_counters* out, int reset);

/* Status bits raised by kernels since the last reset (synchronises the device): bit 0 = a BVH8
 * traversal stack overflowed, bit 1 = a traversal exhausted its node-visit budget.  Such rays
 * return the best hit found so far; the bits make that visible.  0 = clean. */
rq_status rq_device_status(rq_ctx* ctx, uint32_t* bits, int reset);

/* Read bandwidth of the context's device in GB/s (no counterpart in the reference): 16-byte loads
 * that bypass L1, from every SM, over a device buffer of `bytes` (allocated and freed inside the
 * call), re-read `reps` times (up to 50 passes per launch) after three warm-up passes.  A buffer well under the
 * L2 size measures L2 read bandwidth, the roof of the traversal kernels, whose scenes stay
 * L2-resident; one well above it measures HBM.  Synchronises the context's stream. */
rq_status rq_measure_read_gbs(rq_ctx* ctx, int64_t bytes, int32_t reps, double* gbs);

/* ---- BVH construction (host) ------------------------------------------------------------ */

typedef struct rq_bvh rq_bvh;

typedef struct rq_build_opts {
    int32_t leaf_size;      /* MAX_TRIANGLES_PER_LEAF; 0 = 2 (BVHConstructor.cpp:49); 1..15 */
    int32_t swap_children;  /* stackless: OPTIMIZE_FOR_AVERAGE_CASE random child swap
                               (BVHConstructor.cpp:599-609), driven by mt19937(swap_seed) */
    uint32_t swap_seed;
    int32_t n_threads;      /* 0 = all hardware threads */
} rq_build_opts;

typedef struct rq_bvh_info {
    int64_t n_nodes;       /* node array length (LastNodeIndex + 1) */
    int64_t n_nodes_used;  /* stack layout: internal nodes written; stackless: n_nodes */
    int64_t n_tris;
    int32_t node_bytes;    /* 64 (stack) or 32 (stackless) */
    int32_t layout;        /* rq_layout */
    int64_t leaf_count;
    int64_t split_fails;
    double build_ms;
} rq_bvh_info;

/* Replaces BVH::BuildBVH(const Object&, vector<FlattenedStackNode|FlattenedNode>&,
 * vector<Vertex>&, vector<Triangle>&, int) (BVHConstructor.h:86-87, BVHConstructor.cpp:951-1108)
 * for one object whose meshes are already merged: `indices` are object-global vertex indices (3
 * per triangle), `mesh_ids` one per triangle (NULL = 0), `tri_offset` the global index of the
 * object's first triangle.  Output buffers are byte-identical to the reference constructor's
 * (stackless with swap_children = 0 equals the reference with UsesStackless = false). */
rq_status rq_build_bvh(const rq_vertex* verts, int64_t n_verts, const uint32_t* indices,
                       int64_t n_indices, const int32_t* mesh_ids, int32_t tri_offset,
                       rq_layout layout, const rq_build_opts* opts, rq_bvh** out);
/* The same build on the GPU of `ctx` (no counterpart in the reference, whose constructor runs
 * on the host only): the buffers rq_build_bvh returns, byte for byte, from the same host arrays;
 * opts->n_threads is ignored.  The result is an ordinary rq_bvh (host buffers). */
rq_status rq_build_bvh_gpu(rq_ctx* ctx, const rq_vertex* verts, int64_t n_verts, const uint32_t* indices,
                           int64_t n_indices, const int32_t* mesh_ids, int32_t tri_offset,
                           rq_layout layout, const rq_build_opts* opts, rq_bvh** out);
rq_status rq_bvh_info_get(const rq_bvh* bvh, rq_bvh_info* info);
/* Borrowed pointers, valid until rq_bvh_free. */
rq_status rq_bvh_nodes(const rq_bvh* bvh, const void** nodes, int64_t* n_nodes);
rq_status rq_bvh_triangles(const rq_bvh* bvh, const rq_triangle** tris, int64_t* n_tris);
void rq_bvh_free(rq_bvh* bvh);

/* Host-side BVH8 derivation for one object (what rq_scene_build_bvh8 does per object), for
 * inspection and offline use.  `nodes` is a BVH2 buffer of `layout`; the object occupies nodes
 * [node_offset, node_offset + node_count).  Output: 80-byte nodes (root = node 0) and 64-byte
 * triangle records {v0, tri}, {e1, mesh}, {e2, 0}, {n, 0}; the node format is documented in
 * candela_gb300/csrc/bvh8.h.  No counterpart in the reference. */
typedef struct rq_bvh8 rq_bvh8;
rq_status rq_build_bvh8(rq_layout layout, const void* nodes, int64_t n_nodes,
                        const rq_triangle* tris, int64_t n_tris, const rq_vertex* verts,
                        int64_t n_verts, int32_t node_offset, int32_t node_count, rq_bvh8** out);
rq_status rq_bvh8_buffers(const rq_bvh8* b, const uint32_t** nodes, int64_t* n_nodes,
                          const float** tri_records, int64_t* n_records);
void rq_bvh8_free(rq_bvh8* b);

/* ---- Scene upload ----------------------------------------------------------------------- */

typedef struct rq_scene rq_scene;

/* Replaces RayIntersector<T>::BufferData (Intersector.h:321-351) plus BufferEntities
 * (:226-239): copies the global vertex / triangle / node buffers and the entity list to the
 * device.  `layout` is RQ_LAYOUT_BVH2_STACK or RQ_LAYOUT_BVH2_STACKLESS and says what `nodes`
 * holds.  Every link, leaf range and vertex index is validated on the host first (RQ_EINVAL on a
 * malformed buffer), so the kernels never read out of bounds.  The caller keeps ownership of the
 * host arrays. */
rq_status rq_scene_create(rq_ctx* ctx, rq_layout layout, const rq_vertex* verts, int64_t n_verts,
                          const rq_triangle* tris, int64_t n_tris, const void* nodes,
                          int64_t n_nodes, const rq_entity* ents, int32_t n_ents,
                          rq_scene** out);
/* Runs the same host validation as rq_scene_create without touching a device (no context needed):
 * RQ_OK, or RQ_EINVAL with the first problem found written to msg. */
rq_status rq_scene_validate(rq_layout layout, const rq_vertex* verts, int64_t n_verts,
                            const rq_triangle* tris, int64_t n_tris, const void* nodes,
                            int64_t n_nodes, const rq_entity* ents, int32_t n_ents, char* msg,
                            size_t msg_len);
/* Replaces RayIntersector<T>::PushEntities + BufferEntities (Intersector.h:200-239). */
rq_status rq_scene_set_entities(rq_scene* scene, const rq_entity* ents, int32_t n_ents);
/* Derives an 8-wide BVH with 8-bit conservatively quantised child boxes (RQ_LAYOUT_BVH8Q) from
 * the scene's BVH2 buffers, for every object its entities reference, and uploads it.  Queries with
 * RQ_LAYOUT_BVH8Q test leaves with the strict FP32 triangle arithmetic and the lower-index tie
 * rule, so their hits equal RQ_LAYOUT_BVH2_STACK strict hits (iters then counts BVH8 nodes).
 * Needs BVH2 leaves of at most 4 triangles (RQ_ENOTSUP otherwise).  Rebuilt automatically by
 * rq_scene_set_entities once enabled.  No counterpart in the reference. */
typedef struct rq_bvh8_info {
    int64_t nodes, triangles, bytes, bvh2_nodes;
    double build_ms;
} rq_bvh8_info;
rq_status rq_scene_build_bvh8(rq_scene* scene, rq_bvh8_info* info);
/* Device bytes held by the scene (all layouts built so far). */
rq_status rq_scene_bytes(const rq_scene* scene, int64_t* bytes);
/* Top level over the entities, built with the entities (and rebuilt with the BVH8) when a scene
 * has at least 4 of them.  It replaces nothing in the reference's results: IntersectScene walks
 * every entity in turn (TraverseBVHStack.glsl:337-349); queries here walk, in the same order and
 * with the same running TMax, only the entities whose world box (the entity's BVH root mapped by
 * the inverse of its inverse matrix, widened by a margin that covers float rounding) the ray
 * meets before TMax, and count one iteration for each entity passed over (the root visit the
 * loop would have made).  Hits, ties and iteration counts therefore equal the loop's
 * (RQ_FLAG_ENTITY_LOOP runs the loop itself).  The one exception is RQ_LAYOUT_BVH8Q closest
 * hits: these take their candidates nearest box first and drop the ones that start beyond the
 * running TMax.  The hit is the same, because it is the lexicographic minimum of (t, triangle,
 * entity) in any order.  Only iters differs: BVH8 nodes visited plus one per entity not walked.
 * Entities whose walk tests triangles without a box
 * test first (a stack-layout root with a leaf child) or whose transform is singular are never
 * passed over.  Not maintained by rq_scene_update_positions: after it every entity is walked
 * until the entities or the BVH8 are set again. */
typedef struct rq_tlas_info {
    int32_t nodes;     /* 0: no top level (every entity is walked) */
    int32_t entities;
    int32_t cullable;  /* entities that can be passed over */
    int32_t reserved;
    int64_t bytes;
} rq_tlas_info;
rq_status rq_scene_tlas_info(const rq_scene* scene, rq_tlas_info* info);
rq_status rq_scene_destroy(rq_scene* scene);

/* ---- Queries ---------------------------------------------------------------------------- */

/* Closest hit for n rays.  Replaces IntersectRay(o, d, out TUVW, out Mesh, out TriangleIdx, ...)
 * / IntersectScene (TraverseBVHStack.glsl:327-366, 458-502; stackless
 * TraverseBVHStackless.glsl:280-319).  opts may be NULL (strict, lower-index ties). */
rq_status rq_closest(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays, int64_t n,
                     rq_hit* hits, const rq_opts* opts, void* stream);

/* Surface attributes of a hit (32 bytes), the outputs of the reference's GetData
 * (TraverseBVHStack.glsl:422-455) that its IntersectRay overloads return beside TUVW, Mesh and
 * TriangleIdx: normal = the normalised barycentric mix of the three vertices' half-packed normals
 * (UnpackNormal :417-420), albedo = the mesh's albedo texture at the interpolated half-packed UV
 * when it has one (rq_scene_set_textures), else its ModelColor (rq_scene_set_materials; 0.8 grey
 * for a mesh without an entry), emissive and alpha = the hit entity's Data[0] and Data[1].  A miss
 * (t < 0 or mesh < 0) gives normal = -1, albedo = 0, emissive = 0 as GetData does, and alpha = 0
 * (GetData returns before writing it). */
typedef struct rq_hit_attrib {
    float normal[3];
    float alpha;
    float albedo[3];
    float emissive;
} rq_hit_attrib;

/* GetData over n hit records (from rq_closest or any other source), stackless and stack scenes
 * alike: attribs[i] for hits[i].  RQ_FLAG_HOST_BUFFERS in opts: hits and attribs are host memory. */
rq_status rq_hit_attribs(rq_ctx* ctx, const rq_scene* scene, const rq_hit* hits, int64_t n,
                         rq_hit_attrib* attribs, const rq_opts* opts, void* stream);

/* Closest hit plus surface attributes for n rays: replaces the overloads IntersectRay(o, d, out
 * TUVW, out Mesh, out TriangleIdx, out Albedo, out Normal[, out Alpha[, out Iters]]) and
 * IntersectRayIgnoreTransparent (TraverseBVHStack.glsl:458-502; TraverseBVHStackless.glsl the
 * same), Albedo.xyz = attribs.albedo and Albedo.w = attribs.emissive as there.  The query is
 * rq_closest's with the same opts (RQ_FLAG_IGNORE_TRANSPARENT gives the IgnoreTransparent form),
 * followed by rq_hit_attribs over its hits. */
rq_status rq_closest_attribs(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays, int64_t n,
                             rq_hit* hits, rq_hit_attrib* attribs, const rq_opts* opts, void* stream);

/* Autotuner: times every compiled launch variant of the traversal kernel for `query` (0 =
 * closest hit, 1 = any hit) and `layout` on the caller's device rays (3 timed launches each, after
 * one warm-up), and records the fastest for the scene; later queries with an all-zero variant in
 * rq_opts use it.  The variants span threads per block, minimum resident blocks per SM, one thread
 * per ray or the persistent ray queue, and (BVH8 only) the group-stack depth.  out->ms[i] is
 * variant i's best time in ms (-1 = not applicable to the layout, -2 = its stack overflowed on
 * these rays, so it is never picked).  No counterpart in the reference (its traversal is one
 * shader with a fixed 64-entry stack, TraverseBVHStack.glsl:168-324). */
#define RQ_MAX_VARIANTS 10
typedef struct rq_tune_result {
    int32_t variant, block_size, min_blocks, persistent;
    int32_t n_variants;
    int32_t depth;  /* group-stack depth of the chosen variant (BVH8) */
    float ms[RQ_MAX_VARIANTS];
    int32_t block[RQ_MAX_VARIANTS], min_blocks_of[RQ_MAX_VARIANTS], persistent_of[RQ_MAX_VARIANTS];
    int32_t depth_of[RQ_MAX_VARIANTS];
} rq_tune_result;
rq_status rq_autotune(rq_ctx* ctx, rq_scene* scene, const rq_ray* rays, int64_t n, int32_t query,
                      rq_layout layout, rq_tune_result* out);

/* Any hit (occlusion) for n rays: occluded[i] = 1 when a triangle with tmin < t < tmax lies on the
 * ray.  Replaces float IntersectRay(o, d) / IntersectSceneOcclusion (TraverseBVHStack.glsl:
 * 509-682; stackless :463-579), with the per-ray tmax the per-BVH functions accept. */
rq_status rq_anyhit(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays, int64_t n,
                    uint8_t* occluded, const rq_opts* opts, void* stream);

/* FP64 verification of closest hits: for each hit, recomputes t and the barycentrics of the same
 * triangle in double precision (Moller-Trumbore on the entity-transformed ray) and writes
 * err2[2i] = |t - t64| / t64 and err2[2i+1] = max |w - w64| over the three weights (NaN for misses
 * and for hits the FP64 test rejects).  Device buffers.  This is the only FP64 code on the GPU. */
rq_status rq_verify_hits(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays,
                         const rq_hit* hits, int64_t n, float* err2, void* stream);

/* ---- Batched queries --------------------------------------------------------------------- */

/* One query of a batch: device rays in, device hits (kind 0, closest) or occlusion bytes (kind 1,
 * any hit) out, over any scene of the context. */
typedef struct rq_query {
    const rq_scene* scene;
    const rq_ray* rays;
    int64_t n;
    int32_t kind;  /* 0 = closest hit, 1 = any hit */
    int32_t reserved;
    rq_hit* hits;
    uint8_t* occluded;
} rq_query;

/* Runs every query in ONE persistent launch (a work queue over all queries' rays; a batch of
 * uneven sizes keeps every SM busy).  opts->layout: RQ_LAYOUT_BVH8Q (every scene needs its BVH8)
 * or 0 = each scene's BVH2 layout; opts->mode strict or fast.  Results equal per-query
 * rq_closest / rq_anyhit calls with the same options.  At most 1024 queries.  No counterpart in
 * the reference (it issues one dispatch per pass). */
rq_status rq_batch(rq_ctx* ctx, const rq_query* queries, int32_t n_queries, const rq_opts* opts,
                   void* stream);

/* A batch fixed at creation (descriptors uploaded once), replayed as a captured CUDA graph:
 * a memset of the work counter and the persistent launch.  The query buffers must stay valid, and
 * the scenes unchanged: setting entities, materials, the BVH8 or positions after creation leaves
 * the plan pointing at the old device arrays (create a new plan). */
typedef struct rq_batch_plan rq_batch_plan;
rq_status rq_batch_plan_create(rq_ctx* ctx, const rq_query* queries, int32_t n_queries,
                               const rq_opts* opts, rq_batch_plan** out);
rq_status rq_batch_plan_launch(rq_batch_plan* plan, void* stream);
/* Times every batch launch variant (block size x occupancy target, and for BVH8Q the group-stack
 * depth 48 / 32 / 24) for each usable layout family (BVH8Q when every scene has one, the BVH2
 * layouts) on the plan's own queries, keeps the fastest and re-captures the graph.  ms[i] = time
 * of combination i, described by family_of[i] (0 = BVH8Q, 1 = BVH2 strict, 2 = BVH2 fast),
 * block_of[i], min_blocks_of[i], depth_of[i]; -1 = not applicable, -2 = the stack overflowed. */
#define RQ_MAX_BATCH_COMBOS 16
typedef struct rq_batch_tune {
    int32_t family, block_size, min_blocks, n;
    int32_t depth;
    float ms[RQ_MAX_BATCH_COMBOS];
    int32_t family_of[RQ_MAX_BATCH_COMBOS], block_of[RQ_MAX_BATCH_COMBOS], min_blocks_of[RQ_MAX_BATCH_COMBOS];
    int32_t depth_of[RQ_MAX_BATCH_COMBOS];
} rq_batch_tune;
rq_status rq_batch_plan_autotune(rq_batch_plan* plan, int32_t allow_bvh8, rq_batch_tune* out);
rq_status rq_batch_plan_destroy(rq_batch_plan* plan);

/* ---- AABB collision queries ---------------------------------------------------------------- */

/* A world-space query box (xyz used; w ignored), the AABB that Collide.comp reads per entity. */
typedef struct rq_box {
    float min[4];
    float max[4];
} rq_box;
/* First overlap found for a query box: collided = 1, the entity index, the triangle's mesh id and
 * the triangle index; {0, -1, -1, -1} when the box overlaps nothing. */
typedef struct rq_collision {
    int32_t collided, entity, mesh, tri;
} rq_collision;

/* Box/triangle collision queries over the scene's BVH2.  Replaces CollideScene (Shaders/
 * Intersectors/Include/CollideBVHStack.glsl:301-323, CollideBVHStackless.glsl:225-247) as
 * dispatched by Collide.comp:34, and Physics::CollideBox / CollidePoint (Physics.cpp:176-228,
 * a point is the box point -/+ 0.01).  Each box is moved into every entity's object space by its
 * inverse matrix (the two corners, as the reference does) and the entity's BVH is walked: the
 * stack layout descends the overlapping children nearest-centre first (AABBAABBOverlapF), the
 * stackless layout follows the skip links; leaf triangles take the separating-axis test over the
 * nine edge axes.  Entities are tried in order and the first triangle found wins.  Default: the
 * nine distinct axes and the global triangle index.  RQ_FLAG_REF_COMPAT reproduces the
 * reference: axis 5 repeats cross(u2, f2) (the reference writes AxisUxFx[5] = cross(u2, f2) where
 * cross(u1, f2) belongs) and the stack walk reports the index within the leaf.
 * RQ_FLAG_HOST_BUFFERS: boxes/out are host memory.  Strict FP32 arithmetic; RQ_ENOTSUP for a
 * layout other than the scene's BVH2. */
rq_status rq_collide(rq_ctx* ctx, const rq_scene* scene, const rq_box* boxes, int64_t n,
                     rq_collision* out, const rq_opts* opts, void* stream);

/* ---- Diffuse GI / RTAO ------------------------------------------------------------------ */

/* Parameters of the GI / AO pass that consumes the queries (Shaders/DiffuseTrace.glsl:386-662). */
typedef struct rq_gi_params {
    int32_t spp;           /* secondary rays per primary hit */
    uint32_t seed;         /* sample-hash seed (e.g. the frame index) */
    float origin_offset;   /* secondary origin = P + N * offset (DiffuseTrace.glsl:445 uses 0.05) */
    float ray_tmax;        /* secondary tmax: 1e6 for GI, the AO radius for RTAO */
    int32_t normal_mode;   /* 0 = interpolated half-packed vertex normal (GetData), 1 = geometric */
    int32_t query;         /* 0 = closest-hit GI rays + Lambert shading, 1 = any-hit AO rays */
    int32_t shadow_rays;   /* GI only: 1 = sun visibility from an any-hit shadow ray per GI hit
                              (the reference reads a cascaded shadow map, DiffuseTrace.glsl:
                              325-366); 0 = unshadowed */
    float shadow_offset;   /* shadow origin = hit + N * offset */
    float sun_dir[3];      /* u_SunDirection: direction the light travels */
    float sun_color[3];    /* SUN_COLOR_DIFF */
    float sky_color[3];    /* radiance returned by a miss (the reference samples u_Skymap) */
    int32_t sort_rays;     /* rq_gi_frame: 1 = group active secondary rays by direction octant
                              before tracing (same results, more coherent warps) */
    int32_t unfused;       /* rq_gi_frame: 0 = ray generation and shading + accumulation one
                              thread per pixel; 1 = one thread per sample (same pixels) */
    int32_t bounces;       /* GI only: further bounces after each GI hit (u_SecondaryBounces of the
                              RT second-bounce loop, DiffuseTrace.glsl:502-536), 0..8; each adds
                              (GetDirect + emissive) x throughput (the product of the albedos on
                              the path), a miss adds 1.1 x sky x throughput (the loop's 2.2 x
                              skymap against the first bounce's 2.0) and ends the path.  With
                              RQ_FLAG_REF_COMPAT a bounce miss adds nothing, as the reference's
                              loop does (it tests the first bounce's t for the sky) */
    float compact_below;   /* rq_gi_frame: the secondary rays are traced compacted (active rays
                              only) when the fraction of primary rays with a hit is below this
                              value, else in place (one slot per sample, inactive slots included);
                              the fraction is counted on the device.  > 1 = always compact; 0 = the
                              scene's value from rq_gi_autotune (always compact until tuned).  The
                              pixels are the same either way; the bounce loop, sort_rays and
                              unfused always compact */
    int32_t pixel_format;  /* rq_gi_frame / rq_gi_frame_noalloc / rq_gi_autotune output pixels:
                              RQ_PIXELS_RGBA32F (0): 4 floats per pixel; RQ_PIXELS_RGBA16F (1): 4
                              IEEE binary16 values per pixel (8 bytes), the format of the
                              reference's output image (layout(rgba16f) o_OutputData,
                              DiffuseTrace.glsl:17), each the float pixel rounded to nearest, ties
                              to even */
} rq_gi_params;

enum { RQ_PIXELS_RGBA32F = 0, RQ_PIXELS_RGBA16F = 1 };

typedef struct rq_frame_stats {
    int64_t primary_rays, primary_hits;
    int64_t secondary_rays, secondary_hits;  /* active secondary rays and their hits (or occluded) */
    int64_t shadow_rays, shadow_occluded;
    int64_t bounce_rays, bounce_hits;        /* rays traced by rq_gi_params.bounces, their hits */
} rq_frame_stats;

/* Per-mesh albedo (rgb floats, indexed by the triangle's mesh id), the ModelColor of the
 * reference's TextureReferences buffer (Intersector.h:373-418, GetData :440-451).  Meshes without
 * an entry shade with albedo 0.8. */
rq_status rq_scene_set_materials(rq_scene* scene, const float* albedo_rgb, int32_t n_meshes);

/* An albedo texture (GLClasses/Texture.cpp): width x height RGBA8 texels, rows from v = 0 up,
 * 4 bytes per texel (alpha unused).  srgb = 1 decodes the colour channels from sRGB before
 * filtering (the GL_SRGB_ALPHA internal format), wrap 0 = GL_REPEAT, 1 = GL_CLAMP_TO_EDGE. */
typedef struct rq_texture {
    int32_t width, height;
    int32_t srgb, wrap;
    const uint8_t* rgba8;
} rq_texture;

/* Albedo textures per mesh (BVHTextureReferences[mesh].Albedo, Intersector.h:373-418): a mesh m
 * with mesh_texture[m] >= 0 shades with that texture at the hit's UV (GetData,
 * TraverseBVHStack.glsl:436-447: the vertices' half-packed texture coordinates weighted by the
 * barycentrics), sampled bilinearly at level 0 as texture() does in a compute shader; other meshes
 * keep their ModelColor.  The data are copied; n_meshes = 0 removes the textures.  The filter
 * weights are exact binary32 products here, where GL hardware rounds them to 8 fractional bits. */
rq_status rq_scene_set_textures(rq_scene* scene, const rq_texture* textures, int32_t n_textures,
                                const int32_t* mesh_texture, int32_t n_meshes);

/* Cosine-weighted secondary rays from primary hits: for primary ray i with a hit and k < spp,
 * out[i*spp + k] = {P + N*offset, 0, CosWeightedHemisphere(N, hash(seed, i*spp + k)), ray_tmax}
 * with N faced toward the incoming ray (DiffuseTrace.glsl:439-446, 486-488; Sampling.glsl:1-12);
 * other slots are inactive (tmax = -1).  Device buffers. */
rq_status rq_gi_raygen(rq_ctx* ctx, const rq_scene* scene, const rq_ray* primary,
                       const rq_hit* hits, int64_t n, const rq_gi_params* params, rq_ray* out,
                       void* stream);
/* Shadow rays toward -sun_dir from the hits of `rays` (inactive where there is no hit). */
rq_status rq_shadow_raygen(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays,
                           const rq_hit* hits, int64_t n, const rq_gi_params* params, rq_ray* out,
                           void* stream);
/* Lambert shading of secondary hits: out4[j] = (albedo*sun*lit*clamp(dot(N,-sun),0,1) +
 * albedo*emissive, AO) with AO = pow(clamp(t/2.4,0,1),1.23) (GetDirect DiffuseTrace.glsl:368-372,
 * :490-494); a miss gives (sky, 1); an inactive ray (0,0,0,0).  lit may be NULL (all lit). */
rq_status rq_shade(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays, const rq_hit* hits,
                   int64_t n, const uint8_t* lit, const rq_gi_params* params, float* out4,
                   void* stream);
/* Whole GI / RTAO pass for n primary rays (pixels): primary closest hit, secondary ray
 * generation, secondary queries (closest + optional shadow any-hit, or AO any-hit), shading, and
 * the per-pixel mean over spp written to pixels4 (rgb radiance, AO or visibility): n x 4 floats,
 * or n x 4 binary16 values with params->pixel_format = RQ_PIXELS_RGBA16F.  With
 * RQ_FLAG_HOST_BUFFERS in opts, `primary` and `pixels4` are host memory.  `stats` (nullable)
 * synchronises the stream to read the ray counts. */
rq_status rq_gi_frame(rq_ctx* ctx, const rq_scene* scene, const rq_ray* primary, int64_t n,
                      const rq_gi_params* params, const rq_opts* opts, float* pixels4,
                      rq_frame_stats* stats, void* stream);

/* GI-pass autotuner (no counterpart in the reference): runs rq_gi_frame on the caller's device
 * primary rays with the secondary rays compacted and in place (3 timed passes each after a
 * warm-up; pixels4 receives the pixels), and records the threshold for the scene: the frame's
 * fraction of primary hits when the in-place pass was faster (frames at least that full then run
 * in place), else 2 (always compact).  Passes with rq_gi_params.compact_below = 0 use it. */
typedef struct rq_gi_tune {
    float compact_below;  /* the threshold recorded */
    float live_fraction;  /* fraction of the frame's primary rays with a hit */
    float ms_compact, ms_in_place;
} rq_gi_tune;
rq_status rq_gi_autotune(rq_ctx* ctx, rq_scene* scene, const rq_ray* primary, int64_t n,
                         const rq_gi_params* params, const rq_opts* opts, float* pixels4, rq_gi_tune* out);

/* ---- Specular reflections ---------------------------------------------------------------- */

/* The world-trace path of SpecularTrace.glsl (:485-596 with u_FullRT or metallic surfaces):
 * per pixel, from the primary hit P with facing normal N and incident I = normalize(P - origin),
 * a reflection ray from P + N * mix(0.05, 0.1, clamp(1.4 R, 0, 1)) in the direction
 * StochasticReflectionDirection(I, N, 0.9 R) (:102-135: a mirror reflection below roughness
 * 0.01, else the first of up to 12 GGX half-vector samples (Sampling.glsl:63-83, sample scaled by
 * (0.8, 0.7)) above the surface reflected), traced with IntersectRay; a hit is lit by
 * SampleLighting (:420-425): albedo x sun_color x sun visibility + albedo x 2 x ambient (the
 * irradiance the probe volume would return) + albedo x emissive; a miss sees
 * sky x mix(1.4, 2.65, R) (:435-437).  Non-finite radiance becomes 0 with t = -1, then radiance is
 * clamped to [0, 6]; out4 = (radiance, t / 48) (TransformReflectionTransversal), t = -1 for a
 * miss; pixels whose primary ray misses get 0.  Samples come from the counter-based hash of the GI
 * pass (the reference's fract-sin hash2 depends on the driver's sin). */
typedef struct rq_specular_params {
    uint32_t seed;
    float roughness;      /* PBR.x of the shaded surfaces */
    float ray_tmax;
    int32_t normal_mode;  /* as rq_gi_params */
    int32_t shadow_rays;  /* 1 = sun visibility from an any-hit shadow ray (GetDirectShadow) */
    float shadow_offset;
    float sun_dir[3];
    float sun_color[3];   /* SUN_COLOR_SPEC */
    float sky_color[3];   /* u_SkyCube sample */
    float ambient[3];     /* SampleProbes stand-in */
} rq_specular_params;
/* With RQ_FLAG_HOST_BUFFERS in opts, `primary` and `out4` are host memory. */
rq_status rq_specular_frame(rq_ctx* ctx, const rq_scene* scene, const rq_ray* primary, int64_t n,
                            const rq_specular_params* params, const rq_opts* opts, float* out4,
                            void* stream);

/* ---- Radiance probe volume ----------------------------------------------------------------- */

/* One frame of UpdateRadianceProbes.glsl (dispatched by ProbeGI::UpdateProbes, ProbeGI.cpp:
 * 162-238) over a grid of gx x gy x gz probes, probe p = (z * gy + y) * gx + x at
 * origin + (2 (x, y, z) / grid - 1) * size.  Per probe: one closest-hit ray in a uniformly
 * distributed direction (LambertBRDF normalised, :351-372); a miss sees
 * sky x 2.2 x clamp(dir.y, 0, 1), a hit max(albedo x sun_color x sun visibility x
 * clamp(dot(N, -sun_dir), 0, 1), 0) + albedo x emissive (:140-144, :440-450) plus the previous
 * volume's irradiance at the hit, SampleProbes(P + 0.001 N, N) x 0.999 x albedo (:190-237,
 * :462-467: trilinear over the 8 surrounding probes of the previous volume, each weighted by
 * clamp(dot(N, dir to probe), 0, 1)^2 and renormalised, L1 spherical harmonics evaluated at N).
 * The radiance is encoded as L1 SH (SphericalHarmonics.glsl EncodeSH); where the probe position
 * reprojects into the previous volume (at prev_origin), the SH, the raw radiance and this probe's
 * depth moments are blended with the previous frame's by min(1 - 1/frames, 0.98) when temporal
 * (:480-509), and the SH is packed (PackSH: 6 snorm16 pairs scaled by the largest coefficient;
 * word 7 = accumulated frames).
 *
 * Buffers, probe-major: prev_sh / out_sh 8 uint32 per probe (the u_PrevFrameSH / o_SHOutput
 * A.xyzw, B.xyzw texels), prev_raw / out_raw 4 floats per probe (radiance, 0: the o_CurrentRaw
 * texel, kept in float32 where the reference stores r11f_g11f_b10f, :17-18; with
 * RQ_FLAG_REF_COMPAT rounded to what that format holds, the GL conversion with ties to even, so
 * the next frame blends what the reference blends), probe_map 64 x 2 floats per probe
 * (the 8x8 octahedral depth / depth^2 map, MapData), updated in place at the pixel the ray's
 * direction maps to.  prev_sh and out_sh, and prev_raw and out_raw, must not overlap.
 * Differences from the shader, each deliberate: the map of probe (x, y, z) starts at p * 64 (the
 * shader's Get1DIdx adds gx where it means x, :68, so the probes of a row race on one map); the
 * sun visibility comes from an any-hit shadow ray (the shader reads cascaded shadow maps); the sky
 * is a constant colour (u_Skymap); directions come from the counter-based hash of the GI pass
 * (dimensions 0 and 1 of the probe index) with sin(acos c) = sqrt(1 - c^2) and the cube-root
 * radius, which normalisation removes, left out; out-of-range texel reads return 0 (robust image
 * access); packSnorm2x16 rounds half to even and packs NaN as 0 (GLSL leaves both open). */
typedef struct rq_probe_params {
    int32_t grid[3];       /* u_Resolution */
    float origin[3];       /* u_BoxOrigin */
    float prev_origin[3];  /* u_PreviousOrigin: where prev_sh / prev_raw were written */
    float size[3];         /* u_Size (half extent) */
    uint32_t seed;         /* per-frame seed of the direction samples */
    int32_t temporal;      /* u_Temporal */
    int32_t normal_mode;   /* as rq_gi_params */
    int32_t shadow_rays;   /* 1 = any-hit shadow ray toward the sun, 0 = every hit lit */
    float shadow_offset;   /* shadow ray origin = hit + N * shadow_offset */
    float ray_tmax;        /* 1e6 in the shader */
    float sun_dir[3];
    float sun_color[3];    /* SUN_COLOR_PROBES */
    float sky_color[3];    /* u_Skymap sample */
} rq_probe_params;
/* With RQ_FLAG_HOST_BUFFERS in opts, every buffer is host memory. */
rq_status rq_probe_update(rq_ctx* ctx, const rq_scene* scene, const rq_probe_params* params,
                          const uint32_t* prev_sh, const float* prev_raw, float* probe_map,
                          uint32_t* out_sh, float* out_raw, const rq_opts* opts, void* stream);

/* ---- Differentiation: depth + Lambert adjoint w.r.t. vertex positions ---------------------- */

/* No counterpart in the reference (its GI is not differentiable).  Per primary ray i the forward
 * pass renders image[i] = (depth, radiance): depth = closest-hit t (strict traversal), radiance =
 * albedo * sun_color * lit * max(dot(N, -sun_dir), 0) with N the geometric normal of the hit
 * triangle faced toward the ray and lit from an optional any-hit shadow ray (visibility is
 * treated as constant).  The loss is sum over hit pixels of w_depth*(depth - target.x)^2 +
 * w_radiance*(radiance - target.y)^2, reduced in FP64 in a fixed order; misses contribute 0.
 * rq_bwd writes dloss/dposition for every vertex: per-hit closed-form derivatives of t and of the
 * Lambert term, reduced deterministically (pixels sorted by triangle with an integer counting
 * sort, per-triangle sums in pixel order, per-vertex sums over a fixed vertex->triangle list): no
 * floating-point atomics, so gradients are bit-reproducible.  Entities must be identities. */
typedef struct rq_diff_params {
    float sun_dir[3];
    float sun_color;
    float albedo;
    float w_depth, w_radiance;
    int32_t shadow_rays;
    float shadow_offset;
    int32_t recompute;  /* 1 = keep no hit records: rq_bwd re-traces the primary (and shadow) rays */
    int32_t layout;     /* 0 = the scene's BVH2 (strict walk), RQ_LAYOUT_BVH8Q = the BVH8 (same hits;
                           refitted by rq_scene_update_positions) */
    int32_t reserved;
} rq_diff_params;

typedef struct rq_tape rq_tape;

/* rays: n device rays (must stay valid until rq_tape_free when recompute = 1); target2 / image2:
 * n x 2 device floats (image2 written); loss: host double (nullable; reading it synchronises). */
rq_status rq_fwd(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays, int64_t n,
                 const float* target2, const rq_diff_params* params, float* image2, double* loss,
                 rq_tape** tape, void* stream);
/* grad_xyz: n_verts x 3 device floats, overwritten with dloss/dposition. */
rq_status rq_bwd(rq_ctx* ctx, rq_tape* tape, float* grad_xyz, void* stream);
rq_status rq_tape_free(rq_tape* tape);
/* Device bytes the tape holds (hit records unless recompute, plus dloss/dimage). */
rq_status rq_tape_bytes(const rq_tape* tape, int64_t* bytes);

/* Replaces every vertex position (xyz: n_verts x 3 device floats) and refits the BVH2 boxes with
 * the topology kept (exact min/max per level, bottom-up), and the BVH8 when one is built: its
 * triangle records are recomputed and its quantised child boxes refitted level by level, rounded
 * outward onto each node's new grid, so its hits stay those of the strict BVH2 walk.  Stack layout
 * scenes.  The top level over the entities is not refitted: every entity is walked until the
 * entities or the BVH8 are set again. */
rq_status rq_scene_update_positions(rq_scene* scene, const float* xyz, void* stream);

/* ---- Allocation-free GI pass ------------------------------------------------------------ */

/* Capacity of the fixed scratch used by rq_gi_frame_noalloc: at most this many primary rays, and
 * at most this many secondary rays (n * spp). */
#define RQ_NOALLOC_MAX_RAYS 65536

/* The GI / RTAO pass of rq_gi_frame for callers that cannot allocate device memory while they
 * render.  No counterpart in the reference (its GI pass is a GLSL dispatch over preallocated
 * images).  cudaMalloc can synchronise the device and can fail under memory pressure, so frame
 * loops that must keep their timing, and host applications that own all device memory through
 * their own allocator and forbid plugins from allocating, cannot call rq_gi_frame, which grows
 * its scratch on demand.  This variant allocates nothing: it runs rq_gi_frame's kernels (fused
 * per-pixel ray generation and shading, the autotuned or requested launch variant, persistent ray
 * queues included) with every intermediate buffer and counter in one fixed __device__ array of
 * about 8.3 MiB.
 *  - The array is reserved on a device when the first context is created on it: rq_create looks
 *    up its device address (cudaGetSymbolAddress, which also loads the module that holds it) and
 *    keeps it in the context.  It stays reserved until the process exits.  After cudaDeviceReset,
 *    create a new context (the old one's address, like its streams and buffers, is gone).
 *  - Device buffers only (RQ_FLAG_HOST_BUFFERS is rejected); no statistics; bounces = 0;
 *    sort_rays and unfused are ignored (they change the kernel arrangement, not the pixels).
 *  - n > RQ_NOALLOC_MAX_RAYS or n * spp > RQ_NOALLOC_MAX_RAYS is rejected with RQ_EINVAL.
 *  - All calls share the array: calls whose work overlaps on the GPU (different streams or host
 *    threads) race and must be serialised by the caller.  Each call overwrites everything it
 *    reads, so nothing from an earlier call leaks into its result.
 * Pixels equal rq_gi_frame's bit for bit for the same inputs and options. */
rq_status rq_gi_frame_noalloc(rq_ctx* ctx, const rq_scene* scene, const rq_ray* primary, int64_t n,
                              const rq_gi_params* params, const rq_opts* opts, float* pixels4,
                              void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RQ_H_ */
