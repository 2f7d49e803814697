/* rq.h — C ABI of the GB300 ray-query engine (librq.so).
 *
 * A drop-in for the ray-query path of the Candela renderer (swr06/Candela): the SAH BVH
 * constructor, its flattened node / triangle / vertex buffers and the closest-hit / any-hit ray
 * API.  Every entry point names the reference interface it replaces.  Plain C types only: no
 * CUDA, C++ or torch types cross this boundary; `stream` arguments are cudaStream_t passed as
 * void* (NULL = the context's own stream).
 *
 * Conventions
 *  - Every call returns rq_status.  On failure rq_last_error(ctx) holds a message.
 *  - Buffers are device pointers unless RQ_FLAG_HOST_BUFFERS is set in rq_opts.flags, in which
 *    case the library stages them through device memory itself (copies inside the call).
 *  - Calls are ordered on the given stream; results are ready when the stream is synchronised.
 *    With RQ_FLAG_HOST_BUFFERS the call synchronises before returning.
 *  - One rq_ctx per host thread.  One GPU per context.  There is no CPU fallback: a context can
 *    only be created on a CUDA device.
 */
#ifndef RQ_H_
#define RQ_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RQ_ABI_VERSION 1

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
 * -1.  iters = BVH nodes visited, summed over entities. */
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
                                        reported with t = u = v = w = -1 */
    RQ_FLAG_IGNORE_TRANSPARENT = 2,  /* IntersectSceneIgnoreTransparent: skip entities with
                                        alpha < 0.99 (TraverseBVHStack.glsl:368-413) */
    RQ_FLAG_HOST_BUFFERS = 4,        /* ray/hit pointers are host memory */
    RQ_FLAG_NO_PERSISTENT = 8        /* one thread per ray instead of the persistent kernel */
};

typedef struct rq_opts {
    int32_t layout;      /* rq_layout */
    int32_t mode;        /* rq_mode */
    int32_t tie;         /* rq_tie */
    int32_t flags;       /* RQ_FLAG_* */
    int32_t block_size;  /* 0 = tuned default */
    int32_t reserved[3];
} rq_opts;

/* ---- Context ---------------------------------------------------------------------------- */

typedef struct rq_ctx rq_ctx;

int rq_abi_version(void);
const char* rq_status_string(rq_status s);

/* Creates a context on CUDA device `device`.  Fails with RQ_ECUDA when no device is present. */
rq_status rq_create(int device, rq_ctx** out);
rq_status rq_destroy(rq_ctx* ctx);
const char* rq_last_error(const rq_ctx* ctx);

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
rq_status rq_bvh_info_get(const rq_bvh* bvh, rq_bvh_info* info);
/* Borrowed pointers, valid until rq_bvh_free. */
rq_status rq_bvh_nodes(const rq_bvh* bvh, const void** nodes, int64_t* n_nodes);
rq_status rq_bvh_triangles(const rq_bvh* bvh, const rq_triangle** tris, int64_t* n_tris);
void rq_bvh_free(rq_bvh* bvh);

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
/* Device bytes held by the scene (all layouts built so far). */
rq_status rq_scene_bytes(const rq_scene* scene, int64_t* bytes);
rq_status rq_scene_destroy(rq_scene* scene);

/* ---- Queries ---------------------------------------------------------------------------- */

/* Closest hit for n rays.  Replaces IntersectRay(o, d, out TUVW, out Mesh, out TriangleIdx, ...)
 * / IntersectScene (TraverseBVHStack.glsl:327-366, 458-502; stackless
 * TraverseBVHStackless.glsl:280-319).  opts may be NULL (strict, lower-index ties). */
rq_status rq_closest(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays, int64_t n,
                     rq_hit* hits, const rq_opts* opts, void* stream);

/* Any hit (occlusion) for n rays: occluded[i] = 1 when a triangle with tmin < t < tmax lies on the
 * ray.  Replaces float IntersectRay(o, d) / IntersectSceneOcclusion (TraverseBVHStack.glsl:
 * 509-682; stackless :463-579), with the per-ray tmax the per-BVH functions accept. */
rq_status rq_anyhit(rq_ctx* ctx, const rq_scene* scene, const rq_ray* rays, int64_t n,
                    uint8_t* occluded, const rq_opts* opts, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RQ_H_ */
