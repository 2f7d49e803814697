// C ABI implementation: contexts, BVH construction, scene upload and validation, query dispatch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/rq.h"
#include "bvh8.h"
#include "bvh_build.h"
#include "rq_internal.h"
#include "tlas.h"
#include "rq_objects.h"
#include "rq_validate.h"

namespace rq {

thread_local std::string g_err;

rq_status fail(rq_ctx* ctx, rq_status s, const std::string& msg) {
    if (ctx) ctx->err = msg;
    g_err = msg;
    return s;
}

rq_status cuda_fail(rq_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, RQ_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

rq_status scratch(rq_ctx* ctx, int slot, size_t bytes, void** out) {
    if (slot < 0 || slot >= kScratchSlots) return fail(ctx, RQ_EINVAL, "bad scratch slot");
    if (bytes == 0) bytes = 256;
    if (ctx->scratch_bytes[slot] < bytes) {
        if (ctx->scratch[slot]) cudaFree(ctx->scratch[slot]);
        ctx->scratch[slot] = nullptr;
        ctx->scratch_bytes[slot] = 0;
        const size_t want = bytes + bytes / 8;  // headroom so small growth does not reallocate
        if (cudaMalloc(&ctx->scratch[slot], want) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "scratch allocation failed");
        ctx->scratch_bytes[slot] = want;
    }
    *out = ctx->scratch[slot];
    return RQ_OK;
}

rq_status resolve_query(rq_ctx* ctx, const rq_scene* sc, const rq_opts* o, QueryConfig& q) {
    rq_opts d{};
    if (!o) o = &d;
    q.layout = o->layout == RQ_LAYOUT_DEFAULT ? sc->layout : o->layout;
    q.mode = o->mode;
    q.tie_lower = o->tie == RQ_TIE_LOWER_INDEX ? 1 : 0;
    q.flags = o->flags;
    q.block = o->block_size;
    q.counters = (o->flags & RQ_FLAG_COUNT) ? work_counters(ctx) : nullptr;
    q.variant_closest = q.variant_any = -1;
    int di = 0;
    rq_status ds = depth_index_of(ctx, o, di);
    if (ds != RQ_OK) return ds;
    if (o->block_size || o->min_blocks || o->persistent || o->stack_depth) {
        // stack_depth 0 (or 48) names the default-depth variant
        const int want_depth = di == 0 ? 0 : bvh8_depth(di);
        int found = -1;
        for (int v = 0; v < kNumLaunchVariants; ++v)
            if (kLaunchVariants[v].block == o->block_size &&
                kLaunchVariants[v].min_blocks == o->min_blocks &&
                kLaunchVariants[v].persistent == (o->persistent ? 1 : 0) &&
                kLaunchVariants[v].depth == want_depth)
                found = v;
        if (found < 0)
            return fail(ctx, RQ_EINVAL, "no compiled launch variant with that block size / min_blocks / stack depth");
        q.variant_closest = q.variant_any = found;
    } else if (q.layout >= 0 && q.layout < 4) {
        q.variant_closest = sc->tuned[q.layout][0];
        q.variant_any = sc->tuned[q.layout][1];
    }
    if (o->flags & RQ_FLAG_NO_PERSISTENT) {
        q.variant_closest = non_persistent_variant(q.variant_closest);
        q.variant_any = non_persistent_variant(q.variant_any);
    }
    if (o->tie != RQ_TIE_LOWER_INDEX && o->tie != RQ_TIE_FIRST_FOUND)
        return fail(ctx, RQ_EINVAL, "unknown tie rule");
    if (q.mode != RQ_MODE_STRICT && q.mode != RQ_MODE_FAST)
        return fail(ctx, RQ_EINVAL, "unknown mode");
    q.status = status_word(ctx);
    if (q.layout == RQ_LAYOUT_BVH8Q) {
        if (!sc->bvh8) return fail(ctx, RQ_ENOTSUP, "BVH8 not built: call rq_scene_build_bvh8");
        if (!q.tie_lower)
            return fail(ctx, RQ_ENOTSUP, "BVH8 queries use the lower-index tie rule");
        return RQ_OK;
    }
    if (q.layout != sc->layout) return fail(ctx, RQ_ENOTSUP, "layout not built for this scene");
    return RQ_OK;
}

rq_status depth_index_of(rq_ctx* ctx, const rq_opts* o, int& index) {
    index = 0;
    if (!o || o->stack_depth == 0) return RQ_OK;
    for (int k = 0; k < 3; ++k)
        if (kBvh8Depths[k] == o->stack_depth) {
            index = k;
            return RQ_OK;
        }
    return fail(ctx, RQ_EINVAL, "stack_depth must be 0, 48, 32 or 24");
}

rq_status refresh_host(rq_scene* sc) {
    rq_ctx* ctx = sc->ctx;
    if (sc->host_stale) {
        RQ_CUDA(ctx, cudaSetDevice(ctx->device));
        RQ_CUDA(ctx, cudaDeviceSynchronize());
        RQ_CUDA(ctx, cudaMemcpy(sc->h_nodes.data(), sc->d_nodes, sc->h_nodes.size() * 4, cudaMemcpyDeviceToHost));
        RQ_CUDA(ctx, cudaMemcpy(sc->h_verts.data(), sc->d_verts, sc->h_verts.size() * 4, cudaMemcpyDeviceToHost));
        sc->host_stale = false;
    }
    if (sc->bvh8 && sc->b8_bounds_stale) {
        // the root nodes of the refitted BVH8, copied back one by one (a handful per scene)
        RQ_CUDA(ctx, cudaSetDevice(ctx->device));
        RQ_CUDA(ctx, cudaDeviceSynchronize());
        std::vector<uint32_t> roots(sc->h_b8roots.size() * kBvh8NodeWords, 0u);
        for (size_t i = 0; i < sc->h_b8roots.size(); ++i)
            if (sc->h_b8roots[i] >= 0)
                RQ_CUDA(ctx, cudaMemcpy(roots.data() + i * kBvh8NodeWords,
                                        reinterpret_cast<const uint32_t*>(sc->d_b8nodes) +
                                            static_cast<int64_t>(sc->h_b8roots[i]) * kBvh8NodeWords,
                                        kBvh8NodeWords * 4, cudaMemcpyDeviceToHost));
        bvh8_root_bounds(sc, roots);
        sc->b8_bounds_stale = false;
    }
    return RQ_OK;
}

// b8_bounds[6 i ..]: the union of entity i's BVH8 root child boxes, one grid step wider (the kernel
// pads its slab test by half a step plus rounding); root_nodes holds each entity's root node.
void bvh8_root_bounds(rq_scene* sc, const std::vector<uint32_t>& root_nodes) {
    sc->b8_bounds.assign(6 * sc->h_ents.size(), 0.0);
    for (size_t i = 0; i < sc->h_ents.size() && i < sc->h_b8roots.size(); ++i) {
        double* bb = &sc->b8_bounds[6 * i];
        bb[0] = bb[1] = bb[2] = 1e300;
        bb[3] = bb[4] = bb[5] = -1e300;
        if (sc->h_b8roots[i] < 0) continue;
        const uint32_t* nd = root_nodes.data() + i * kBvh8NodeWords;
        for (int c = 0; c < 8; ++c) {
            float lo[3], hi[3];
            bvh8_decode_child(nd, c, lo, hi);
            if (!(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2])) continue;  // empty slot
            for (int a = 0; a < 3; ++a) {
                const double step = std::ldexp(1.0, static_cast<int>((nd[3] >> (8 * a)) & 0xFFu) - 127);
                bb[a] = std::min(bb[a], double(lo[a]) - step);
                bb[3 + a] = std::max(bb[3 + a], double(hi[a]) + step);
            }
        }
    }
}

rq_status rebuild_tlas(rq_scene* sc) {
    rq_ctx* ctx = sc->ctx;
    sc->view.tlas = nullptr;
    sc->view.tlas_pre = nullptr;
    sc->tlas_nodes = sc->tlas_cullable = 0;
    if (sc->d_tlas) cudaFree(sc->d_tlas);
    if (sc->d_tlas_pre) cudaFree(sc->d_tlas_pre);
    sc->d_tlas = nullptr;
    sc->d_tlas_pre = nullptr;
    sc->tlas_bytes = 0;
    const int32_t n = sc->n_ents;
    if (n < kTlasMinEntities) return RQ_OK;
    rq_status s = refresh_host(sc);
    if (s != RQ_OK) return s;
    std::vector<TlasEntity> te(n);
    const bool stack = sc->layout == RQ_LAYOUT_BVH2_STACK;
    for (int32_t i = 0; i < n; ++i) {
        const rq_entity& e = sc->h_ents[i];
        TlasEntity& t = te[i];
        std::memcpy(t.inverse, e.inverse, sizeof(t.inverse));
        float alpha;
        std::memcpy(&alpha, &e.data[1], 4);
        t.opaque = !(alpha < 0.99f);  // IntersectSceneIgnoreTransparent skips alpha < 0.99
        t.b8 = sc->bvh8 && static_cast<size_t>(i) < sc->h_b8roots.size() && sc->h_b8roots[i] >= 0;
        t.cullable = false;
        const int64_t off = e.node_offset;
        if (off < 0 || off >= sc->n_nodes || e.node_count < 0) continue;
        const float* nd = sc->h_nodes.data() + off * (stack ? 16 : 8);
        int32_t w0, w1;
        if (stack) {  // both root children must be internal: leaf children are tested box-free
            std::memcpy(&w0, &nd[3], 4);
            std::memcpy(&w1, &nd[11], 4);
            if (w0 != -1 || w1 != -1) continue;
            for (int a = 0; a < 3; ++a) {
                t.lo[a] = std::min(nd[a], nd[8 + a]);
                t.hi[a] = std::max(nd[4 + a], nd[12 + a]);
            }
        } else {  // the root's box is tested first; its skip link must end the walk
            std::memcpy(&w1, &nd[7], 4);
            if (w1 != -1) continue;
            for (int a = 0; a < 3; ++a) {
                t.lo[a] = nd[a];
                t.hi[a] = nd[4 + a];
            }
        }
        if (t.b8 && sc->b8_bounds[6 * i] <= sc->b8_bounds[6 * i + 3])
            for (int a = 0; a < 3; ++a) {
                t.lo[a] = std::min(t.lo[a], sc->b8_bounds[6 * i + a]);
                t.hi[a] = std::max(t.hi[a], sc->b8_bounds[6 * i + 3 + a]);
            }
        t.cullable = true;
    }
    TlasOut out;
    std::string why;
    if (!build_tlas(te, out, why)) return fail(ctx, RQ_EINVAL, "top-level build: " + why);
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t nb = out.nodes.size() * 4, pb = out.prefix.size() * 4;
    if (cudaMalloc(&sc->d_tlas, nb) != cudaSuccess || cudaMalloc(&sc->d_tlas_pre, pb) != cudaSuccess)
        return fail(ctx, RQ_ENOMEM, "top-level allocation failed");
    RQ_CUDA(ctx, cudaMemcpy(sc->d_tlas, out.nodes.data(), nb, cudaMemcpyHostToDevice));
    RQ_CUDA(ctx, cudaMemcpy(sc->d_tlas_pre, out.prefix.data(), pb, cudaMemcpyHostToDevice));
    sc->tlas_bytes = static_cast<int64_t>(nb + pb);
    sc->tlas_nodes = out.n_nodes;
    sc->tlas_cullable = out.n_cullable;
    sc->view.tlas = sc->d_tlas;
    sc->view.tlas_pre = sc->d_tlas_pre;
    sc->view.tlas_margin = out.ray_margin;
    return RQ_OK;
}

}  // namespace rq

namespace {

using rq::fail;
using rq::cuda_fail;
using rq::status_word;
using rq::kLaunchVariants;
using rq::kNumLaunchVariants;

bool is_identity(const float* m) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            const float want = (c == r) ? 1.0f : 0.0f;
            uint32_t a, b;
            std::memcpy(&a, &m[c * 4 + r], 4);
            std::memcpy(&b, &want, 4);
            if (a != b) return false;
        }
    return true;
}

rq_status ensure_stage(rq_ctx* ctx, int k, size_t in_bytes, size_t out_bytes) {
    if (ctx->stage_in_bytes[k] < in_bytes) {
        if (ctx->stage_in[k]) cudaFree(ctx->stage_in[k]);
        ctx->stage_in[k] = nullptr;
        ctx->stage_in_bytes[k] = 0;
        if (cudaMalloc(&ctx->stage_in[k], in_bytes) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "staging buffer allocation failed");
        ctx->stage_in_bytes[k] = in_bytes;
    }
    if (ctx->stage_out_bytes[k] < out_bytes) {
        if (ctx->stage_out[k]) cudaFree(ctx->stage_out[k]);
        ctx->stage_out[k] = nullptr;
        ctx->stage_out_bytes[k] = 0;
        if (cudaMalloc(&ctx->stage_out[k], out_bytes) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "staging buffer allocation failed");
        ctx->stage_out_bytes[k] = out_bytes;
    }
    return RQ_OK;
}

// Host-buffer pipeline: chunks alternate between two streams so that the copy of one chunk
// overlaps the traversal of the previous one (H2D and D2H use separate copy engines).
template <class Launch>
rq_status staged(rq_ctx* ctx, const void* h_in, size_t in_stride, void* h_out, size_t out_stride,
                 int64_t n, cudaStream_t user, Launch launch) {
    const int64_t chunk = int64_t(1) << 20;
    for (int k = 0; k < 2; ++k) {
        rq_status s = ensure_stage(ctx, k, std::min<int64_t>(n, chunk) * in_stride,
                                   std::min<int64_t>(n, chunk) * out_stride);
        if (s != RQ_OK) return s;
    }
    RQ_CUDA(ctx, cudaEventRecord(ctx->ev, user));
    RQ_CUDA(ctx, cudaStreamWaitEvent(ctx->pipe[0], ctx->ev, 0));
    RQ_CUDA(ctx, cudaStreamWaitEvent(ctx->pipe[1], ctx->ev, 0));
    int k = 0;
    for (int64_t off = 0; off < n; off += chunk, k ^= 1) {
        const int64_t m = std::min(chunk, n - off);
        cudaStream_t st = ctx->pipe[k];
        RQ_CUDA(ctx, cudaMemcpyAsync(ctx->stage_in[k], static_cast<const char*>(h_in) + off * in_stride,
                                     m * in_stride, cudaMemcpyHostToDevice, st));
        RQ_CUDA(ctx, launch(ctx->stage_in[k], ctx->stage_out[k], m, st, rq::queue_counter(ctx, 4 + k)));
        RQ_CUDA(ctx, cudaMemcpyAsync(static_cast<char*>(h_out) + off * out_stride, ctx->stage_out[k],
                                     m * out_stride, cudaMemcpyDeviceToHost, st));
    }
    RQ_CUDA(ctx, cudaStreamSynchronize(ctx->pipe[0]));
    RQ_CUDA(ctx, cudaStreamSynchronize(ctx->pipe[1]));
    return RQ_OK;
}

}  // namespace

extern "C" {

int rq_abi_version(void) { return RQ_ABI_VERSION; }

const char* rq_status_string(rq_status s) {
    switch (s) {
        case RQ_OK: return "ok";
        case RQ_EINVAL: return "invalid argument";
        case RQ_ENOMEM: return "out of memory";
        case RQ_ECUDA: return "CUDA error";
        case RQ_EBUDGET: return "iteration budget exhausted";
        case RQ_ENOTSUP: return "not supported";
        case RQ_ESTATE: return "invalid state";
    }
    return "unknown status";
}

const char* rq_last_error(const rq_ctx* ctx) { return ctx ? ctx->err.c_str() : rq::g_err.c_str(); }

rq_status rq_create(int device, rq_ctx** out) {
    if (!out) return fail(nullptr, RQ_EINVAL, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(nullptr, RQ_ECUDA, "no CUDA device available (the engine has no CPU path)");
    if (device < 0 || device >= n) return fail(nullptr, RQ_EINVAL, "device index out of range");
    auto* ctx = new (std::nothrow) rq_ctx;
    if (!ctx) return fail(nullptr, RQ_ENOMEM, "context allocation failed");
    ctx->device = device;
    if ((e = cudaSetDevice(device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->pipe[0], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->pipe[1], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->ev, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->counters, 64 * sizeof(int))) != cudaSuccess ||
        (e = cudaMemset(ctx->counters, 0, 64 * sizeof(int))) != cudaSuccess) {
        rq_status s = cuda_fail(nullptr, e, "context setup");
        rq_destroy(ctx);
        return s;
    }
    rq::noalloc_resolve(ctx);  // reserves rq_gi_frame_noalloc's fixed array on this device
    *out = ctx;
    return RQ_OK;
}

rq_status rq_destroy(rq_ctx* ctx) {
    if (!ctx) return RQ_OK;
    cudaSetDevice(ctx->device);
    for (int k = 0; k < 2; ++k) {
        if (ctx->stage_in[k]) cudaFree(ctx->stage_in[k]);
        if (ctx->stage_out[k]) cudaFree(ctx->stage_out[k]);
        if (ctx->pipe[k]) cudaStreamDestroy(ctx->pipe[k]);
    }
    if (ctx->counters) cudaFree(ctx->counters);
    for (int k = 0; k < kScratchSlots; ++k)
        if (ctx->scratch[k]) cudaFree(ctx->scratch[k]);
    if (ctx->ev) cudaEventDestroy(ctx->ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return RQ_OK;
}

rq_status rq_counters_read(rq_ctx* ctx, rq_counters* out, int reset) {
    if (!ctx || !out) return fail(ctx, RQ_EINVAL, "NULL argument");
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    RQ_CUDA(ctx, cudaDeviceSynchronize());
    unsigned long long c[2];
    RQ_CUDA(ctx, cudaMemcpy(c, rq::work_counters(ctx), sizeof(c), cudaMemcpyDeviceToHost));
    out->node_visits = static_cast<int64_t>(c[0]);
    out->triangle_tests = static_cast<int64_t>(c[1]);
    if (reset) RQ_CUDA(ctx, cudaMemset(rq::work_counters(ctx), 0, sizeof(c)));
    return RQ_OK;
}

// ---- BVH construction ----------------------------------------------------------------------

rq_status rq_build_bvh(const rq_vertex* verts, int64_t n_verts, const uint32_t* indices,
                       int64_t n_indices, const int32_t* mesh_ids, int32_t tri_offset,
                       rq_layout layout, const rq_build_opts* opts, rq_bvh** out) {
    if (!out) return fail(nullptr, RQ_EINVAL, "out is NULL");
    *out = nullptr;
    if (!verts || !indices || n_verts <= 0 || n_indices <= 0 || n_indices % 3 != 0)
        return fail(nullptr, RQ_EINVAL, "vertex/index arrays empty or not a multiple of 3");
    if (layout != RQ_LAYOUT_BVH2_STACK && layout != RQ_LAYOUT_BVH2_STACKLESS)
        return fail(nullptr, RQ_EINVAL, "layout must be BVH2_STACK or BVH2_STACKLESS");
    if (tri_offset < 0) return fail(nullptr, RQ_EINVAL, "tri_offset < 0");
    rq_build_opts d{};
    if (!opts) opts = &d;
    rq::BuildInput in{};
    in.vert_records = reinterpret_cast<const float*>(verts);
    in.n_verts = n_verts;
    in.indices = indices;
    in.n_tris = n_indices / 3;
    in.mesh_ids = mesh_ids;
    in.tri_offset = tri_offset;
    in.leaf_size = opts->leaf_size == 0 ? 2 : opts->leaf_size;
    in.layout = layout == RQ_LAYOUT_BVH2_STACK ? 0 : 1;
    in.swap_children = opts->swap_children;
    in.swap_seed = opts->swap_seed;
    in.n_threads = opts->n_threads;
    auto* b = new (std::nothrow) rq_bvh;
    if (!b) return fail(nullptr, RQ_ENOMEM, "bvh allocation failed");
    b->layout = layout;
    int r;
    try {
        r = rq::build_bvh(in, b->out);
    } catch (const std::bad_alloc&) {
        delete b;
        return fail(nullptr, RQ_ENOMEM, "host allocation failed during BVH build");
    }
    if (r != 0) {
        delete b;
        return fail(nullptr, RQ_EINVAL,
                    "invalid build input (leaf size 1..15, index < n_verts, < 2^27 triangles, "
                    "stack layout needs more triangles than one leaf)");
    }
    *out = b;
    return RQ_OK;
}

rq_status rq_build_bvh_gpu(rq_ctx* ctx, const rq_vertex* verts, int64_t n_verts, const uint32_t* indices,
                           int64_t n_indices, const int32_t* mesh_ids, int32_t tri_offset, rq_layout layout,
                           const rq_build_opts* opts, rq_bvh** out) {
    if (!out) return fail(ctx, RQ_EINVAL, "out is NULL");
    *out = nullptr;
    if (!ctx) return fail(nullptr, RQ_EINVAL, "NULL context");
    if (!verts || !indices || n_verts <= 0 || n_indices <= 0 || n_indices % 3 != 0)
        return fail(ctx, RQ_EINVAL, "vertex/index arrays empty or not a multiple of 3");
    if (layout != RQ_LAYOUT_BVH2_STACK && layout != RQ_LAYOUT_BVH2_STACKLESS)
        return fail(ctx, RQ_EINVAL, "layout must be BVH2_STACK or BVH2_STACKLESS");
    if (tri_offset < 0) return fail(ctx, RQ_EINVAL, "tri_offset < 0");
    rq_build_opts d{};
    if (!opts) opts = &d;
    rq::BuildInput in{};
    in.vert_records = reinterpret_cast<const float*>(verts);
    in.n_verts = n_verts;
    in.indices = indices;
    in.n_tris = n_indices / 3;
    in.mesh_ids = mesh_ids;
    in.tri_offset = tri_offset;
    in.leaf_size = opts->leaf_size == 0 ? 2 : opts->leaf_size;
    in.layout = layout == RQ_LAYOUT_BVH2_STACK ? 0 : 1;
    in.swap_children = opts->swap_children;
    in.swap_seed = opts->swap_seed;
    auto* b = new (std::nothrow) rq_bvh;
    if (!b) return fail(ctx, RQ_ENOMEM, "bvh allocation failed");
    b->layout = layout;
    std::string why;
    rq_status s;
    try {
        s = rq::build_bvh_gpu(ctx, in, b->out, why);
    } catch (const std::bad_alloc&) {
        delete b;
        return fail(ctx, RQ_ENOMEM, "host allocation failed during GPU BVH build");
    }
    if (s != RQ_OK) {
        delete b;
        return fail(ctx, s, why.c_str());
    }
    *out = b;
    return RQ_OK;
}

rq_status rq_bvh_info_get(const rq_bvh* b, rq_bvh_info* info) {
    if (!b || !info) return fail(nullptr, RQ_EINVAL, "NULL argument");
    info->n_nodes = b->out.n_nodes;
    info->n_nodes_used = b->out.n_nodes_used;
    info->n_tris = static_cast<int64_t>(b->out.tris.size() / 4);
    info->node_bytes = b->layout == RQ_LAYOUT_BVH2_STACK ? 64 : 32;
    info->layout = b->layout;
    info->leaf_count = b->out.leaf_count;
    info->split_fails = b->out.split_fails;
    info->build_ms = b->out.build_ms;
    return RQ_OK;
}

rq_status rq_bvh_nodes(const rq_bvh* b, const void** nodes, int64_t* n_nodes) {
    if (!b || !nodes || !n_nodes) return fail(nullptr, RQ_EINVAL, "NULL argument");
    *nodes = b->out.nodes.data();
    *n_nodes = b->out.n_nodes;
    return RQ_OK;
}

rq_status rq_bvh_triangles(const rq_bvh* b, const rq_triangle** tris, int64_t* n_tris) {
    if (!b || !tris || !n_tris) return fail(nullptr, RQ_EINVAL, "NULL argument");
    *tris = reinterpret_cast<const rq_triangle*>(b->out.tris.data());
    *n_tris = static_cast<int64_t>(b->out.tris.size() / 4);
    return RQ_OK;
}

void rq_bvh_free(rq_bvh* b) { delete b; }

// ---- BVH8 (host) ---------------------------------------------------------------------------

struct rq_bvh8 {
    rq::Bvh8Out out;
};

rq_status rq_build_bvh8(rq_layout layout, const void* nodes, int64_t n_nodes, const rq_triangle* tris,
                        int64_t n_tris, const rq_vertex* verts, int64_t n_verts, int32_t node_offset,
                        int32_t node_count, rq_bvh8** out) {
    if (!out || !nodes || !tris || !verts) return fail(nullptr, RQ_EINVAL, "NULL argument");
    *out = nullptr;
    auto* b = new (std::nothrow) rq_bvh8;
    if (!b) return fail(nullptr, RQ_ENOMEM, "allocation failed");
    std::string why;
    std::vector<rq::Bvh8Range> r{{node_offset, node_count}};
    bool ok;
    try {
        ok = rq::build_bvh8(layout, static_cast<const float*>(nodes), n_nodes,
                            reinterpret_cast<const int32_t*>(tris), n_tris,
                            reinterpret_cast<const float*>(verts), n_verts, r, b->out, why);
    } catch (const std::bad_alloc&) {
        delete b;
        return fail(nullptr, RQ_ENOMEM, "host allocation failed");
    }
    if (!ok) {
        delete b;
        return fail(nullptr, RQ_EINVAL, "BVH8 build: " + why);
    }
    *out = b;
    return RQ_OK;
}

rq_status rq_bvh8_buffers(const rq_bvh8* b, const uint32_t** nodes, int64_t* n_nodes,
                          const float** tri_records, int64_t* n_records) {
    if (!b || !nodes || !n_nodes || !tri_records || !n_records)
        return fail(nullptr, RQ_EINVAL, "NULL argument");
    *nodes = b->out.nodes.data();
    *n_nodes = b->out.n_nodes;
    *tri_records = b->out.tris.data();
    *n_records = b->out.n_tris;
    return RQ_OK;
}

void rq_bvh8_free(rq_bvh8* b) { delete b; }

// ---- Scene -----------------------------------------------------------------------------------

rq_status rq_scene_validate(rq_layout layout, const rq_vertex* verts, int64_t n_verts,
                            const rq_triangle* tris, int64_t n_tris, const void* nodes,
                            int64_t n_nodes, const rq_entity* ents, int32_t n_ents, char* msg,
                            size_t msg_len) {
    std::string why;
    const bool ok = rq::validate_scene(layout, verts, n_verts, tris, n_tris, nodes, n_nodes, ents,
                                       n_ents, why);
    if (msg && msg_len) {
        std::snprintf(msg, msg_len, "%s", why.c_str());
    }
    if (!ok) return fail(nullptr, RQ_EINVAL, why);
    return RQ_OK;
}

rq_status rq_scene_create(rq_ctx* ctx, rq_layout layout, const rq_vertex* verts, int64_t n_verts,
                          const rq_triangle* tris, int64_t n_tris, const void* nodes,
                          int64_t n_nodes, const rq_entity* ents, int32_t n_ents,
                          rq_scene** out) {
    if (!ctx || !out) return fail(ctx, RQ_EINVAL, "NULL context or out");
    *out = nullptr;
    std::string why;
    if (!rq::validate_scene(layout, verts, n_verts, tris, n_tris, nodes, n_nodes, ents, n_ents, why))
        return fail(ctx, RQ_EINVAL, why);
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    auto* sc = new (std::nothrow) rq_scene;
    if (!sc) return fail(ctx, RQ_ENOMEM, "scene allocation failed");
    sc->ctx = ctx;
    sc->layout = layout;
    sc->n_nodes = n_nodes;
    sc->n_tris = n_tris;
    sc->n_verts = n_verts;
    const size_t node_bytes = layout == RQ_LAYOUT_BVH2_STACK ? 64 : 32;
    sc->h_nodes.assign(static_cast<const float*>(nodes),
                       static_cast<const float*>(nodes) + n_nodes * (node_bytes / 4));
    sc->h_tris.assign(reinterpret_cast<const int32_t*>(tris),
                      reinterpret_cast<const int32_t*>(tris) + 4 * n_tris);
    sc->h_verts.assign(reinterpret_cast<const float*>(verts),
                       reinterpret_cast<const float*>(verts) + 8 * n_verts);
    const size_t nb = node_bytes * n_nodes, tb = 16 * n_tris, vb = 32 * n_verts;
    cudaError_t e;
    if ((e = cudaMalloc(&sc->d_nodes, nb)) != cudaSuccess || (e = cudaMalloc(&sc->d_tris, tb)) != cudaSuccess ||
        (e = cudaMalloc(&sc->d_verts, vb)) != cudaSuccess) {
        rq_scene_destroy(sc);
        return fail(ctx, RQ_ENOMEM, std::string("scene device allocation: ") + cudaGetErrorString(e));
    }
    sc->bytes = static_cast<int64_t>(nb + tb + vb);
    if ((e = cudaMalloc(&sc->d_tri_fast, 48 * n_tris)) != cudaSuccess) {
        rq_scene_destroy(sc);
        return fail(ctx, RQ_ENOMEM, "fast triangle records allocation failed");
    }
    sc->bytes += 48 * n_tris;
    if ((e = cudaMemcpy(sc->d_nodes, nodes, nb, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(sc->d_tris, tris, tb, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(sc->d_verts, verts, vb, cudaMemcpyHostToDevice)) != cudaSuccess) {
        rq_scene_destroy(sc);
        return cuda_fail(ctx, e, "scene upload");
    }
    sc->view.nodes = sc->d_nodes;
    sc->view.n_nodes = n_nodes;
    sc->view.tris = sc->d_tris;
    sc->view.n_tris = n_tris;
    sc->view.verts = sc->d_verts;
    sc->view.n_verts = n_verts;
    sc->view.layout = layout;
    sc->view.tri_fast = sc->d_tri_fast;
    if ((e = rq::launch_tri_fast(sc->d_tris, n_tris, sc->d_verts, sc->d_tri_fast, nullptr)) != cudaSuccess ||
        (e = cudaDeviceSynchronize()) != cudaSuccess) {
        rq_scene_destroy(sc);
        return cuda_fail(ctx, e, "fast triangle records");
    }
    rq_status s = rq_scene_set_entities(sc, ents, n_ents);
    if (s != RQ_OK) {
        rq_scene_destroy(sc);
        return s;
    }
    *out = sc;
    return RQ_OK;
}

rq_status rq_scene_set_entities(rq_scene* sc, const rq_entity* ents, int32_t n_ents) {
    if (!sc) return fail(nullptr, RQ_EINVAL, "NULL scene");
    rq_ctx* ctx = sc->ctx;
    std::string why;
    if (!rq::validate_entities(sc->layout, sc->h_nodes.data(), sc->n_nodes, sc->n_tris, ents,
                               n_ents, why))
        return fail(ctx, RQ_EINVAL, why);
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    if (n_ents > sc->ents_cap) {
        if (sc->d_ents) cudaFree(sc->d_ents);
        sc->d_ents = nullptr;
        sc->ents_cap = 0;
        if (cudaMalloc(&sc->d_ents, sizeof(rq_entity) * n_ents) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "entity buffer allocation failed");
        sc->ents_cap = n_ents;
    }
    RQ_CUDA(ctx, cudaMemcpy(sc->d_ents, ents, sizeof(rq_entity) * n_ents, cudaMemcpyHostToDevice));
    sc->n_ents = n_ents;
    sc->view.ents = sc->d_ents;
    sc->view.n_ents = n_ents;
    bool ident = true;
    for (int i = 0; i < n_ents; ++i) ident = ident && is_identity(ents[i].inverse);
    sc->view.all_identity = ident ? 1 : 0;
    sc->h_ents.assign(ents, ents + n_ents);
    if (sc->bvh8) return rq_scene_build_bvh8(sc, nullptr);  // rebuilds the top level too
    return rq::rebuild_tlas(sc);
}

rq_status rq_scene_build_bvh8(rq_scene* sc, rq_bvh8_info* info) {
    if (!sc) return fail(nullptr, RQ_EINVAL, "NULL scene");
    rq_ctx* ctx = sc->ctx;
    rq_status st0 = rq::refresh_host(sc);  // positions may have been updated on the device
    if (st0 != RQ_OK) return st0;
    std::vector<rq::Bvh8Range> ranges;
    for (const rq_entity& e : sc->h_ents) ranges.push_back({e.node_offset, e.node_count});
    rq::Bvh8Out b;
    std::string why;
    bool ok;
    try {
        ok = rq::build_bvh8(sc->layout, sc->h_nodes.data(), sc->n_nodes, sc->h_tris.data(), sc->n_tris,
                            sc->h_verts.data(), sc->n_verts, ranges, b, why);
    } catch (const std::bad_alloc&) {
        return fail(ctx, RQ_ENOMEM, "host allocation failed during BVH8 build");
    }
    if (!ok) return fail(ctx, RQ_ENOTSUP, "BVH8 build: " + why);
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    if (sc->d_b8nodes) cudaFree(sc->d_b8nodes);
    if (sc->d_b8tris) cudaFree(sc->d_b8tris);
    sc->d_b8nodes = nullptr;
    sc->d_b8tris = nullptr;
    sc->bvh8 = false;
    const size_t nb = b.nodes.size() * 4, tb = std::max<size_t>(16, b.tris.size() * 4);
    if (cudaMalloc(&sc->d_b8nodes, nb) != cudaSuccess || cudaMalloc(&sc->d_b8tris, tb) != cudaSuccess)
        return fail(ctx, RQ_ENOMEM, "BVH8 device allocation failed");
    RQ_CUDA(ctx, cudaMemcpy(sc->d_b8nodes, b.nodes.data(), nb, cudaMemcpyHostToDevice));
    if (!b.tris.empty())
        RQ_CUDA(ctx, cudaMemcpy(sc->d_b8tris, b.tris.data(), b.tris.size() * 4, cudaMemcpyHostToDevice));
    const int32_t ne = static_cast<int32_t>(b.roots.size());
    if (ne > sc->b8roots_cap) {
        if (sc->d_b8roots) cudaFree(sc->d_b8roots);
        sc->d_b8roots = nullptr;
        sc->b8roots_cap = 0;
        if (cudaMalloc(&sc->d_b8roots, sizeof(int32_t) * ne) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "BVH8 root table allocation failed");
        sc->b8roots_cap = ne;
    }
    if (ne) RQ_CUDA(ctx, cudaMemcpy(sc->d_b8roots, b.roots.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice));
    sc->b8_nodes = b.n_nodes;
    sc->b8_tris = b.n_tris;
    sc->b8_bytes = static_cast<int64_t>(nb + tb + sizeof(int32_t) * sc->b8roots_cap);
    sc->b8_build_ms = b.build_ms;
    sc->view.b8_nodes = sc->d_b8nodes;
    sc->view.b8_tris = sc->d_b8tris;
    sc->view.b8_roots = sc->d_b8roots;
    sc->bvh8 = true;
    sc->h_b8roots = b.roots;
    {
        std::vector<uint32_t> roots(b.roots.size() * rq::kBvh8NodeWords, 0u);
        for (size_t i = 0; i < b.roots.size(); ++i)
            if (b.roots[i] >= 0)
                std::memcpy(roots.data() + i * rq::kBvh8NodeWords,
                            b.nodes.data() + static_cast<size_t>(b.roots[i]) * rq::kBvh8NodeWords,
                            rq::kBvh8NodeWords * 4);
        rq::bvh8_root_bounds(sc, roots);
    }
    sc->b8_bounds_stale = false;
    // refit plan: nodes level by level from each distinct root down (children of node x are
    // child_base + 0 .. popc(imask) - 1)
    {
        std::vector<int32_t> level(static_cast<size_t>(b.n_nodes), -1);
        std::vector<int32_t> cur, next;
        for (int32_t r : b.roots)
            if (r >= 0 && level[r] < 0) {
                level[r] = 0;
                cur.push_back(r);
            }
        std::vector<int32_t> order;
        sc->b8_level_off.assign(1, 0);
        while (!cur.empty()) {
            order.insert(order.end(), cur.begin(), cur.end());
            sc->b8_level_off.push_back(static_cast<int64_t>(order.size()));
            next.clear();
            for (int32_t x : cur) {
                const uint32_t* nd = b.nodes.data() + static_cast<size_t>(x) * rq::kBvh8NodeWords;
                const int ni = __builtin_popcount(nd[3] >> 24);
                for (int i = 0; i < ni; ++i) {
                    const int32_t c = static_cast<int32_t>(nd[4]) + i;
                    if (c >= 0 && c < b.n_nodes && level[c] < 0) {
                        level[c] = level[x] + 1;
                        next.push_back(c);
                    }
                }
            }
            cur.swap(next);
        }
        if (sc->d_b8_order) cudaFree(sc->d_b8_order);
        if (sc->d_b8box) cudaFree(sc->d_b8box);
        sc->d_b8_order = nullptr;
        sc->d_b8box = nullptr;
        if (cudaMalloc(&sc->d_b8_order, sizeof(int32_t) * std::max<size_t>(1, order.size())) != cudaSuccess ||
            cudaMalloc(&sc->d_b8box, sizeof(float) * 6 * std::max<int64_t>(1, b.n_nodes)) != cudaSuccess)
            return fail(ctx, RQ_ENOMEM, "BVH8 refit plan allocation failed");
        if (!order.empty())
            RQ_CUDA(ctx, cudaMemcpy(sc->d_b8_order, order.data(), sizeof(int32_t) * order.size(),
                                    cudaMemcpyHostToDevice));
        sc->b8_bytes += static_cast<int64_t>(sizeof(int32_t) * order.size() + sizeof(float) * 6 * b.n_nodes);
    }
    if ((st0 = rq::rebuild_tlas(sc)) != RQ_OK) return st0;
    if (info) {
        info->nodes = b.n_nodes;
        info->triangles = b.n_tris;
        info->bytes = sc->b8_bytes;
        info->bvh2_nodes = b.bvh2_nodes;
        info->build_ms = b.build_ms;
    }
    return RQ_OK;
}

rq_status rq_autotune(rq_ctx* ctx, rq_scene* sc, const rq_ray* rays, int64_t n, int32_t query,
                      rq_layout layout, rq_tune_result* out) {
    if (!ctx || !sc || !out || !rays || n <= 0 || (query != 0 && query != 1))
        return fail(ctx, RQ_EINVAL, "bad autotune arguments");
    rq_opts o{};
    o.layout = layout;
    rq::QueryConfig q{};
    rq_status s = rq::resolve_query(ctx, sc, &o, q);
    if (s != RQ_OK) return s;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    void* out_buf = nullptr;
    if ((s = rq::scratch(ctx, rq::kSlotTuneOut, query == 0 ? sizeof(rq_hit) * n : n, &out_buf)) != RQ_OK) return s;
    cudaEvent_t a, b;
    RQ_CUDA(ctx, cudaEventCreate(&a));
    RQ_CUDA(ctx, cudaEventCreate(&b));
    std::memset(out, 0, sizeof(*out));
    out->n_variants = kNumLaunchVariants;
    float best = 1e30f;
    int best_v = 0;
    cudaStream_t st = ctx->stream;
    // status bits of earlier work are kept aside; a trial that overflows its group stack is rejected
    unsigned prior = 0;
    RQ_CUDA(ctx, cudaDeviceSynchronize());
    RQ_CUDA(ctx, cudaMemcpy(&prior, rq::status_word(ctx), sizeof(unsigned), cudaMemcpyDeviceToHost));
    for (int v = 0; v < kNumLaunchVariants; ++v) {
        out->block[v] = kLaunchVariants[v].block;
        out->min_blocks_of[v] = kLaunchVariants[v].min_blocks;
        out->persistent_of[v] = kLaunchVariants[v].persistent;
        out->depth_of[v] = kLaunchVariants[v].depth ? kLaunchVariants[v].depth : rq::bvh8_depth(0);
        out->ms[v] = -1.0f;
        if (kLaunchVariants[v].persistent && q.mode == RQ_MODE_FAST) continue;
        // the group-stack depth is a BVH8 knob: the BVH2 walks keep the reference's stack
        if (kLaunchVariants[v].depth && q.layout != RQ_LAYOUT_BVH8Q) continue;
        q.variant_closest = q.variant_any = v;
        RQ_CUDA(ctx, cudaMemsetAsync(rq::status_word(ctx), 0, sizeof(unsigned), st));
        float vbest = 1e30f;
        for (int rep = 0; rep < 4; ++rep) {
            RQ_CUDA(ctx, cudaEventRecord(a, st));
            cudaError_t e = query == 0
                ? rq::launch_closest(sc->view, q, rays, n, static_cast<rq_hit*>(out_buf), rq::queue_counter(ctx, 8), st)
                : rq::launch_anyhit(sc->view, q, rays, n, static_cast<uint8_t*>(out_buf), rq::queue_counter(ctx, 8), st);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "autotune launch");
            RQ_CUDA(ctx, cudaEventRecord(b, st));
            RQ_CUDA(ctx, cudaEventSynchronize(b));
            float ms = 0.0f;
            RQ_CUDA(ctx, cudaEventElapsedTime(&ms, a, b));
            if (rep > 0) vbest = std::min(vbest, ms);  // rep 0 is the warm-up
        }
        unsigned bits = 0;
        RQ_CUDA(ctx, cudaMemcpy(&bits, rq::status_word(ctx), sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (bits & rq::kStatusOverflowBit) {
            out->ms[v] = -2.0f;  // the stack overflowed on these rays: not usable
            continue;
        }
        out->ms[v] = vbest;
        if (vbest < best) {
            best = vbest;
            best_v = v;
        }
    }
    RQ_CUDA(ctx, cudaMemcpy(rq::status_word(ctx), &prior, sizeof(unsigned), cudaMemcpyHostToDevice));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    sc->tuned[q.layout][query] = static_cast<int8_t>(best_v);
    out->variant = best_v;
    out->block_size = kLaunchVariants[best_v].block;
    out->min_blocks = kLaunchVariants[best_v].min_blocks;
    out->persistent = kLaunchVariants[best_v].persistent;
    out->depth = out->depth_of[best_v];
    return RQ_OK;
}

rq_status rq_device_status(rq_ctx* ctx, uint32_t* bits, int reset) {
    if (!ctx || !bits) return fail(ctx, RQ_EINVAL, "NULL argument");
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    RQ_CUDA(ctx, cudaDeviceSynchronize());
    RQ_CUDA(ctx, cudaMemcpy(bits, rq::status_word(ctx), sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (reset) RQ_CUDA(ctx, cudaMemset(rq::status_word(ctx), 0, sizeof(uint32_t)));
    return RQ_OK;
}

rq_status rq_scene_bytes(const rq_scene* sc, int64_t* bytes) {
    if (!sc || !bytes) return fail(nullptr, RQ_EINVAL, "NULL argument");
    *bytes = sc->bytes + static_cast<int64_t>(sizeof(rq_entity)) * sc->ents_cap + sc->b8_bytes + sc->tlas_bytes +
             sc->tex_bytes;
    return RQ_OK;
}

rq_status rq_scene_tlas_info(const rq_scene* sc, rq_tlas_info* info) {
    if (!sc || !info) return fail(nullptr, RQ_EINVAL, "NULL argument");
    info->nodes = sc->view.tlas ? sc->tlas_nodes : 0;
    info->entities = sc->n_ents;
    info->cullable = sc->view.tlas ? sc->tlas_cullable : 0;
    info->reserved = 0;
    info->bytes = sc->view.tlas ? sc->tlas_bytes : 0;
    return RQ_OK;
}

rq_status rq_scene_destroy(rq_scene* sc) {
    if (!sc) return RQ_OK;
    if (sc->ctx) cudaSetDevice(sc->ctx->device);
    if (sc->d_nodes) cudaFree(sc->d_nodes);
    if (sc->d_tris) cudaFree(sc->d_tris);
    if (sc->d_verts) cudaFree(sc->d_verts);
    if (sc->d_ents) cudaFree(sc->d_ents);
    if (sc->d_albedo) cudaFree(sc->d_albedo);
    if (sc->d_mesh_tex) cudaFree(sc->d_mesh_tex);
    if (sc->d_tex) cudaFree(sc->d_tex);
    if (sc->d_texels) cudaFree(sc->d_texels);
    if (sc->d_srgb) cudaFree(sc->d_srgb);
    if (sc->d_b8nodes) cudaFree(sc->d_b8nodes);
    if (sc->d_b8tris) cudaFree(sc->d_b8tris);
    if (sc->d_b8roots) cudaFree(sc->d_b8roots);
    if (sc->d_b8_order) cudaFree(sc->d_b8_order);
    if (sc->d_b8box) cudaFree(sc->d_b8box);
    if (sc->d_refit) cudaFree(sc->d_refit);
    if (sc->d_tri_fast) cudaFree(sc->d_tri_fast);
    if (sc->d_adj_off) cudaFree(sc->d_adj_off);
    if (sc->d_adj) cudaFree(sc->d_adj);
    if (sc->d_tlas) cudaFree(sc->d_tlas);
    if (sc->d_tlas_pre) cudaFree(sc->d_tlas_pre);
    delete sc;
    return RQ_OK;
}

// ---- Queries --------------------------------------------------------------------------------

rq_status rq_closest(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays, int64_t n, rq_hit* hits,
                     const rq_opts* opts, void* stream) {
    if (!ctx || !sc) return fail(ctx, RQ_EINVAL, "NULL context or scene");
    if (n < 0 || (n > 0 && (!rays || !hits))) return fail(ctx, RQ_EINVAL, "bad ray/hit arrays");
    if (sc->ctx != ctx) return fail(ctx, RQ_EINVAL, "scene belongs to another context");
    rq::QueryConfig q{};
    rq_status s = rq::resolve_query(ctx, sc, opts, q);
    if (s != RQ_OK) return s;
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = the default stream
    const rq::SceneView view = sc->view;
    if (q.flags & RQ_FLAG_HOST_BUFFERS) {
        return staged(ctx, rays, sizeof(rq_ray), hits, sizeof(rq_hit), n, st,
                      [&](void* din, void* dout, int64_t m, cudaStream_t cs, unsigned long long* qc) {
                          return rq::launch_closest(view, q, static_cast<const rq_ray*>(din), m,
                                                    static_cast<rq_hit*>(dout), qc, cs);
                      });
    }
    RQ_CUDA(ctx, rq::launch_closest(view, q, rays, n, hits, rq::queue_counter(ctx, 0), st));
    return RQ_OK;
}

rq_status rq_anyhit(rq_ctx* ctx, const rq_scene* sc, const rq_ray* rays, int64_t n,
                    uint8_t* occluded, const rq_opts* opts, void* stream) {
    if (!ctx || !sc) return fail(ctx, RQ_EINVAL, "NULL context or scene");
    if (n < 0 || (n > 0 && (!rays || !occluded))) return fail(ctx, RQ_EINVAL, "bad ray/result arrays");
    if (sc->ctx != ctx) return fail(ctx, RQ_EINVAL, "scene belongs to another context");
    rq::QueryConfig q{};
    rq_status s = rq::resolve_query(ctx, sc, opts, q);
    if (s != RQ_OK) return s;
    if (n == 0) return RQ_OK;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);  // NULL = the default stream
    const rq::SceneView view = sc->view;
    if (q.flags & RQ_FLAG_HOST_BUFFERS) {
        return staged(ctx, rays, sizeof(rq_ray), occluded, 1, n, st,
                      [&](void* din, void* dout, int64_t m, cudaStream_t cs, unsigned long long* qc) {
                          return rq::launch_anyhit(view, q, static_cast<const rq_ray*>(din), m,
                                                   static_cast<uint8_t*>(dout), qc, cs);
                      });
    }
    RQ_CUDA(ctx, rq::launch_anyhit(view, q, rays, n, occluded, rq::queue_counter(ctx, 0), st));
    return RQ_OK;
}

}  // extern "C"
