// Batched queries: descriptor tables, the one-launch path, and plans replayed as CUDA graphs.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <vector>

#include "rq_objects.h"

struct rq_batch_plan {
    rq_ctx* ctx = nullptr;
    std::vector<rq::QueryDesc> desc;  // host copy, rebuilt per family
    std::vector<rq_query> queries;
    rq_opts opts{};
    int32_t family = rq::kFamilyStrict;
    int32_t variant = 0;
    int32_t depth_index = 0;  // BVH8 group-stack depth (bvh8::kStackDepths)
    int64_t total = 0;
    int64_t total_c = -1;  // rays of the closest-hit queries when the lane-refill kernel applies, else -1
    rq::QueryDesc* d_desc = nullptr;
    unsigned long long* d_queue = nullptr;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace rq {
namespace {

// Validates queries and fills device descriptors for `family`: the closest-hit queries first, then
// the any-hit queries (each in the caller's order; every query writes its own outputs).  total_c:
// the closest-hit queries' rays when the BVH8 lane-refill kernel applies (BVH8 family, no scene
// with a top level), else -1.
rq_status describe(rq_ctx* ctx, const rq_query* q, int32_t nq, const rq_opts* o, int family,
                   std::vector<QueryDesc>& out, int64_t& total, int64_t& total_c) {
    if (nq < 1 || nq > kMaxBatchQueries) return fail(ctx, RQ_EINVAL, "1..1024 queries per batch");
    out.assign(nq, QueryDesc{});
    total = 0;
    total_c = 0;
    bool plain = true;
    std::vector<int32_t> order;
    order.reserve(nq);
    for (int kind = 0; kind < 2; ++kind)
        for (int32_t k = 0; k < nq; ++k)
            if (q[k].kind == kind || (kind == 1 && q[k].kind != 0)) order.push_back(k);
    for (int32_t j = 0; j < nq; ++j) {
        const int32_t k = order[j];
        const rq_query& x = q[k];
        if (!x.scene || x.scene->ctx != ctx || x.n < 0 || (x.kind != 0 && x.kind != 1) ||
            (x.n > 0 && (!x.rays || (x.kind == 0 ? !x.hits : !x.occluded))))
            return fail(ctx, RQ_EINVAL, "query " + std::to_string(k) + ": bad scene, rays or outputs");
        if (family == kFamilyBvh8 && !x.scene->bvh8)
            return fail(ctx, RQ_ENOTSUP, "query " + std::to_string(k) + ": scene has no BVH8");
        QueryDesc& d = out[j];
        d.s = entity_view(x.scene->view, o ? o->flags : 0);
        d.rays = x.rays;
        d.hits = x.hits;
        d.occ = x.occluded;
        d.n = x.n;
        d.base = total;
        d.kind = x.kind;
        d.flags = o ? (o->flags & (RQ_FLAG_REF_COMPAT | RQ_FLAG_IGNORE_TRANSPARENT)) : 0;
        d.tie_lower = (!o || o->tie == RQ_TIE_LOWER_INDEX) ? 1 : 0;
        total += x.n;
        if (x.kind == 0) total_c += x.n;
        plain = plain && d.s.tlas == nullptr;
    }
    if (family != kFamilyBvh8 || !plain) total_c = -1;
    return RQ_OK;
}

int family_of(const rq_opts* o) {
    if (o && o->layout == RQ_LAYOUT_BVH8Q) return kFamilyBvh8;
    if (o && o->mode == RQ_MODE_FAST) return kFamilyFast;
    return kFamilyStrict;
}

rq_status capture(rq_batch_plan* p) {
    rq_ctx* ctx = p->ctx;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
    // occupancy queries happen here, before the capture starts
    RQ_CUDA(ctx, launch_batch(p->d_desc, 1, 1, p->family, p->variant, nullptr, nullptr, nullptr, p->depth_index));
    RQ_CUDA(ctx, cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(p->d_queue, 0, 2 * sizeof(unsigned long long), p->cap);
    if (e == cudaSuccess)
        e = launch_batch(p->d_desc, static_cast<int>(p->desc.size()), p->total, p->family, p->variant,
                         p->d_queue, status_word(ctx), p->cap, p->depth_index, p->total_c);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(p->cap, &g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch capture");
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "batch capture end");
    p->graph = g;
    RQ_CUDA(ctx, cudaGraphInstantiate(&p->exec, g, 0));
    return RQ_OK;
}

rq_status upload(rq_batch_plan* p) {
    rq_ctx* ctx = p->ctx;
    rq_status s = describe(ctx, p->queries.data(), static_cast<int32_t>(p->queries.size()), &p->opts,
                           p->family, p->desc, p->total, p->total_c);
    if (s != RQ_OK) return s;
    RQ_CUDA(ctx, cudaMemcpy(p->d_desc, p->desc.data(), sizeof(QueryDesc) * p->desc.size(),
                            cudaMemcpyHostToDevice));
    return RQ_OK;
}

}  // namespace
}  // namespace rq

using rq::fail;

extern "C" {

rq_status rq_batch(rq_ctx* ctx, const rq_query* queries, int32_t n_queries, const rq_opts* opts,
                   void* stream) {
    if (!ctx || !queries) return fail(ctx, RQ_EINVAL, "NULL argument");
    const int family = rq::family_of(opts);
    std::vector<rq::QueryDesc> desc;
    int64_t total = 0, total_c = -1;
    rq_status s = rq::describe(ctx, queries, n_queries, opts, family, desc, total, total_c);
    if (s != RQ_OK) return s;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    void* d = nullptr;
    if ((s = rq::scratch(ctx, rq::kSlotBatchDesc, sizeof(rq::QueryDesc) * desc.size(), &d)) != RQ_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // Pageable source: the copy completes before the call returns, so `desc` may go out of scope.
    RQ_CUDA(ctx, cudaMemcpyAsync(d, desc.data(), sizeof(rq::QueryDesc) * desc.size(),
                                 cudaMemcpyHostToDevice, st));
    unsigned long long* queue = rq::queue_counter(ctx, 10);  // and counter 11 (the any-hit queue)
    RQ_CUDA(ctx, cudaMemsetAsync(queue, 0, 2 * sizeof(unsigned long long), st));
    int variant = 0;
    if (opts && (opts->block_size || opts->min_blocks)) {
        variant = -1;
        for (int v = 0; v < rq::kNumBatchVariants; ++v)
            if (rq::kBatchVariants[v].block == opts->block_size &&
                rq::kBatchVariants[v].min_blocks == opts->min_blocks)
                variant = v;
        if (variant < 0) return fail(ctx, RQ_EINVAL, "no compiled batch variant with that block size");
    }
    int di = 0;
    if ((s = rq::depth_index_of(ctx, opts, di)) != RQ_OK) return s;
    RQ_CUDA(ctx, rq::launch_batch(static_cast<rq::QueryDesc*>(d), n_queries, total, family, variant,
                                  queue, rq::status_word(ctx), st, di, total_c));
    return RQ_OK;
}

rq_status rq_batch_plan_create(rq_ctx* ctx, const rq_query* queries, int32_t n_queries,
                               const rq_opts* opts, rq_batch_plan** out) {
    if (!ctx || !queries || !out) return fail(ctx, RQ_EINVAL, "NULL argument");
    *out = nullptr;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    auto* p = new (std::nothrow) rq_batch_plan;
    if (!p) return fail(ctx, RQ_ENOMEM, "plan allocation failed");
    p->ctx = ctx;
    p->queries.assign(queries, queries + std::max(0, n_queries));
    if (opts) p->opts = *opts;
    p->family = rq::family_of(opts);
    rq_status s;
    if (n_queries < 1 || n_queries > rq::kMaxBatchQueries) {
        delete p;
        return fail(ctx, RQ_EINVAL, "1..1024 queries per batch");
    }
    if ((s = rq::depth_index_of(ctx, opts, p->depth_index)) != RQ_OK) {
        delete p;
        return s;
    }
    if (cudaMalloc(&p->d_desc, sizeof(rq::QueryDesc) * n_queries) != cudaSuccess ||
        cudaMalloc(&p->d_queue, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking) != cudaSuccess) {
        rq_batch_plan_destroy(p);
        return fail(ctx, RQ_ENOMEM, "plan device allocation failed");
    }
    if ((s = rq::upload(p)) != RQ_OK || (s = rq::capture(p)) != RQ_OK) {
        rq_batch_plan_destroy(p);
        return s;
    }
    *out = p;
    return RQ_OK;
}

rq_status rq_batch_plan_launch(rq_batch_plan* p, void* stream) {
    if (!p) return fail(nullptr, RQ_EINVAL, "NULL plan");
    RQ_CUDA(p->ctx, cudaSetDevice(p->ctx->device));
    RQ_CUDA(p->ctx, cudaGraphLaunch(p->exec, static_cast<cudaStream_t>(stream)));
    return RQ_OK;
}

rq_status rq_batch_plan_autotune(rq_batch_plan* p, int32_t allow_bvh8, rq_batch_tune* out) {
    if (!p || !out) return fail(nullptr, RQ_EINVAL, "NULL argument");
    rq_ctx* ctx = p->ctx;
    RQ_CUDA(ctx, cudaSetDevice(ctx->device));
    std::memset(out, 0, sizeof(*out));
    bool all_b8 = allow_bvh8 != 0;
    for (const rq_query& q : p->queries) all_b8 = all_b8 && q.scene->bvh8;
    const int fams[2] = {rq::kFamilyBvh8, p->opts.mode == RQ_MODE_FAST ? rq::kFamilyFast : rq::kFamilyStrict};
    cudaEvent_t a, b;
    RQ_CUDA(ctx, cudaEventCreate(&a));
    RQ_CUDA(ctx, cudaEventCreate(&b));
    // the status bits of earlier work are kept aside: a stack overflow during a trial marks that
    // depth as unusable for this batch
    unsigned prior = 0;
    RQ_CUDA(ctx, cudaDeviceSynchronize());
    RQ_CUDA(ctx, cudaMemcpy(&prior, rq::status_word(ctx), sizeof(unsigned), cudaMemcpyDeviceToHost));
    float best = 1e30f;
    int best_f = p->family, best_v = p->variant, best_d = p->depth_index;
    int k = 0;
    for (int fi = 0; fi < 2; ++fi) {
        const int n_depths = fams[fi] == rq::kFamilyBvh8 ? rq::kNumBatchDepths : 1;
        for (int di = 0; di < n_depths; ++di) {
            for (int v = 0; v < rq::kNumBatchVariants; ++v, ++k) {
                out->family_of[k] = fams[fi];
                out->block_of[k] = rq::kBatchVariants[v].block;
                out->min_blocks_of[k] = rq::kBatchVariants[v].min_blocks;
                out->depth_of[k] = fams[fi] == rq::kFamilyBvh8 ? rq::bvh8_depth(di) : 0;
                out->ms[k] = -1.0f;
                if (fams[fi] == rq::kFamilyBvh8 && !all_b8) continue;
                p->family = fams[fi];
                rq_status s = rq::upload(p);
                if (s != RQ_OK) return s;
                RQ_CUDA(ctx, cudaMemset(rq::status_word(ctx), 0, sizeof(unsigned)));
                float vbest = 1e30f;
                for (int rep = 0; rep < 4; ++rep) {
                    RQ_CUDA(ctx, cudaMemsetAsync(p->d_queue, 0, 2 * sizeof(unsigned long long), p->cap));
                    RQ_CUDA(ctx, cudaEventRecord(a, p->cap));
                    RQ_CUDA(ctx, rq::launch_batch(p->d_desc, static_cast<int>(p->desc.size()), p->total,
                                                  p->family, v, p->d_queue, rq::status_word(ctx), p->cap, di,
                                                  p->total_c));
                    RQ_CUDA(ctx, cudaEventRecord(b, p->cap));
                    RQ_CUDA(ctx, cudaEventSynchronize(b));
                    float ms = 0.0f;
                    RQ_CUDA(ctx, cudaEventElapsedTime(&ms, a, b));
                    if (rep > 0) vbest = std::min(vbest, ms);
                }
                unsigned bits = 0;
                RQ_CUDA(ctx, cudaMemcpy(&bits, rq::status_word(ctx), sizeof(unsigned), cudaMemcpyDeviceToHost));
                if (bits & rq::kStatusOverflowBit) {
                    out->ms[k] = -2.0f;  // overflowed: results would be incomplete
                    continue;
                }
                out->ms[k] = vbest;
                if (vbest < best) {
                    best = vbest;
                    best_f = fams[fi];
                    best_v = v;
                    best_d = di;
                }
            }
        }
    }
    RQ_CUDA(ctx, cudaMemcpy(rq::status_word(ctx), &prior, sizeof(unsigned), cudaMemcpyHostToDevice));
    out->n = k;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    p->family = best_f;
    p->variant = best_v;
    p->depth_index = best_f == rq::kFamilyBvh8 ? best_d : 0;
    rq_status s = rq::upload(p);
    if (s != RQ_OK) return s;
    if ((s = rq::capture(p)) != RQ_OK) return s;
    out->family = best_f;
    out->block_size = rq::kBatchVariants[best_v].block;
    out->min_blocks = rq::kBatchVariants[best_v].min_blocks;
    out->depth = best_f == rq::kFamilyBvh8 ? rq::bvh8_depth(p->depth_index) : 0;
    return RQ_OK;
}

rq_status rq_batch_plan_destroy(rq_batch_plan* p) {
    if (!p) return RQ_OK;
    if (p->ctx) cudaSetDevice(p->ctx->device);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->cap) cudaStreamDestroy(p->cap);
    if (p->d_desc) cudaFree(p->d_desc);
    if (p->d_queue) cudaFree(p->d_queue);
    delete p;
    return RQ_OK;
}

}  // extern "C"
