// BVH8 walks over a batch of rays, shared by the query kernels and the fused GI kernels:
// one ray per thread (bvh8_ray) or a persistent ray queue (bvh8_persistent_loop; its plain form,
// bvh8_plain_queue_loop, also runs the batched queries through a per-lane ray source), with the
// reference's entity loop (IntersectScene, TraverseBVHStack.glsl:327-366) around the walk.
#pragma once
#include <cuda_runtime.h>

#include "rq_bvh8.cuh"
#include "rq_internal.h"
#include "rq_persistent.cuh"
#include "rq_strict.cuh"

namespace rq {

__device__ __forceinline__ void load_ray(const rq_ray* rays, int64_t i, float4& r0, float4& r1) {
    const float4* p = reinterpret_cast<const float4*>(rays) + 2 * i;
    r0 = __ldg(p);
    r1 = __ldg(p + 1);
}

__device__ __forceinline__ void store_hit(rq_hit* hits, int64_t i, const rq_hit& h) {
    float4* p = reinterpret_cast<float4*>(hits) + 2 * i;
    __stcs(p, make_float4(h.t, h.u, h.v, h.w));
    __stcs(p + 1, make_float4(__int_as_float(h.tri), __int_as_float(h.mesh), __int_as_float(h.entity),
                              __int_as_float(h.iters)));
}

// Closest-hit record of a BVH8 query: barycentrics from the hit point with the strict arithmetic
// (TraverseBVHStack.glsl:351-363), the reference's tri-0 quirk under RQ_FLAG_REF_COMPAT.
__device__ __forceinline__ void bvh8_finish(const SceneView& s, int flags, const strict::f3 o,
                                            const strict::f3 d, float closest, int32_t tri,
                                            int32_t mesh, int32_t ent, int32_t visits, rq_hit& hh) {
    hh.t = hh.u = hh.v = hh.w = -1.0f;
    hh.tri = hh.mesh = hh.entity = -1;
    hh.iters = visits;
    if (closest > 0.0f) {
        hh.tri = tri;
        hh.mesh = mesh;
        hh.entity = ent;
        const bool report = (flags & RQ_FLAG_REF_COMPAT) ? tri > 0 : tri >= 0;
        if (report) {
            const rq_entity& E = s.ents[ent];
            const strict::f3 ro = strict::xform(E.inverse, o, 1.0f);
            const strict::f3 rd = strict::xform(E.inverse, d, 0.0f);
            const int4 tr = strict::ldg4i(s.tris + tri);
            const strict::f3 p = strict::add(ro, strict::muls(rd, closest));
            float u, v, w;
            strict::barycentrics(p, strict::vpos(s, tr.x), strict::vpos(s, tr.y), strict::vpos(s, tr.z),
                                 u, v, w);
            hh.t = closest;
            hh.u = u;
            hh.v = v;
            hh.w = w;
        }
    }
}

// BVH8 traversal of one ray with the strict scene loop around it.
template <bool kAny, bool kTlas = true, int kDepth = bvh8::kStack>
__device__ __forceinline__ void bvh8_ray(const SceneView& s, const float4 r0, const float4 r1, int flags,
                                         rq_hit& hh, bool& occluded, int32_t& visits,
                                         int32_t& tests, unsigned& status) {
    const float rtmin = r0.w, rtmax = r1.w;
    const strict::f3 o = strict::xyz(r0), d = strict::xyz(r1);
    float tmax = rtmax, closest = -1.0f;
    int32_t mesh = -1, tri = -1, ent = -1;
    occluded = false;
    if (rtmax > rtmin) {
        const bool skip_transparent = !kAny && (flags & RQ_FLAG_IGNORE_TRANSPARENT);
        const float3 wo = make_float3(o.x, o.y, o.z), wd = make_float3(d.x, d.y, d.z);
        int32_t cur = tlas::begin<kTlas>(s, wo, wd);
        if (!kAny && kTlas && cur != tlas::kPlain) {
            // closest hit through the top level: candidates nearest first (tlas::near_next)
            const int count = skip_transparent ? tlas::kBvh8Opaque : tlas::kBvh8;
            uint64_t nst[tlas::kNearStack];
            tlas::Near nw;
            tlas::near_begin(s, nw, nst, wo, wd, tmax, status);
            int32_t walked = 0;
            for (int e; (e = tlas::near_next(s, nw, nst, wo, wd, tmax, 0x7FFFFFFF, status)) >= 0;) {
                const rq_entity& E = s.ents[e];
                if (skip_transparent && strict::ent_alpha(E) < 0.99f) continue;
                const int32_t root = s.b8_roots[e];
                if (root < 0) continue;
                ++walked;
                const bvh8::Ray8 r = bvh8::make_ray(strict::xform(E.inverse, o, 1.0f),
                                                    strict::xform(E.inverse, d, 0.0f));
                // an equal (t, triangle) from a lower entity wins: let the walk take it
                bvh8::Hit8 h{tmax, -1.0f, (ent >= 0 && e < ent) ? tri + 1 : tri, -1};
                visits += bvh8::traverse<false, true, kDepth>(s.b8_nodes, s.b8_tris, root, r, rtmin, h, tests, status);
                const float T = h.closest;
                if (T > 0.0f && (T < tmax || (T == tmax && (h.tri < tri || (h.tri == tri && e < ent))))) {
                    tmax = T;
                    closest = T;
                    mesh = h.mesh;
                    tri = h.tri;
                    ent = e;
                }
            }
            visits += tlas::walked(s, 0, s.n_ents, count) - walked;  // one per entity not walked
            bvh8_finish(s, flags, o, d, closest, tri, mesh, ent, visits, hh);
            return;
        }
        for (int e = -1; (e = tlas::next<kTlas>(s, cur, e, wo, wd, kAny ? rtmax : tmax,
                                    skip_transparent ? tlas::kBvh8Opaque : tlas::kBvh8, visits)) >= 0;) {
            const rq_entity& E = s.ents[e];
            if (skip_transparent && strict::ent_alpha(E) < 0.99f) continue;
            const int32_t root = s.b8_roots[e];
            if (root < 0) continue;
            const bvh8::Ray8 r = bvh8::make_ray(strict::xform(E.inverse, o, 1.0f),
                                                strict::xform(E.inverse, d, 0.0f));
            bvh8::Hit8 h{kAny ? rtmax : tmax, -1.0f, kAny ? -1 : tri, -1};
            visits += bvh8::traverse<kAny, true, kDepth>(s.b8_nodes, s.b8_tris, root, r, rtmin, h, tests,
                                                 status);
            const float T = h.closest;
            if (kAny) {
                if (T > 0.0f) {
                    occluded = true;
                    break;
                }
            } else if (T > 0.0f && (T < tmax || (T == tmax && h.tri < tri))) {
                tmax = T;
                closest = T;
                mesh = h.mesh;
                tri = h.tri;
                ent = e;
            }
        }
    }
    if (kAny) return;
    bvh8_finish(s, flags, o, d, closest, tri, mesh, ent, visits, hh);
}

// Persistent BVH8 traversal loop (run by every thread of a resident grid until the ray queue is
// empty); `sink.put<kAny>(id, ...)` receives each ray's result.  Each iteration
// visits one node per lane.  At the top of every iteration the whole warp (converged by the
// full-mask vote) hands new rays to its idle lanes from a warp-private pool of consecutive ray
// indices, refilled kPoolRays at a time from the global counter by one atomicAdd, so lanes stay
// busy while the warp's longest rays finish and a warp keeps working on neighbouring rays.
// Inactive rays are answered in the refill loop itself.  Per ray the walk, the entity loop and
// the acceptance tests are those of k_bvh8 (same step function), so results are identical; only
// the assignment of rays to lanes changes.  The world ray is re-read from `rays` when a later
// entity or the final record needs it, which keeps it out of the loop's registers.
constexpr int kPoolRays = 64;
// Idle lanes a warp gathers before it stores their results and refills them while other lanes
// are still walking.  Measured on the C2 secondary closest-hit launch (8.3M slots, 128 x 8
// persistent): 1 (serve at once) 0.831 ms, 4: 0.823, 8: 0.791, 12: 0.777, 16: 0.780, 20: 0.789,
// 24: 0.829, 32 (only when no lane walks) 1.26; at 128 x 7 (GI pass) 8: 1.001, 12: 0.989, 16:
// 0.993, 20: 1.009 ms.  The top-level branch refills every iteration: serving there measured
// slower.
constexpr int kServeBatch = 12;
// Guided hand-out: once fewer than kTailPools x kPoolRays x (warps of the grid) rays remain past a
// warp's last pool, the warp takes only the rays its idle lanes need, so that the warps run out of
// work together.  C2 secondary launch: 0 (always pools) 0.769 ms, 1: 0.768, 2: 0.767, 4: 0.764,
// 8: 0.767, 16: 0.763, always exact: 0.790.
constexpr int kTailPools = 4;

template <class Sink>
struct OneQuery;
template <bool kAny, int kDepth, class Src>
__device__ __forceinline__ void bvh8_plain_queue_loop(Src& src, int64_t n, unsigned long long* queue,
                                                      int32_t& tests, int32_t& nodes_total, unsigned& status);

template <bool kAny, class Sink, bool kTlas = true, int kDepth = bvh8::kStack>
__device__ __forceinline__ void bvh8_persistent_loop(const SceneView& s, const rq_ray* __restrict__ rays,
                                                     int64_t n, int flags, unsigned long long* queue,
                                                     const Sink& sink, int32_t& tests,
                                                     int32_t& nodes_total, unsigned& status) {
    const unsigned kFull = 0xFFFFFFFFu;
    const unsigned lane = threadIdx.x & 31u;
    uint64_t stack[kDepth];
    bvh8::Ray8 r;
    bvh8::Hit8 h;
    bvh8::Walk w;
    float tmin = 0.0f, tmax = 0.0f, closest = -1.0f;
    int32_t mesh = -1, tri = -1, ent_hit = -1, ent = -1, visits = 0;
    int32_t ents = tlas::kPlain;  // entity cursor (rq_tlas.cuh); `ent` is the last entity it gave
    int64_t id = -1;
    bool live = false, exhausted = false;
    unsigned long long pool_next = 0, pool_end = 0;  // warp-uniform
    // Starts the walk of entity `ent` or a later one that is traversed; false when none is left.
    auto begin = [&](const float4 r0, const float4 r1) -> bool {
        const bool skip_transparent = !kAny && (flags & RQ_FLAG_IGNORE_TRANSPARENT);
        const float3 wo = make_float3(r0.x, r0.y, r0.z), wd = make_float3(r1.x, r1.y, r1.z);
        while ((ent = tlas::next<kTlas>(s, ents, ent, wo, wd, kAny ? r1.w : tmax,
                                 skip_transparent ? tlas::kBvh8Opaque : tlas::kBvh8, visits)) >= 0) {
            const rq_entity& E = s.ents[ent];
            if (skip_transparent && strict::ent_alpha(E) < 0.99f) continue;
            const int32_t root = s.b8_roots[ent];
            if (root < 0) continue;
            r = bvh8::make_ray(strict::xform(E.inverse, strict::xyz(r0), 1.0f),
                               strict::xform(E.inverse, strict::xyz(r1), 0.0f));
            h = bvh8::Hit8{kAny ? r1.w : tmax, -1.0f, kAny ? -1 : tri, -1};
            w = bvh8::walk_begin(root);
            return true;
        }
        return false;
    };
    auto store = [&](const float4 r0, const float4 r1, bool occluded) {
        nodes_total += visits;
        sink.template put<kAny>(id, r0, r1, closest, tri, mesh, ent_hit, visits, occluded);
    };
    if constexpr (kTlas) {
        // Scenes with a top level: a lane looking for its ray's next entity (`seek`) advances the
        // top-level cursor by at most kSeekNodes nodes per iteration, interleaved with the node
        // steps of the lanes that are walking an entity, so that a long top-level walk does not
        // hold the warp.  The entities, their order and every count are those of the loop below.
        constexpr int kSeekNodes = 4;
        bool seek = false;
        // closest hit through the top level: candidates nearest first (tlas::near_next, which
        // expands two children per node, so half the node budget); any hit keeps the ascending
        // cursor (its early exit takes the first occluder in either order)
        bool nearest = false;
        uint64_t nst[kAny ? 1 : tlas::kNearStack];
        tlas::Near nw{0};
        int32_t walked = 0;
        const bool skip_transparent = !kAny && (flags & RQ_FLAG_IGNORE_TRANSPARENT);
        const int count = skip_transparent ? tlas::kBvh8Opaque : tlas::kBvh8;
        // One bounded seek: 1 = the walk of entity `ent` is set up, 0 = keep seeking, -1 = none left.
        auto seek_step = [&](const float4 r0, const float4 r1) -> int {
            const float3 wo = make_float3(r0.x, r0.y, r0.z), wd = make_float3(r1.x, r1.y, r1.z);
            int32_t e;
            if (!kAny && nearest)
                e = tlas::near_next(s, nw, nst, wo, wd, tmax, kSeekNodes / 2, status);
            else
                e = tlas::next_n<true>(s, ents, ent, wo, wd, kAny ? r1.w : tmax, count, visits, kSeekNodes);
            if (e == tlas::kMore) return 0;
            if (e < 0) {
                if (!kAny && nearest) visits += tlas::walked(s, 0, s.n_ents, count) - walked;
                return -1;
            }
            ent = e;
            const rq_entity& E = s.ents[ent];
            if (skip_transparent && strict::ent_alpha(E) < 0.99f) return 0;
            const int32_t root = s.b8_roots[ent];
            if (root < 0) return 0;
            ++walked;
            r = bvh8::make_ray(strict::xform(E.inverse, strict::xyz(r0), 1.0f),
                               strict::xform(E.inverse, strict::xyz(r1), 0.0f));
            // an equal (t, triangle) from a lower entity wins: let the walk take it
            h = bvh8::Hit8{kAny ? r1.w : tmax, -1.0f, kAny ? -1 : ((ent_hit >= 0 && ent < ent_hit) ? tri + 1 : tri), -1};
            w = bvh8::walk_begin(root);
            return 1;
        };
        while (true) {
            // refill idle lanes (warp-uniform loop; inactive rays are answered here)
            while (true) {
                const unsigned want = __ballot_sync(kFull, !live && !exhausted);
                if (!want) break;
                const unsigned cnt = __popc(want);
                const unsigned rank = __popc(want & persist::lanemask_lt());
                const unsigned long long avail = pool_end - pool_next;
                unsigned long long mine = pool_next + rank;
                if (avail >= cnt) {
                    pool_next += cnt;
                } else {
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(queue, static_cast<unsigned long long>(kPoolRays));
                    base = __shfl_sync(kFull, base, 0);
                    if (rank >= avail) mine = base + (rank - avail);
                    pool_next = base + (cnt - avail);
                    pool_end = base + kPoolRays;
                }
                if (!live && !exhausted) {
                    if (static_cast<int64_t>(mine) >= n) {
                        exhausted = true;
                    } else {
                        id = static_cast<int64_t>(mine);
                        float4 r0, r1;
                        load_ray(rays, id, r0, r1);
                        tmin = r0.w;
                        tmax = r1.w;
                        closest = -1.0f;
                        mesh = tri = ent_hit = -1;
                        visits = 0;
                        ent = -1;
                        ents = tlas::begin<true>(s, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z));
                        live = r1.w > r0.w;
                        seek = live;
                        walked = 0;
                        nearest = !kAny && ents != tlas::kPlain;
                        if (live && nearest)
                            tlas::near_begin(s, nw, nst, make_float3(r0.x, r0.y, r0.z), make_float3(r1.x, r1.y, r1.z),
                                             tmax, status);
                        if (!live) store(r0, r1, false);
                    }
                }
            }
            if (!__any_sync(kFull, live)) break;
            if (!live) continue;
            if (seek) {
                float4 r0, r1;
                load_ray(rays, id, r0, r1);
                const int g = seek_step(r0, r1);
                if (g > 0) {
                    seek = false;
                } else if (g < 0) {
                    store(r0, r1, false);
                    live = false;
                }
                continue;
            }
            if (bvh8::step<kAny, true, kDepth>(s.b8_nodes, s.b8_tris, r, tmin, h, w, stack, tests, status)) continue;
            // the walk of entity `ent` has ended
            visits += w.visits;
            const float T = h.closest;
            if (kAny) {
                if (T > 0.0f) {
                    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    store(z, z, true);
                    live = false;
                    continue;
                }
            } else if (T > 0.0f && (T < tmax || (T == tmax && (h.tri < tri || (h.tri == tri && ent < ent_hit))))) {
                tmax = T;
                closest = T;
                mesh = h.mesh;
                tri = h.tri;
                ent_hit = ent;
            }
            seek = true;
        }
    } else {
        OneQuery<Sink> src{s, rays, flags, sink, -1};
        bvh8_plain_queue_loop<kAny, kDepth>(src, n, queue, tests, nodes_total, status);
    }
}


// The plain lane-refill loop (scenes without a top level) over a ray source: the rays of one
// query (OneQuery) or the rays of a batch's queries of one kind (BatchQueries).  Each warp hands
// its idle lanes rays from a warp-private pool of consecutive indices refilled kPoolRays at a time
// from `queue` (by need near the end of the queue); each lane walks its ray's entities one node
// per iteration.  A lane whose ray is finished keeps its result (`pending`) until the warp serves
// its idle lanes: the result stores and the refills then run together, with at least kServeBatch
// lanes (or whenever no lane is walking), instead of for one or two lanes in every iteration.  Per
// ray the entity loop, the walk, the acceptance tests and the record are those of bvh8_ray, so
// results are identical whatever the assignment of rays to lanes.
template <bool kAny, int kDepth, class Src>
__device__ __forceinline__ void bvh8_plain_queue_loop(Src& src, int64_t n, unsigned long long* queue,
                                                      int32_t& tests, int32_t& nodes_total, unsigned& status) {
    if (n <= 0) return;
    const unsigned kFull = 0xFFFFFFFFu;
    const unsigned lane = threadIdx.x & 31u;
    uint64_t stack[kDepth];
    bvh8::Ray8 r;
    bvh8::Hit8 h;
    bvh8::Walk w;
    float tmin = 0.0f, tmax = 0.0f, closest = -1.0f;
    int32_t mesh = -1, tri = -1, ent_hit = -1, ent = -1, visits = 0;
    int32_t ents = tlas::kPlain;
    bool live = false, exhausted = false, pending = false, pending_occ = false;
    unsigned long long pool_next = 0, pool_end = 0;  // warp-uniform
    const unsigned long long tail_rays = static_cast<unsigned long long>(kTailPools) * kPoolRays *
                                         (static_cast<unsigned long long>(gridDim.x) * blockDim.x / 32u);
    // Starts the walk of entity `ent` or a later one of the lane's scene; false when none is left.
    auto begin = [&](const float4 r0, const float4 r1) -> bool {
        const SceneView& s = src.scene();
        const bool skip_transparent = !kAny && (src.flags() & RQ_FLAG_IGNORE_TRANSPARENT);
        const float3 wo = make_float3(r0.x, r0.y, r0.z), wd = make_float3(r1.x, r1.y, r1.z);
        while ((ent = tlas::next<false>(s, ents, ent, wo, wd, kAny ? r1.w : tmax,
                                        skip_transparent ? tlas::kBvh8Opaque : tlas::kBvh8, visits)) >= 0) {
            const rq_entity& E = s.ents[ent];
            if (skip_transparent && strict::ent_alpha(E) < 0.99f) continue;
            const int32_t root = s.b8_roots[ent];
            if (root < 0) continue;
            r = bvh8::make_ray(strict::xform(E.inverse, strict::xyz(r0), 1.0f),
                               strict::xform(E.inverse, strict::xyz(r1), 0.0f));
            h = bvh8::Hit8{kAny ? r1.w : tmax, -1.0f, kAny ? -1 : tri, -1};
            w = bvh8::walk_begin(root);
            return true;
        }
        return false;
    };
    auto store = [&](const float4 r0, const float4 r1, bool occluded) {
        nodes_total += visits;
        src.template put<kAny>(r0, r1, closest, tri, mesh, ent_hit, visits, occluded);
    };
    while (true) {
        const unsigned idle = __ballot_sync(kFull, !live && !exhausted);
        const unsigned walking = __ballot_sync(kFull, live);
        const bool serve = !(idle && walking && __popc(idle) < kServeBatch);
        if (serve) {
            if (pending) {
                float4 r0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), r1 = r0;
                if (!kAny) src.load(r0, r1);
                store(r0, r1, pending_occ);
                pending = false;
            }
            // refill idle lanes (warp-uniform loop; inactive rays are answered here)
            while (true) {
                const unsigned want = __ballot_sync(kFull, !live && !exhausted);
                if (!want) break;
                const unsigned cnt = __popc(want);
                const unsigned rank = __popc(want & persist::lanemask_lt());
                const unsigned long long avail = pool_end - pool_next;
                unsigned long long mine = pool_next + rank;
                if (avail >= cnt) {
                    pool_next += cnt;
                } else {
                    // near the end of the queue a warp takes only the rays its idle lanes need
                    const unsigned long long need = cnt - avail;
                    const unsigned long long grab =
                        pool_end + tail_rays >= static_cast<unsigned long long>(n) ? need : kPoolRays;
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(queue, grab);
                    base = __shfl_sync(kFull, base, 0);
                    if (rank >= avail) mine = base + (rank - avail);
                    pool_next = base + need;
                    pool_end = base + grab;
                }
                if (!live && !exhausted) {
                    if (static_cast<int64_t>(mine) >= n) {
                        exhausted = true;
                    } else {
                        src.take(static_cast<int64_t>(mine));
                        float4 r0, r1;
                        src.load(r0, r1);
                        tmin = r0.w;
                        tmax = r1.w;
                        closest = -1.0f;
                        mesh = tri = ent_hit = -1;
                        visits = 0;
                        ent = -1;
                        ents = tlas::kPlain;
                        live = (r1.w > r0.w) && begin(r0, r1);
                        if (!live) store(r0, r1, false);
                    }
                }
            }
            if (!__any_sync(kFull, live)) break;  // every lane exhausted, every result stored
        }
        if (!live) continue;
        if (bvh8::step<kAny, true, kDepth>(src.nodes(), src.recs(), r, tmin, h, w, stack, tests, status)) continue;
        // the walk of entity `ent` has ended
        visits += w.visits;
        const float T = h.closest;
        bool done = false;
        if (kAny) {
            done = T > 0.0f;
        } else if (T > 0.0f && (T < tmax || (T == tmax && h.tri < tri))) {
            tmax = T;
            closest = T;
            mesh = h.mesh;
            tri = h.tri;
            ent_hit = ent;
        }
        if (!done) {
            float4 r0, r1;
            src.load(r0, r1);
            if (begin(r0, r1)) continue;
        }
        pending = true;  // stored when the warp next serves its idle lanes
        pending_occ = done;
        live = false;
    }
}

// Ray source of one query: ray `id` of `rays`, results through `sink` (QuerySink).
template <class Sink>
struct OneQuery {
    const SceneView& s;
    const rq_ray* __restrict__ rays;
    int flags_;
    const Sink& sink;
    int64_t id;
    __device__ __forceinline__ void take(int64_t item) { id = item; }
    __device__ __forceinline__ void load(float4& r0, float4& r1) const { load_ray(rays, id, r0, r1); }
    __device__ __forceinline__ const SceneView& scene() const { return s; }
    __device__ __forceinline__ int flags() const { return flags_; }
    __device__ __forceinline__ const uint4* nodes() const { return s.b8_nodes; }
    __device__ __forceinline__ const float4* recs() const { return s.b8_tris; }
    template <bool kAny>
    __device__ __forceinline__ void put(const float4 r0, const float4 r1, float closest, int32_t tri, int32_t mesh,
                                        int32_t ent, int32_t visits, bool occluded) const {
        sink.template put<kAny>(id, r0, r1, closest, tri, mesh, ent, visits, occluded);
    }
};

// Ray source of a batch's queries of one kind (scenes without a top level): work items
// [lo, lo + n) of the batch, query q holding items base[q] .. base[q + 1] - 1.  A lane that takes
// an item finds its query by binary search and keeps the query's BVH8 pointers in registers.
struct BatchQueries {
    const QueryDesc* __restrict__ qd;
    const int64_t* base;
    int nq;
    int64_t lo;
    const QueryDesc* q;  // the lane's query
    int64_t id;          // ray index within it
    const uint4* nodes_;
    const float4* recs_;
    __device__ __forceinline__ void take(int64_t item) {
        item += lo;
        int a = 0, z = nq - 1;
        while (a < z) {
            const int mid = (a + z + 1) >> 1;
            if (base[mid] <= item) a = mid; else z = mid - 1;
        }
        q = qd + a;
        id = item - base[a];
        nodes_ = q->s.b8_nodes;
        recs_ = q->s.b8_tris;
    }
    __device__ __forceinline__ void load(float4& r0, float4& r1) const { load_ray(q->rays, id, r0, r1); }
    __device__ __forceinline__ const SceneView& scene() const { return q->s; }
    __device__ __forceinline__ int flags() const { return q->flags; }
    __device__ __forceinline__ const uint4* nodes() const { return nodes_; }
    __device__ __forceinline__ const float4* recs() const { return recs_; }
    template <bool kAny>
    __device__ __forceinline__ void put(const float4 r0, const float4 r1, float closest, int32_t tri, int32_t mesh,
                                        int32_t ent, int32_t visits, bool occluded) const {
        if (kAny) {
            q->occ[id] = occluded ? 1 : 0;
        } else {
            rq_hit hh;
            bvh8_finish(q->s, q->flags, strict::xyz(r0), strict::xyz(r1), closest, tri, mesh, ent, visits, hh);
            store_hit(q->hits, id, hh);
        }
    }
};

// The batched BVH8 queries of one kind over scenes without a top level: work items [lo, hi) of
// the batch from `queue`, through bvh8_plain_queue_loop (results equal k_batch's).
template <bool kAny, int kDepth>
__device__ __forceinline__ void bvh8_batch_loop(const QueryDesc* __restrict__ qd, const int64_t* base, int nq,
                                                int64_t lo, int64_t hi, unsigned long long* queue,
                                                unsigned& status) {
    BatchQueries src{qd, base, nq, lo, qd, -1, nullptr, nullptr};
    int32_t tests = 0, nodes_total = 0;
    bvh8_plain_queue_loop<kAny, kDepth>(src, hi - lo, queue, tests, nodes_total, status);
}

// Sink of the query kernels: hit records (closest) or occlusion bytes (any hit).
struct QuerySink {
    const SceneView& s;
    int flags;
    rq_hit* hits;
    uint8_t* occ;
    template <bool kAny>
    __device__ __forceinline__ void put(int64_t id, const float4 r0, const float4 r1, float closest,
                                        int32_t tri, int32_t mesh, int32_t ent, int32_t visits,
                                        bool occluded) const {
        if (kAny) {
            occ[id] = occluded ? 1 : 0;
        } else {
            rq_hit hh;
            bvh8_finish(s, flags, strict::xyz(r0), strict::xyz(r1), closest, tri, mesh, ent, visits, hh);
            store_hit(hits, id, hh);
        }
    }
};

}  // namespace rq
