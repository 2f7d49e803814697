// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's ray-query path, used as the parity checker for the CUDA
// kernels and as the timed CPU baseline.  The reference implements this path only as GLSL compute
// shaders; there is no CPU intersector in it (BVH/Intersector.h:353-357 is a stub), so this file
// restates the GLSL arithmetic statement by statement in C++.  Every function cites the lines it
// follows.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
//
// Parity status.  Pinned against the reference's own sources compiled here (oracle/Makefile):
//  * traversal (both layouts, closest and any hit, scene loop, entity transforms,
//    ignore-transparent, the tri-0 test, iteration counts) against the traversal functions of
//    TraverseBVHStack.glsl / TraverseBVHStackless.glsl compiled as C++ (ref_glsl_harness.cpp):
//    bit for bit, with the dot / mat*vec summation order defined here (GLSL leaves it open);
//  * GetData (TraverseBVHStack.glsl: interpolated normal, UV, ModelColor, emissive, alpha) the
//    same way: bit for bit;
//  * CosWeightedHemisphere (Sampling.glsl) and StochasticReflectionDirection / SampleGGXVNDF
//    (SpecularTrace.glsl, Sampling.glsl) the same way, with the same samples: a mirror bit for bit,
//    sampled directions within a few ulps (the C library's cos / sin there, turn-based polynomials
//    here; GGX's sqrt(1 - cos^2) cancellation spreads that to 1e-4 in rare samples);
//  * the collision walks (both layouts, the reference's axis set and leaf index) against
//    CollideBVHStack.glsl / CollideBVHStackless.glsl compiled the same way, and the stackless one
//    also against Physics::CollideBox, compiled from Physics.cpp (ref_physics_harness.cpp);
//  * the shading sums: the diffuse pass's hit shading (DiffuseTrace.glsl:486-494 with GetDirect)
//    and the specular pass's (SpecularTrace.glsl:554-563, 588-596 with SampleLighting, Sky,
//    IsValid, the clamp and the t / 48 store), compiled the same way with the renderer state they
//    read (shadow-map lookup, probe volume, sky textures) given as values: bit for bit;
//  * the RT second-bounce loop (DiffuseTrace.glsl:499-535) the same way, fed the restatement's
//    per-bounce hits: bounce ray origins and FinalRadiance + Bounced bit for bit;
//  * the BVH constructor (ref_bvh_harness.cpp), byte for byte.
// Parity unpinned for the texture filter only: the reference samples through bindless GL
// samplers, which cannot run here, so bilinear filtering, wrap modes and the sRGB decode are
// checked by analytic known-answer tests (tests/test_oracle.py).
//
// Arithmetic conventions (the definition that the strict GPU kernels must reproduce bit for bit):
//  * IEEE binary32, round to nearest, no contraction (built with -ffp-contract=off);
//  * GLSL min/max as specified: min(x,y) = y < x ? y : x, max(x,y) = x < y ? y : x;
//  * dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z;  cross(a,b) = (a.y*b.z - a.z*b.y, ...);
//  * mat4*vec4 (column-major) = ((M[0]*v.x + M[1]*v.y) + M[2]*v.z) + M[3]*v.w, per row;
//  * 1.0/x and a/b are IEEE divisions; normalize(v) = v / sqrt(dot(v,v)).
#include "rq_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

namespace {

struct V3 {
    float x, y, z;
};

inline float gmin(float x, float y) { return y < x ? y : x; }  // GLSL min
inline float gmax(float x, float y) { return x < y ? y : x; }  // GLSL max
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 muls(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot(V3 a, V3 b) {
    float r = a.x * b.x;
    r = r + a.y * b.y;
    r = r + a.z * b.z;
    return r;
}
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 vmin(V3 a, V3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
inline V3 normalize(V3 v) {
    float l = std::sqrt(dot(v, v));
    return {v.x / l, v.y / l, v.z / l};
}
inline float clamp01(float x) { return gmin(gmax(x, 0.0f), 1.0f); }

inline int32_t f2i(float f) {
    int32_t i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline V3 ld3(const float* p) { return {p[0], p[1], p[2]}; }

// glm/GLSL column-major mat4 * vec4, returning xyz.
inline V3 xform(const float* m, V3 v, float w) {
    V3 r;
    r.x = m[0] * v.x;
    r.x = r.x + m[4] * v.y;
    r.x = r.x + m[8] * v.z;
    r.x = r.x + m[12] * w;
    r.y = m[1] * v.x;
    r.y = r.y + m[5] * v.y;
    r.y = r.y + m[9] * v.z;
    r.y = r.y + m[13] * w;
    r.z = m[2] * v.x;
    r.z = r.z + m[6] * v.y;
    r.z = r.z + m[10] * v.z;
    r.z = r.z + m[14] * w;
    return r;
}

struct Scene {
    const float* nodes;  // 16 floats per stack node, 8 per stackless node
    int64_t n_nodes;
    const int32_t* tris;
    const float* verts;  // 8 words per vertex; position = first 3
    const orc_entity* ents;
    int n_ents;
    int layout;
};

inline V3 vpos(const Scene& s, int32_t vi) { return ld3(s.verts + (int64_t)vi * 8); }

// RayTriangle, Include/TraverseBVHStack.glsl:87-105 (identical in TraverseBVHStackless.glsl:79-97).
inline void ray_triangle(V3 ro, V3 rd, V3 v0, V3 v1, V3 v2, float& t, float& u, float& v) {
    V3 v1v0 = sub(v1, v0);
    V3 v2v0 = sub(v2, v0);
    V3 rov0 = sub(ro, v0);
    V3 n = cross(v1v0, v2v0);
    V3 q = cross(rov0, rd);
    float d = 1.0f / dot(rd, n);
    u = d * dot(neg(q), v2v0);
    v = d * dot(q, v1v0);
    t = d * dot(neg(n), rov0);
    if (u < 0.0f || v < 0.0f || (u + v) > 1.0f) t = -1.0f;
}

// RayBounds (stack), Include/TraverseBVHStack.glsl:107-116.
inline float ray_bounds_stack(V3 ro, V3 invdir, V3 bmin, V3 bmax, float maxt) {
    V3 f = mul(sub(bmax, ro), invdir);
    V3 n = mul(sub(bmin, ro), invdir);
    V3 tmax = vmax(f, n);
    V3 tmin = vmin(f, n);
    float t1 = gmin(gmin(tmax.x, gmin(tmax.y, tmax.z)), maxt);
    float t0 = gmax(gmax(tmin.x, gmax(tmin.y, tmin.z)), 0.0f);
    return (t1 >= t0) ? (t0 > 0.0f ? t0 : t1) : -1.0f;
}

// RayBounds (stackless), Include/TraverseBVHStackless.glsl:67-75 (max3/min3) and 100-109.
inline float ray_bounds_stackless(V3 bmin, V3 bmax, V3 ro, V3 invdir, float t_min, float t_max) {
    V3 t0 = mul(sub(bmin, ro), invdir);
    V3 t1 = mul(sub(bmax, ro), invdir);
    V3 a = vmin(t0, t1);
    V3 b = vmax(t0, t1);
    float tmin = gmax(gmax(gmax(a.x, a.y), a.z), t_min);
    float tmax = gmin(gmin(b.x, gmin(b.y, b.z)), t_max);
    return (tmax >= tmin) ? tmin : -1.0f;
}

// ComputeBarycentrics, Include/TraverseBVHStack.glsl:150-166.
inline void barycentrics(V3 p, V3 a, V3 b, V3 c, float& u, float& v, float& w) {
    V3 v0 = sub(b, a), v1 = sub(c, a), v2 = sub(p, a);
    float d00 = dot(v0, v0);
    float d01 = dot(v0, v1);
    float d11 = dot(v1, v1);
    float d20 = dot(v2, v0);
    float d21 = dot(v2, v1);
    float denom = d00 * d11 - d01 * d01;
    v = (d11 * d20 - d01 * d21) / denom;
    w = (d00 * d21 - d01 * d20) / denom;
    u = 1.0f - v - w;
}

struct Best {
    float tmax;     // running TMax
    float closest;  // ClosestTraversal
    int32_t tri;
    int32_t mesh;
};

// Triangle acceptance: the reference keeps the first hit found (`t > 0 && t < TMax`,
// TraverseBVHStack.glsl:239); the lower-index rule also accepts an exact tie in t when the
// triangle index is lower, which makes the result independent of traversal order.
inline bool accept(float t, float tmin, int32_t idx, const Best& b, int tie) {
    if (!(t > tmin)) return false;
    if (t < b.tmax) return true;
    return tie == ORC_TIE_LOWER_INDEX && t == b.tmax && idx < b.tri;
}

inline void test_leaf(const Scene& s, V3 ro, V3 rd, int32_t start, int32_t len, float tmin,
                      Best& b, int tie, int32_t& tests) {
    for (int32_t idx = start; idx < start + len; ++idx) {
        const int32_t* tr = s.tris + (int64_t)idx * 4;
        float t, u, v;
        ray_triangle(ro, rd, vpos(s, tr[0]), vpos(s, tr[1]), vpos(s, tr[2]), t, u, v);
        ++tests;
        if (accept(t, tmin, idx, b, tie)) {
            b.tmax = t;
            b.closest = t;
            b.mesh = tr[3];
            b.tri = idx;
        }
    }
}

// IntersectBVHStack, Include/TraverseBVHStack.glsl:168-324.  `b` carries TMax in and the best
// hit out.  Returns the iteration count.
int32_t bvh_stack_closest(const Scene& s, V3 ro, V3 rd, int32_t start, int32_t count, float tmin,
                          Best& b, int tie, int32_t& tests) {
    V3 inv = {1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z};
    int32_t stack[64];
    int32_t sp = 0;
    int32_t iters = 0;
    int32_t cur = start;
    const int64_t total = s.n_nodes;
    while (iters < 1024) {
        // Bounds guard, TraverseBVHStack.glsl:201-205.  `cur >= total` replaces the reference's
        // `cur > u_TotalNodes`, whose equality case reads one node past the buffer.
        if (sp >= 64 || sp < 0 || cur < start || cur > start + count || cur < 0 || cur >= total)
            break;
        ++iters;
        const float* nd = s.nodes + (int64_t)cur * 16;
        const int32_t lw = f2i(nd[3]), rw = f2i(nd[11]);
        const bool lleaf = lw != -1, rleaf = rw != -1;
        float lt = lleaf ? -1.0f : ray_bounds_stack(ro, inv, ld3(nd + 0), ld3(nd + 4), b.tmax);
        float rt = rleaf ? -1.0f : ray_bounds_stack(ro, inv, ld3(nd + 8), ld3(nd + 12), b.tmax);
        if (lleaf) test_leaf(s, ro, rd, lw >> 4, lw & 0xF, tmin, b, tie, tests);
        if (rleaf) test_leaf(s, ro, rd, rw >> 4, rw & 0xF, tmin, b, tie, tests);
        if (lt > 0.0f && rt > 0.0f) {
            cur = f2i(nd[7]) + start;
            int32_t post = f2i(nd[15]) + start;
            if (rt < lt) {
                int32_t tmp = cur;
                cur = post;
                post = tmp;
            }
            if (sp >= 63) break;
            stack[sp++] = post;
            continue;
        } else if (lt > 0.0f) {
            cur = f2i(nd[7]) + start;
            continue;
        } else if (rt > 0.0f) {
            cur = f2i(nd[15]) + start;
            continue;
        }
        if (sp <= 0) break;
        cur = stack[--sp];
    }
    return iters;
}

// IntersectBVHStackless, Include/TraverseBVHStackless.glsl:175-278.
int32_t bvh_stackless_closest(const Scene& s, V3 ro, V3 rd, int32_t start, int32_t count,
                              float tmin, Best& b, int tie, int32_t& tests) {
    V3 inv = {1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z};
    int32_t iters = 0;
    int32_t ptr = start;
    const int64_t total = s.n_nodes;
    while (ptr >= 0 && iters < 1024) {
        if (ptr < start || ptr > start + count || ptr < 0 || ptr >= total) break;
        ++iters;
        const float* nd = s.nodes + (int64_t)ptr * 8;
        float bt = ray_bounds_stackless(ld3(nd), ld3(nd + 4), ro, inv, 0.0001f, b.tmax);
        if (bt > 0.0f && bt < b.tmax) {
            const int32_t packed = f2i(nd[3]);
            if (packed != -1) {
                test_leaf(s, ro, rd, packed >> 4, packed & 0xF, tmin, b, tie, tests);
                ptr = f2i(nd[7]);
                if (ptr < 0) break;
                ptr += start;
                continue;
            }
            ptr++;
            continue;
        }
        ptr = f2i(nd[7]);
        if (ptr < 0) break;
        ptr += start;
    }
    return iters;
}

// IntersectBVHStackOcclusion, Include/TraverseBVHStack.glsl:509-657.  Returns hit t or -1.
float bvh_stack_any(const Scene& s, V3 ro, V3 rd, int32_t start, int32_t count, float tmin,
                    float tmax, int32_t& iters, int32_t& tests) {
    V3 inv = {1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z};
    int32_t stack[64];
    int32_t sp = 0;
    int32_t cur = start;
    const int64_t total = s.n_nodes;
    int32_t it = 0;
    while (it < 1024) {
        if (sp >= 64 || sp < 0 || cur < start || cur > start + count || cur < 0 || cur >= total)
            break;
        ++it;
        ++iters;
        const float* nd = s.nodes + (int64_t)cur * 16;
        const int32_t lw = f2i(nd[3]), rw = f2i(nd[11]);
        const bool lleaf = lw != -1, rleaf = rw != -1;
        float lt = lleaf ? -1.0f : ray_bounds_stack(ro, inv, ld3(nd + 0), ld3(nd + 4), tmax);
        float rt = rleaf ? -1.0f : ray_bounds_stack(ro, inv, ld3(nd + 8), ld3(nd + 12), tmax);
        for (int side = 0; side < 2; ++side) {
            const bool leaf = side == 0 ? lleaf : rleaf;
            if (!leaf) continue;
            const int32_t w = side == 0 ? lw : rw;
            for (int32_t idx = w >> 4; idx < (w >> 4) + (w & 0xF); ++idx) {
                const int32_t* tr = s.tris + (int64_t)idx * 4;
                float t, u, v;
                ray_triangle(ro, rd, vpos(s, tr[0]), vpos(s, tr[1]), vpos(s, tr[2]), t, u, v);
                ++tests;
                if (t > tmin && t < tmax) return t;
            }
        }
        if (lt > 0.0f && rt > 0.0f) {
            cur = f2i(nd[7]) + start;
            int32_t post = f2i(nd[15]) + start;
            if (rt < lt) {
                int32_t tmp = cur;
                cur = post;
                post = tmp;
            }
            if (sp >= 63) break;
            stack[sp++] = post;
            continue;
        } else if (lt > 0.0f) {
            cur = f2i(nd[7]) + start;
            continue;
        } else if (rt > 0.0f) {
            cur = f2i(nd[15]) + start;
            continue;
        }
        if (sp <= 0) break;
        cur = stack[--sp];
    }
    return -1.0f;
}

// IntersectBVHStacklessOcclusion, Include/TraverseBVHStackless.glsl:463-556.
float bvh_stackless_any(const Scene& s, V3 ro, V3 rd, int32_t start, int32_t count, float tmin,
                        float tmax, int32_t& iters, int32_t& tests) {
    V3 inv = {1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z};
    int32_t ptr = start;
    int32_t it = 0;
    const int64_t total = s.n_nodes;
    while (ptr >= 0 && it < 1024) {
        if (ptr < start || ptr > start + count || ptr < 0 || ptr >= total) break;
        ++it;
        ++iters;
        const float* nd = s.nodes + (int64_t)ptr * 8;
        float bt = ray_bounds_stackless(ld3(nd), ld3(nd + 4), ro, inv, 0.0001f, tmax);
        if (bt > 0.0f && bt < tmax) {
            const int32_t packed = f2i(nd[3]);
            if (packed != -1) {
                for (int32_t idx = packed >> 4; idx < (packed >> 4) + (packed & 0xF); ++idx) {
                    const int32_t* tr = s.tris + (int64_t)idx * 4;
                    float t, u, v;
                    ray_triangle(ro, rd, vpos(s, tr[0]), vpos(s, tr[1]), vpos(s, tr[2]), t, u,
                                 v);
                    ++tests;
                    if (t > tmin && t < tmax) return t;
                }
                ptr = f2i(nd[7]);
                if (ptr < 0) break;
                ptr += start;
                continue;
            }
            ptr++;
            continue;
        }
        ptr = f2i(nd[7]);
        if (ptr < 0) break;
        ptr += start;
    }
    return -1.0f;
}

inline float ent_alpha(const orc_entity& e) {
    float a;
    std::memcpy(&a, &e.data[1], 4);
    return a;
}

// IntersectScene / IntersectSceneIgnoreTransparent, Include/TraverseBVHStack.glsl:327-413
// (stackless: Include/TraverseBVHStackless.glsl:280-366).
void scene_closest(const Scene& s, const orc_ray& r, orc_hit& h, int tie, int flags,
                   int32_t& tests) {
    h.t = h.u = h.v = h.w = -1.0f;
    h.tri = h.mesh = h.entity = -1;
    h.iters = 0;
    if (!(r.tmax > r.tmin)) return;  // inactive ray
    const V3 o = ld3(r.o), d = ld3(r.d);
    float tmax = r.tmax;  // scene TMax (1000000.0 in the reference, :331)
    float closest = -1.0f;
    int32_t mesh = -1, tri = -1, ent = -1, last = 0;
    for (int i = 0; i < s.n_ents; ++i) {
        const orc_entity& e = s.ents[i];
        if ((flags & ORC_FLAG_IGNORE_TRANSPARENT) && ent_alpha(e) < 0.99f) continue;
        V3 ro = xform(e.inverse, o, 1.0f);
        V3 rd = xform(e.inverse, d, 0.0f);
        // Per-BVH call: TMax is the running scene TMax and ClosestTraversal starts at -1, so T
        // is this BVH's closest hit only.  Under the lower-index rule the best triangle so far
        // seeds the tie comparison.
        Best bb{tmax, -1.0f, tie == ORC_TIE_LOWER_INDEX ? tri : -1, -1};
        int32_t it = s.layout == ORC_STACK
                         ? bvh_stack_closest(s, ro, rd, e.node_offset, e.node_count, r.tmin, bb,
                                             tie, tests)
                         : bvh_stackless_closest(s, ro, rd, e.node_offset, e.node_count, r.tmin,
                                                 bb, tie, tests);
        h.iters += it;
        last = it;  // IntersectScene hands one `out int Iters` to every walk (:337-349)
        const float T = bb.closest;
        if (T > 0.0f && (T < tmax || (tie == ORC_TIE_LOWER_INDEX && T == tmax && bb.tri < tri))) {
            tmax = T;
            closest = T;
            mesh = bb.mesh;
            tri = bb.tri;
            ent = i;
        }
    }
    // the reference reports the last walked entity's count; the sum over entities otherwise
    if (flags & ORC_FLAG_REF_COMPAT) h.iters = last;
    if (closest > 0.0f) {
        h.tri = tri;
        h.mesh = mesh;
        h.entity = ent;
        const bool report = (flags & ORC_FLAG_REF_COMPAT) ? tri > 0 : tri >= 0;
        if (report) {
            const orc_entity& e = s.ents[ent];
            V3 ro = xform(e.inverse, o, 1.0f);
            V3 rd = xform(e.inverse, d, 0.0f);
            const int32_t* tr = s.tris + (int64_t)tri * 4;
            V3 p = add(ro, muls(rd, closest));
            float u, v, w;
            barycentrics(p, vpos(s, tr[0]), vpos(s, tr[1]), vpos(s, tr[2]), u, v, w);
            h.t = closest;
            h.u = u;
            h.v = v;
            h.w = w;
        }
    }
}

// IntersectSceneOcclusion, Include/TraverseBVHStack.glsl:659-676 (stackless: :558-575), with the
// per-ray TMax passed to every BVH (the per-BVH functions take TMax, :509).
bool scene_any(const Scene& s, const orc_ray& r, int32_t& iters, int32_t& tests) {
    if (!(r.tmax > r.tmin)) return false;
    const V3 o = ld3(r.o), d = ld3(r.d);
    for (int i = 0; i < s.n_ents; ++i) {
        const orc_entity& e = s.ents[i];
        V3 ro = xform(e.inverse, o, 1.0f);
        V3 rd = xform(e.inverse, d, 0.0f);
        float T = s.layout == ORC_STACK
                      ? bvh_stack_any(s, ro, rd, e.node_offset, e.node_count, r.tmin, r.tmax,
                                      iters, tests)
                      : bvh_stackless_any(s, ro, rd, e.node_offset, e.node_count, r.tmin,
                                          r.tmax, iters, tests);
        if (T > 0.0f) return true;
    }
    return false;
}

Scene make_scene(const orc_scene* s) {
    return Scene{static_cast<const float*>(s->nodes), s->n_nodes, s->tris,
                 static_cast<const float*>(s->verts), s->ents, s->n_ents, s->layout};
}

template <class F>
void parallel_for(int64_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 4096) {
        f(int64_t(0), n);
        return;
    }
    std::vector<std::thread> th;
    const int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        const int64_t b = t * chunk, e = std::min<int64_t>(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([=] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

// ---- AABB collision queries -------------------------------------------------------------------
// Collide.comp with Include/CollideBVHStack.glsl (stack layout) and
// Include/CollideBVHStackless.glsl (stackless layout; the same walk as Physics.cpp:79-174).

// BoxTriangleOverlap, CollideBVHStack.glsl:104-152 / Physics.cpp:29-77: separating-axis test on the
// nine edge cross products, with the full box extent as e.  The reference fills AxisUxFx[5] with
// cross(u2, f2) (a repeat of [8]) where cross(u1, f2) belongs; ref_axis keeps that.
bool box_triangle_overlap(V3 v0, V3 v1, V3 v2, V3 bmin, V3 bmax, bool ref_axis) {
    const V3 c = {(bmin.x + bmax.x) / 2.0f, (bmin.y + bmax.y) / 2.0f, (bmin.z + bmax.z) / 2.0f};
    const V3 e = sub(bmax, bmin);
    v0 = sub(v0, c);
    v1 = sub(v1, c);
    v2 = sub(v2, c);
    const V3 f0 = sub(v1, v0), f1 = sub(v2, v1), f2 = sub(v0, v2);
    const V3 u0 = {1.0f, 0.0f, 0.0f}, u1 = {0.0f, 1.0f, 0.0f}, u2 = {0.0f, 0.0f, 1.0f};
    V3 ax[9];
    ax[0] = cross(u0, f0);
    ax[1] = cross(u0, f1);
    ax[2] = cross(u0, f2);
    ax[3] = cross(u1, f0);
    ax[4] = cross(u1, f1);
    ax[5] = ref_axis ? cross(u2, f2) : cross(u1, f2);
    ax[6] = cross(u2, f0);
    ax[7] = cross(u2, f1);
    ax[8] = cross(u2, f2);
    for (int i = 0; i < 9; ++i) {
        const V3 a = ax[i];
        const float p0 = dot(v0, a), p1 = dot(v1, a), p2 = dot(v2, a);
        float r = e.x * std::fabs(dot(u0, a));
        r = r + e.y * std::fabs(dot(u1, a));
        r = r + e.z * std::fabs(dot(u2, a));
        if (gmax(-gmax(gmax(p0, p1), p2), gmin(gmin(p0, p1), p2)) > r) return false;
    }
    return true;
}

// AABBAABBOverlap and AABBAABBOverlapF (squared centre distance, -1 when apart),
// CollideBVHStack.glsl:90-102 (Physics.cpp:23-27).
inline bool aabb_overlap(V3 amin, V3 amax, V3 bmin, V3 bmax) {
    return (amin.x <= bmax.x && amax.x >= bmin.x) && (amin.y <= bmax.y && amax.y >= bmin.y) &&
           (amin.z <= bmax.z && amax.z >= bmin.z);
}
inline float aabb_overlap_f(V3 amin, V3 amax, V3 bmin, V3 bmax) {
    const bool hit = aabb_overlap(amin, amax, bmin, bmax);
    const V3 ca = {(amin.x + amax.x) / 2.0f, (amin.y + amax.y) / 2.0f, (amin.z + amax.z) / 2.0f};
    const V3 cb = {(bmin.x + bmax.x) / 2.0f, (bmin.y + bmax.y) / 2.0f, (bmin.z + bmax.z) / 2.0f};
    const V3 d = sub(cb, ca);
    const float dist = dot(d, d);
    return hit ? dist : -1.0f;
}

// One leaf's triangles against the box; tri = the reported index (the reference's stack walk
// reports the index inside the leaf, ref_tri).
inline bool collide_leaf(const Scene& s, int32_t packed, V3 bmin, V3 bmax, bool ref_axis, bool leaf_index,
                         int32_t& mesh, int32_t& tri) {
    const int32_t st = packed >> 4, len = packed & 0xF;
    for (int32_t i = 0; i < len; ++i) {
        const int32_t* t = s.tris + (int64_t)(st + i) * 4;
        if (box_triangle_overlap(vpos(s, t[0]), vpos(s, t[1]), vpos(s, t[2]), bmin, bmax, ref_axis)) {
            mesh = t[3];
            tri = leaf_index ? i : st + i;
            return true;
        }
    }
    return false;
}

// CollideBVH, CollideBVHStack.glsl:154-299.
bool collide_bvh_stack(const Scene& s, V3 bmin, V3 bmax, int32_t start, int32_t count, bool ref, int32_t& mesh,
                       int32_t& tri) {
    int32_t stack[64];
    int32_t sp = 0, iters = 0, cur = start;
    while (iters < 1024) {
        if (sp >= 64 || sp < 0 || cur < start || cur > start + count || cur < 0 || cur >= s.n_nodes) break;
        ++iters;
        const float* nd = s.nodes + (int64_t)cur * 16;
        const V3 lmin = ld3(nd), lmax = ld3(nd + 4), rmin = ld3(nd + 8), rmax = ld3(nd + 12);
        const int32_t lw = f2i(nd[3]), rw = f2i(nd[11]);
        const bool ll = lw != -1, rl = rw != -1;
        const float lt = ll ? -1.0f : aabb_overlap_f(lmin, lmax, bmin, bmax);
        const float rt = rl ? -1.0f : aabb_overlap_f(rmin, rmax, bmin, bmax);
        if (ll && collide_leaf(s, lw, bmin, bmax, ref, ref, mesh, tri)) return true;
        if (rl && collide_leaf(s, rw, bmin, bmax, ref, ref, mesh, tri)) return true;
        if (lt > 0.0f && rt > 0.0f) {
            int32_t a = f2i(nd[7]) + start, b = f2i(nd[15]) + start;
            if (rt < lt) {
                const int32_t x = a;
                a = b;
                b = x;
            }
            cur = a;
            if (sp >= 63) break;
            stack[sp++] = b;
            continue;
        } else if (lt > 0.0f) {
            cur = f2i(nd[7]) + start;
            continue;
        } else if (rt > 0.0f) {
            cur = f2i(nd[15]) + start;
            continue;
        }
        if (sp <= 0) break;
        cur = stack[--sp];
    }
    return false;
}

// CollideBVH, CollideBVHStackless.glsl:131-223 (Physics.cpp:79-174).
bool collide_bvh_stackless(const Scene& s, V3 bmin, V3 bmax, int32_t start, int32_t count, bool ref,
                           int32_t& mesh, int32_t& tri) {
    int32_t iters = 0, ptr = start;
    while (ptr >= 0 && iters < 1024) {
        if (ptr < start || ptr > start + count || ptr < 0 || ptr >= s.n_nodes) break;
        ++iters;
        const float* nd = s.nodes + (int64_t)ptr * 8;
        if (aabb_overlap(ld3(nd), ld3(nd + 4), bmin, bmax)) {
            const int32_t packed = f2i(nd[3]);
            if (packed != -1) {
                if (collide_leaf(s, packed, bmin, bmax, ref, false, mesh, tri)) return true;
                const int32_t nx = f2i(nd[7]);
                if (nx < 0) break;
                ptr = nx + start;
                continue;
            }
            ++ptr;
            continue;
        }
        const int32_t nx = f2i(nd[7]);
        if (nx < 0) break;
        ptr = nx + start;
    }
    return false;
}

// CollideScene, CollideBVHStack.glsl:301-323 (CollideBVHStackless.glsl:225-247): entities in order, the first collision wins; the box
// corners are moved by the entity's inverse matrix (two corners, as the reference does).
void collide_scene(const Scene& s, const float box[8], bool ref, int32_t out[4]) {
    out[0] = 0;
    out[1] = out[2] = out[3] = -1;
    const V3 wmin = ld3(box), wmax = ld3(box + 4);
    for (int i = 0; i < s.n_ents; ++i) {
        const orc_entity& e = s.ents[i];
        const V3 bmin = xform(e.inverse, wmin, 1.0f), bmax = xform(e.inverse, wmax, 1.0f);
        int32_t mesh = -1, tri = -1;
        const bool hit = s.layout == ORC_STACKLESS
                             ? collide_bvh_stackless(s, bmin, bmax, e.node_offset, e.node_count, ref, mesh, tri)
                             : collide_bvh_stack(s, bmin, bmax, e.node_offset, e.node_count, ref, mesh, tri);
        if (hit) {
            out[0] = 1;
            out[1] = i;
            out[2] = mesh;
            out[3] = tri;
            return;
        }
    }
}

// ---- GI ray generation and shading ---------------------------------------------------------

// Exact binary16 -> binary32 conversion (GLSL unpackHalf2x16 component).
float half_to_float(uint32_t h) {
    const uint32_t sign = (h >> 15) & 1u, exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign << 31;
        } else {  // subnormal: normalise
            int e = -1;
            uint32_t m = man;
            do {
                ++e;
                m <<= 1;
            } while ((m & 0x400u) == 0);
            bits = (sign << 31) | (uint32_t(127 - 15 - e) << 23) | ((m & 0x3FFu) << 13);
        }
    } else if (exp == 31) {
        bits = (sign << 31) | 0x7F800000u | (man << 13);
    } else {
        bits = (sign << 31) | ((exp + 112u) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// UnpackNormal, Include/TraverseBVHStack.glsl:417-420.
V3 unpack_normal(const Scene& s, int32_t vi) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(s.verts + (int64_t)vi * 8) + 4;
    return {half_to_float(w[0] & 0xFFFFu), half_to_float(w[0] >> 16), half_to_float(w[1] & 0xFFFFu)};
}

// Shading normal at a hit: GetData's interpolated vertex normal (TraverseBVHStack.glsl:438) or the
// geometric normal.
V3 hit_normal(const Scene& s, const orc_hit& h, int mode) {
    const int32_t* tr = s.tris + (int64_t)h.tri * 4;
    if (mode == 0) {
        V3 a = muls(unpack_normal(s, tr[0]), h.u);
        V3 b = muls(unpack_normal(s, tr[1]), h.v);
        V3 c = muls(unpack_normal(s, tr[2]), h.w);
        return normalize(add(add(a, b), c));
    }
    V3 A = vpos(s, tr[0]), B = vpos(s, tr[1]), C = vpos(s, tr[2]);
    return normalize(cross(sub(B, A), sub(C, A)));
}

// ---- GetData's albedo (Include/TraverseBVHStack.glsl:422-455) ------------------------------
// ModelColor of the mesh, or its texture at the hit's UV: the three vertices' half-packed
// texture coordinates (Vertex.PackedData.w) weighted by the barycentrics (u, v, w), then
// texture() of a compute shader: level 0, GL_LINEAR (bilinear, texel centres at half integers),
// GL_REPEAT or GL_CLAMP_TO_EDGE, sRGB channels decoded (IEC 61966-2-1) before filtering.

float srgb_decode(uint32_t c) {
    static const std::vector<float> lut = [] {
        std::vector<float> t(256);
        for (int k = 0; k < 256; ++k) {
            const double x = k / 255.0;
            t[k] = float(x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4));
        }
        return t;
    }();
    return lut[c & 0xFFu];
}

V3 texel_rgb(const orc_materials& m, int32_t first, int32_t w, int32_t i, int32_t j, bool srgb) {
    const uint32_t t = m.texels[first + int64_t(j) * w + i];
    const uint32_t r = t & 0xFFu, g = (t >> 8) & 0xFFu, b = (t >> 16) & 0xFFu;
    if (srgb) return {srgb_decode(r), srgb_decode(g), srgb_decode(b)};
    return {float(r) / 255.0f, float(g) / 255.0f, float(b) / 255.0f};
}

int32_t wrap_index(int32_t i, int32_t n, bool clamp) {
    if (clamp) return std::min(std::max(i, 0), n - 1);
    const int32_t r = i % n;
    return r < 0 ? r + n : r;
}

V3 sample_bilinear(const orc_materials& m, int32_t t, float u, float v) {
    const int32_t* d = m.tex + 4 * t;
    const bool srgb = d[3] & 1, clamp = d[3] & 2;
    const float x = u * float(d[1]) - 0.5f, y = v * float(d[2]) - 0.5f;
    const float lim = 1073741824.0f;
    const float fx = std::min(std::max(std::floor(x), -lim), lim), fy = std::min(std::max(std::floor(y), -lim), lim);
    const float a = std::min(std::max(x - fx, 0.0f), 1.0f), b = std::min(std::max(y - fy, 0.0f), 1.0f);
    const int32_t ix = int32_t(fx), iy = int32_t(fy);
    const int32_t i0 = wrap_index(ix, d[1], clamp), i1 = wrap_index(ix + 1, d[1], clamp);
    const int32_t j0 = wrap_index(iy, d[2], clamp), j1 = wrap_index(iy + 1, d[2], clamp);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    const V3 t00 = texel_rgb(m, d[0], d[1], i0, j0, srgb), t10 = texel_rgb(m, d[0], d[1], i1, j0, srgb);
    const V3 t01 = texel_rgb(m, d[0], d[1], i0, j1, srgb), t11 = texel_rgb(m, d[0], d[1], i1, j1, srgb);
    return add(add(add(muls(t00, w00), muls(t10, w10)), muls(t01, w01)), muls(t11, w11));
}

// The hit's texture coordinates (TraverseBVHStack.glsl:436): the vertices' half-packed UVs
// weighted by the barycentrics u, v, w, summed left to right.
void hit_uv(const Scene& s, const orc_hit& h, float& u, float& v) {
    const int32_t* tr = s.tris + int64_t(h.tri) * 4;
    const uint32_t* va = reinterpret_cast<const uint32_t*>(s.verts + int64_t(tr[0]) * 8);
    const uint32_t* vb = reinterpret_cast<const uint32_t*>(s.verts + int64_t(tr[1]) * 8);
    const uint32_t* vc = reinterpret_cast<const uint32_t*>(s.verts + int64_t(tr[2]) * 8);
    u = (half_to_float(va[7] & 0xFFFFu) * h.u + half_to_float(vb[7] & 0xFFFFu) * h.v) + half_to_float(vc[7] & 0xFFFFu) * h.w;
    v = (half_to_float(va[7] >> 16) * h.u + half_to_float(vb[7] >> 16) * h.v) + half_to_float(vc[7] >> 16) * h.w;
}

V3 hit_albedo(const Scene& s, const orc_materials& m, const orc_hit& h) {
    if (h.mesh >= 0 && h.mesh < m.n_mesh_tex && h.t > 0.0f && m.mesh_tex[h.mesh] >= 0) {
        float u, v;
        hit_uv(s, h, u, v);
        return sample_bilinear(m, m.mesh_tex[h.mesh], u, v);
    }
    if (h.mesh >= 0 && h.mesh < m.n_albedo) return ld3(m.albedo + 3 * h.mesh);
    return {0.8f, 0.8f, 0.8f};
}

float u01(uint32_t h) { return float(h >> 8) * (1.0f / 16777216.0f); }

uint32_t pcg_hash(uint32_t x) {
    uint32_t state = x * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// sin(2*pi*x), cos(2*pi*x) for x in [0,1): quadrant reduction, reflection to [0, pi/4], then
// Taylor polynomials (sin to x^9, cos to x^10) evaluated by Horner without contraction.
void sincos_turns(float x, float& so, float& co) {
    const float x4 = x * 4.0f;
    const float q = std::floor(x4);
    float f = x4 - q;
    const int quad = int(q) & 3;
    const bool refl = f > 0.5f;
    if (refl) f = 1.0f - f;
    const float th = f * 1.57079637f;
    const float t2 = th * th;
    float sp = 2.75573192e-06f;
    sp = sp * t2 + -1.98412698e-04f;
    sp = sp * t2 + 8.33333333e-03f;
    sp = sp * t2 + -1.66666667e-01f;
    sp = sp * t2 + 1.0f;
    float S = th * sp;
    float cp = -2.75573192e-07f;
    cp = cp * t2 + 2.48015873e-05f;
    cp = cp * t2 + -1.38888889e-03f;
    cp = cp * t2 + 4.16666667e-02f;
    cp = cp * t2 + -0.5f;
    cp = cp * t2 + 1.0f;
    float C = cp;
    if (refl) {
        float tmp = S;
        S = C;
        C = tmp;
    }
    switch (quad) {
        case 0: so = S; co = C; break;
        case 1: so = C; co = -S; break;
        case 2: so = -S; co = -C; break;
        default: so = -C; co = S; break;
    }
}

// CosWeightedHemisphere, Include/Sampling.glsl:1-12, with cos/sin(2*pi*r.x) from sincos_turns.
V3 cos_weighted_hemisphere(V3 n, float rx_, float ry_) {
    V3 uu = normalize(cross(n, V3{0.0f, 1.0f, 1.0f}));
    V3 vv = cross(uu, n);
    float ra = std::sqrt(ry_);
    float s, c;
    sincos_turns(rx_, s, c);
    float rx = ra * c;
    float ry = ra * s;
    float rz = std::sqrt(1.0f - ry_);
    V3 rr = add(add(muls(uu, rx), muls(vv, ry)), muls(n, rz));
    return normalize(rr);
}

uint32_t sample_key(uint32_t seed, uint32_t ray, uint32_t dim) {
    return pcg_hash(pcg_hash(pcg_hash(seed) + ray) + dim);
}

// The value GL_R11F_G11F_B10F holds for x in a channel with `mbits` mantissa bits (5-bit exponent,
// bias 15, no sign), converted as the GL specification (section "Unsigned 11-Bit / 10-Bit
// Floating-Point Numbers") describes: the closest representable finite value (ties to even),
// negative values and -inf to 0, values above the largest finite one to it, +inf and NaN kept.
float small_ufloat(float x, int mbits) {
    if (std::isnan(x) || x == INFINITY) return x;
    if (!(x > 0.0f)) return 0.0f;
    const float maxf = std::ldexp(2.0f - std::ldexp(1.0f, -mbits), 15);
    if (x >= maxf) return maxf;
    int k;
    std::frexp(x, &k);
    const int e = std::max(k - 1, -14);
    const float step = std::ldexp(1.0f, e - mbits);
    const float q = std::nearbyint(x / step) * step;
    return q > maxf ? maxf : q;
}

}  // namespace

extern "C" {

void orc_closest(const orc_scene* sc, const orc_ray* rays, int64_t n, orc_hit* hits, int tie,
                 int flags, int nthreads, int32_t* tri_tests) {
    const Scene s = make_scene(sc);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            int32_t tests = 0;
            scene_closest(s, rays[i], hits[i], tie, flags, tests);
            if (tri_tests) tri_tests[i] = tests;
        }
    });
}

void orc_anyhit(const orc_scene* sc, const orc_ray* rays, int64_t n, uint8_t* occluded,
                int nthreads, int32_t* iters, int32_t* tri_tests) {
    const Scene s = make_scene(sc);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            int32_t it = 0, tests = 0;
            occluded[i] = scene_any(s, rays[i], it, tests) ? 1 : 0;
            if (iters) iters[i] = it;
            if (tri_tests) tri_tests[i] = tests;
        }
    });
}

void orc_ray_triangle(const float ro[3], const float rd[3], const float v0[3], const float v1[3],
                      const float v2[3], float out[3]) {
    ray_triangle(ld3(ro), ld3(rd), ld3(v0), ld3(v1), ld3(v2), out[0], out[1], out[2]);
}

float orc_ray_bounds_stack(const float ro[3], const float invdir[3], const float bmin[3],
                           const float bmax[3], float maxt) {
    return ray_bounds_stack(ld3(ro), ld3(invdir), ld3(bmin), ld3(bmax), maxt);
}

float orc_ray_bounds_stackless(const float bmin[3], const float bmax[3], const float ro[3],
                               const float invdir[3], float t_min, float t_max) {
    return ray_bounds_stackless(ld3(bmin), ld3(bmax), ld3(ro), ld3(invdir), t_min, t_max);
}

void orc_barycentrics(const float p[3], const float a[3], const float b[3], const float c[3],
                      float out[3]) {
    barycentrics(ld3(p), ld3(a), ld3(b), ld3(c), out[0], out[1], out[2]);
}

float orc_small_ufloat(float x, int mbits) { return small_ufloat(x, mbits); }

uint32_t orc_pcg_hash(uint32_t x) { return pcg_hash(x); }
void orc_sincos_turns(float x, float* s, float* c) { sincos_turns(x, *s, *c); }
void orc_cos_hemisphere(const float* normals, const float* r, int64_t n, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        const V3 d = cos_weighted_hemisphere(ld3(normals + 3 * i), r[2 * i], r[2 * i + 1]);
        out[3 * i] = d.x;
        out[3 * i + 1] = d.y;
        out[3 * i + 2] = d.z;
    }
}

void orc_gi_raygen(const orc_scene* sc, const orc_ray* primary, const orc_hit* hits, int64_t n,
                   int32_t spp, uint32_t seed, float origin_offset, float ray_tmax,
                   int32_t normal_mode, int nthreads, orc_ray* out) {
    const Scene s = make_scene(sc);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const orc_hit& h = hits[i];
            for (int k = 0; k < spp; ++k) {
                orc_ray& o = out[i * spp + k];
                if (!(h.t > 0.0f)) {
                    o = orc_ray{{0, 0, 0}, 0.0f, {0, 0, 1}, -1.0f};
                    continue;
                }
                const V3 ro = ld3(primary[i].o), rd = ld3(primary[i].d);
                V3 P = add(ro, muls(rd, h.t));
                V3 N = hit_normal(s, h, normal_mode);
                // Face the normal toward the incoming ray (DiffuseTrace.glsl:486-488).
                if (dot(N, rd) > 0.0001f) N = neg(N);
                const uint32_t rid = uint32_t(i * spp + k);
                float r0 = u01(sample_key(seed, rid, 0u));
                float r1 = u01(sample_key(seed, rid, 1u));
                V3 dir = cos_weighted_hemisphere(N, r0, r1);
                V3 org = add(P, muls(N, origin_offset));  // DiffuseTrace.glsl:445
                o.o[0] = org.x; o.o[1] = org.y; o.o[2] = org.z;
                o.d[0] = dir.x; o.d[1] = dir.y; o.d[2] = dir.z;
                o.tmin = 0.0f;
                o.tmax = ray_tmax;
            }
        }
    });
}

void orc_shadow_raygen(const orc_scene* sc, const orc_ray* rays, const orc_hit* hits, int64_t n,
                       const float sun_dir[3], float origin_offset, int32_t normal_mode,
                       int nthreads, orc_ray* out) {
    const Scene s = make_scene(sc);
    const V3 L = neg(ld3(sun_dir));
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const orc_hit& h = hits[i];
            orc_ray& o = out[i];
            if (!(h.t > 0.0f) || !(rays[i].tmax > rays[i].tmin)) {
                o = orc_ray{{0, 0, 0}, 0.0f, {0, 0, 1}, -1.0f};
                continue;
            }
            const V3 ro = ld3(rays[i].o), rd = ld3(rays[i].d);
            V3 P = add(ro, muls(rd, h.t));
            V3 N = hit_normal(s, h, normal_mode);
            if (dot(N, rd) > 0.0001f) N = neg(N);
            V3 org = add(P, muls(N, origin_offset));
            o.o[0] = org.x; o.o[1] = org.y; o.o[2] = org.z;
            o.d[0] = L.x; o.d[1] = L.y; o.d[2] = L.z;
            o.tmin = 0.0f;
            o.tmax = 1000000.0f;
        }
    });
}

// Rays of bounce `bounce` of the RT second-bounce loop (DiffuseTrace.glsl:502-536): from hit i of
// `rays` (alive[i] != 0), origin P + N * offset (0.02 in the reference, :518) and a cosine
// direction about the facing normal (:519) from sample sample_id[i], dimensions 2 + 2*bounce and
// 3 + 2*bounce of the counter-based hash that draws the first GI ray (dimensions 0 and 1).
void orc_bounce_raygen(const orc_scene* sc, const orc_ray* rays, const orc_hit* hits, const uint8_t* alive,
                       const uint32_t* sample_id, int64_t n, uint32_t seed, int32_t bounce, float offset,
                       float ray_tmax, int32_t normal_mode, int nthreads, orc_ray* out) {
    const Scene s = make_scene(sc);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const orc_hit& h = hits[i];
            orc_ray& o = out[i];
            if (!alive[i] || !(h.t > 0.0f)) {
                o = orc_ray{{0, 0, 0}, 0.0f, {0, 0, 1}, -1.0f};
                continue;
            }
            const V3 ro = ld3(rays[i].o), rd = ld3(rays[i].d);
            const V3 P = add(ro, muls(rd, h.t));
            V3 N = hit_normal(s, h, normal_mode);
            if (dot(N, rd) > 0.0001f) N = neg(N);
            const float r0 = u01(sample_key(seed, sample_id[i], 2u + 2u * uint32_t(bounce)));
            const float r1 = u01(sample_key(seed, sample_id[i], 3u + 2u * uint32_t(bounce)));
            const V3 dir = cos_weighted_hemisphere(N, r0, r1);
            const V3 org = add(P, muls(N, offset));
            o.o[0] = org.x; o.o[1] = org.y; o.o[2] = org.z;
            o.d[0] = dir.x; o.d[1] = dir.y; o.d[2] = dir.z;
            o.tmin = 0.0f;
            o.tmax = ray_tmax;
        }
    });
}

// ---- Specular reflections (SpecularTrace.glsl:485-596, world-trace path) ----------------------

namespace {

// reflect(I, N) = I - 2 dot(N, I) N.
V3 reflect_dir(V3 i, V3 n) { return sub(i, muls(n, 2.0f * dot(n, i))); }

// SampleGGXVNDF, Include/Sampling.glsl:63-83, with sin / cos of 2 pi x0 from sincos_turns.
V3 sample_ggx(V3 n, float roughness, float x0, float x1) {
    const float alpha = roughness * roughness;
    const float alpha2 = alpha * alpha;
    float sp, cp;
    sincos_turns(x0, sp, cp);
    const float ct = std::sqrt((1.0f - x1) / (1.0f + (alpha2 - 1.0f) * x1));
    const float st = std::sqrt(1.0f - ct * ct);
    const V3 h = {cp * st, sp * st, ct};
    const V3 up = std::fabs(n.z) < 0.999f ? V3{0.0f, 0.0f, 1.0f} : V3{1.0f, 0.0f, 0.0f};
    const V3 tangent = normalize(cross(up, n));
    const V3 bitangent = cross(n, tangent);
    return normalize(add(add(muls(tangent, h.x), muls(bitangent, h.y)), muls(n, h.z)));
}

float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }

// StochasticReflectionDirection(I, N, 0.9 * roughness) (SpecularTrace.glsl:102-135) with sample
// `rid` of the counter-based hash (dimensions 2k, 2k+1 for try k).
V3 spec_direction(V3 I, V3 N, float roughness, uint32_t seed, uint32_t rid) {
    const float r = roughness * 0.9f;
    if (r < 0.01f) return reflect_dir(I, N);
    V3 micro = N;
    for (uint32_t k = 0; k < 12; ++k) {
        const float x0 = u01(sample_key(seed, rid, 2u * k)) * 0.8f;
        const float x1 = u01(sample_key(seed, rid, 2u * k + 1u)) * 0.7f;
        const V3 smp = sample_ggx(N, r, x0, x1);
        if (dot(smp, N) > 0.001f) {
            micro = smp;
            break;
        }
    }
    return reflect_dir(I, micro);
}

}  // namespace

// Reflection ray per pixel: origin P + N * mix(0.05, 0.1, clamp(1.4 R, 0, 1)) (:509), direction
// StochasticReflectionDirection(normalize(P - origin), N, 0.9 R) (:102-135): a mirror below 0.01,
// else the first of 12 GGX samples (hash dimensions 2k, 2k+1 scaled by 0.8, 0.7) above the surface.
void orc_spec_raygen(const orc_scene* sc, const orc_ray* primary, const orc_hit* hits, int64_t n, uint32_t seed,
                     float roughness, float ray_tmax, int32_t normal_mode, int nthreads, orc_ray* out) {
    const Scene s = make_scene(sc);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const orc_hit& h = hits[i];
            orc_ray& o = out[i];
            if (!(h.t > 0.0f)) {
                o = orc_ray{{0, 0, 0}, 0.0f, {0, 0, 1}, -1.0f};
                continue;
            }
            const V3 ro = ld3(primary[i].o), rd = ld3(primary[i].d);
            const V3 P = add(ro, muls(rd, h.t));
            V3 N = hit_normal(s, h, normal_mode);
            if (dot(N, rd) > 0.0001f) N = neg(N);
            const V3 I = normalize(sub(P, ro));
            const V3 dir = spec_direction(I, N, roughness, seed, uint32_t(i));
            const float off = mixf(0.05f, 0.1f, clamp01(roughness * 1.4f));
            const V3 org = add(P, muls(N, off));
            o.o[0] = org.x; o.o[1] = org.y; o.o[2] = org.z;
            o.d[0] = dir.x; o.d[1] = dir.y; o.d[2] = dir.z;
            o.tmin = 0.0f;
            o.tmax = ray_tmax;
        }
    });
}

// StochasticReflectionDirection for given incident directions and normals (sample rid[i]).
void orc_spec_direction(const float* incident, const float* normals, int64_t n, float roughness, uint32_t seed,
                        const uint32_t* rid, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        const V3 d = spec_direction(ld3(incident + 3 * i), ld3(normals + 3 * i), roughness, seed, rid[i]);
        out[3 * i] = d.x;
        out[3 * i + 1] = d.y;
        out[3 * i + 2] = d.z;
    }
}

// SampleLighting (:420-425) + emissive for a hit, the sky x mix(1.4, 2.65, R) (:435-437) for a
// miss; IsValid, clamp to [0, 6], w = t / 48 (:588-596); 0 where the primary ray missed.
void orc_spec_shade(const orc_scene* sc, const orc_ray* rays, const orc_hit* hits, int64_t n, const uint8_t* lit,
                    const orc_materials* mat, float roughness, const float sun_color[3], const float sky[3],
                    const float ambient[3], int nthreads, float* out4) {
    const Scene s = make_scene(sc);
    const V3 sunc = ld3(sun_color), skyc = ld3(sky), amb = ld3(ambient);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            float* o = out4 + 4 * i;
            if (!(rays[i].tmax > rays[i].tmin)) {
                o[0] = o[1] = o[2] = o[3] = 0.0f;
                continue;
            }
            const orc_hit& h = hits[i];
            float t = h.t;
            V3 rad;
            if (h.t > 0.0f) {
                const V3 alb = hit_albedo(s, *mat, h);
                float em;
                std::memcpy(&em, &s.ents[h.entity].data[0], 4);
                const float l = lit ? (lit[i] ? 1.0f : 0.0f) : 1.0f;
                rad = add(add(muls(mul(alb, sunc), l), mul(muls(alb, 2.0f), amb)), muls(alb, em));
            } else {
                rad = muls(skyc, mixf(1.4f, 2.65f, roughness));
            }
            if (!std::isfinite(rad.x) || !std::isfinite(rad.y) || !std::isfinite(rad.z)) {
                rad = {0.0f, 0.0f, 0.0f};
                t = -1.0f;
            }
            o[0] = gmin(gmax(rad.x, 0.0f), 6.0f);
            o[1] = gmin(gmax(rad.y, 0.0f), 6.0f);
            o[2] = gmin(gmax(rad.z, 0.0f), 6.0f);
            o[3] = t / 48.0f;
        }
    });
}

void orc_hit_normal(const orc_scene* sc, const orc_hit* hits, int64_t n, int32_t normal_mode, float* out3) {
    const Scene s = make_scene(sc);
    for (int64_t i = 0; i < n; ++i) {
        const V3 nn = hit_normal(s, hits[i], normal_mode);
        out3[3 * i] = nn.x;
        out3[3 * i + 1] = nn.y;
        out3[3 * i + 2] = nn.z;
    }
}

void orc_hit_uv(const orc_scene* sc, const orc_hit* hits, int64_t n, float* out2) {
    const Scene s = make_scene(sc);
    for (int64_t i = 0; i < n; ++i) hit_uv(s, hits[i], out2[2 * i], out2[2 * i + 1]);
}

void orc_hit_albedo(const orc_scene* sc, const orc_hit* hits, int64_t n, const orc_materials* mat,
                    int nthreads, float* out3) {
    const Scene s = make_scene(sc);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const V3 a = hit_albedo(s, *mat, hits[i]);
            out3[3 * i] = a.x;
            out3[3 * i + 1] = a.y;
            out3[3 * i + 2] = a.z;
        }
    });
}

void orc_shade(const orc_scene* sc, const orc_ray* rays, const orc_hit* hits, int64_t n,
               const uint8_t* shadow_lit, const orc_materials* mat,
               const float sun_dir[3], const float sun_color[3], const float sky_color[3],
               int32_t normal_mode, int nthreads, float* out4) {
    const Scene s = make_scene(sc);
    const V3 sd = ld3(sun_dir), sunc = ld3(sun_color), sky = ld3(sky_color);
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const orc_hit& h = hits[i];
            float* o = out4 + i * 4;
            if (!(rays[i].tmax > rays[i].tmin)) {
                o[0] = o[1] = o[2] = 0.0f;
                o[3] = 0.0f;
                continue;
            }
            if (!(h.t > 0.0f)) {  // sky (DiffuseTrace.glsl:490) and unoccluded AO (:494)
                o[0] = sky.x; o[1] = sky.y; o[2] = sky.z;
                o[3] = 1.0f;
                continue;
            }
            const V3 rd = ld3(rays[i].d);
            V3 N = hit_normal(s, h, normal_mode);
            if (dot(N, rd) > 0.0001f) N = neg(N);
            const V3 alb = hit_albedo(s, *mat, h);
            float em;
            std::memcpy(&em, &s.ents[h.entity].data[0], 4);
            const float lit = shadow_lit ? (shadow_lit[i] ? 1.0f : 0.0f) : 1.0f;
            // GetDirect, DiffuseTrace.glsl:368-372, plus Albedo*emissive (:491).
            const float ndl = clamp01(dot(N, neg(sd)));
            V3 direct = muls(muls(mul(alb, sunc), lit), ndl);
            V3 rad = add(direct, muls(alb, em));
            o[0] = rad.x; o[1] = rad.y; o[2] = rad.z;
            o[3] = std::pow(clamp01(h.t / 2.4f), 1.23f);  // DiffuseTrace.glsl:494
        }
    });
}

void orc_collide(const orc_scene* sc, const float* boxes, int64_t n, int32_t* out, int flags, int nthreads) {
    const Scene s = make_scene(sc);
    const bool ref = (flags & ORC_FLAG_REF_COMPAT) != 0;
    parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) collide_scene(s, boxes + i * 8, ref, out + i * 4);
    });
}

}  // extern "C"

// ---- Radiance probe volume: UpdateRadianceProbes.glsl, one frame ----------------------------

namespace {

// SphericalHarmonics.glsl: struct SH {L00, L11, L10, L1_1} and its first-order basis constants.
struct SH4 {
    V3 l00, l11, l10, l1_1;
};
constexpr float kY00 = 0.28209479177387814347f;
constexpr float kY11 = -0.48860251190291992159f;
constexpr float kY10 = 0.48860251190291992159f;
constexpr float kY1_1 = -0.48860251190291992159f;

inline V3 vdiv(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 vadds(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline V3 vmaxs(V3 a, float s) { return {gmax(a.x, s), gmax(a.y, s), gmax(a.z, s)}; }
inline V3 vmix(V3 x, V3 y, float a) { return {mixf(x.x, y.x, a), mixf(x.y, y.y, a), mixf(x.z, y.z, a)}; }
inline float bits_f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline uint32_t f_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

struct ProbeGrid {
    int gx, gy, gz;
    V3 res, size, origin, prev;
    int64_t count() const { return int64_t(gx) * gy * gz; }
    bool inside(int x, int y, int z) const { return x >= 0 && x < gx && y >= 0 && y < gy && z >= 0 && z < gz; }
    int64_t index(int x, int y, int z) const { return (int64_t(z) * gy + y) * gx + x; }
};
ProbeGrid probe_grid(const orc_probe_params& p) {
    ProbeGrid g;
    g.gx = p.grid[0];
    g.gy = p.grid[1];
    g.gz = p.grid[2];
    g.res = {float(g.gx), float(g.gy), float(g.gz)};
    g.size = ld3(p.size);
    g.origin = ld3(p.origin);
    g.prev = ld3(p.prev_origin);
    return g;
}

// Probe (texel) position about `base`: TexCoords = vec3(Pixel) / u_Resolution,
// Clip = TexCoords * 2 - 1, base + Clip * u_Size (:412-417; GetVisibility :178-180).
V3 probe_position(const ProbeGrid& g, V3 base, int x, int y, int z) {
    const V3 tc = vdiv(V3{float(x), float(y), float(z)}, g.res);
    const V3 clip = vadds(muls(tc, 2.0f), -1.0f);
    return add(base, mul(clip, g.size));
}

// LambertBRDF(vec3(hash2(), hash2().x)) normalised (:351-372): phi = 2 pi h.x, cos(theta) =
// 2 h.y - 1; sin(theta) as sqrt(1 - cos^2) and the radius u^(1/3) (which the normalisation
// removes) left out; h from dimensions 0 and 1 of the counter-based hash for the probe index.
V3 probe_direction(uint32_t seed, uint32_t id) {
    const float hx = u01(sample_key(seed, id, 0u)), hy = u01(sample_key(seed, id, 1u));
    float sp, cp;
    sincos_turns(hx, sp, cp);
    const float c = 2.0f * hy - 1.0f;
    const float st = std::sqrt(1.0f - c * c);
    return normalize(V3{st * cp, st * sp, c});
}

// The 8x8 map pixel of a direction: UnitVectorToOctahedron (Octahedral.glsl) scaled by 7 and
// truncated, Get1DIdx(ivec2, ivec2(8)) = x * 8 + y (:470-472).
int oct_pixel(V3 d) {
    const float s = dot(V3{std::fabs(d.x), std::fabs(d.y), std::fabs(d.z)}, V3{1.0f, 1.0f, 1.0f});
    float x = d.x / s, z = d.z / s;
    if (d.y < 0.0f) {
        const float ox = x, oz = z;
        x = (ox >= 0.0f ? 1.0f : -1.0f) * (1.0f - std::fabs(oz));
        z = (oz >= 0.0f ? 1.0f : -1.0f) * (1.0f - std::fabs(ox));
    }
    const float u = clamp01(0.5f * x + 0.5f), v = clamp01(0.5f * z + 0.5f);
    return int(u * 7.0f) * 8 + int(v * 7.0f);
}

// EncodeSH (SphericalHarmonics.glsl): each coefficient is 0 + Y * radiance * A.
SH4 encode_sh(V3 rad, V3 dir) {
    const float pi = 3.14159265359f, m = 2.0f;
    const float a0 = m * pi, a1 = ((2.0f * pi) / 3.0f) * m;
    const V3 z = {0.0f, 0.0f, 0.0f};
    SH4 r;
    r.l00 = add(z, muls(muls(rad, kY00), a0));
    r.l1_1 = add(z, muls(muls(rad, kY1_1 * dir.y), a1));
    r.l10 = add(z, muls(muls(rad, kY10 * dir.z), a1));
    r.l11 = add(z, muls(muls(rad, kY11 * dir.x), a1));
    return r;
}

// SampleSH(sh, direction): the four clamped lobes summed in the shader's order.
V3 sample_sh(const SH4& sh, V3 d) {
    V3 r = {0.0f, 0.0f, 0.0f};
    r = add(r, vmaxs(muls(sh.l00, kY00), 0.0f));
    r = add(r, vmaxs(muls(muls(sh.l1_1, kY1_1), d.y), 0.0f));
    r = add(r, vmaxs(muls(muls(sh.l10, kY10), d.z), 0.0f));
    r = add(r, vmaxs(muls(muls(sh.l11, kY11), d.x), 0.0f));
    return r;
}

// packSnorm2x16 of one component: round(clamp(c, -1, 1) * 32767), half to even, NaN as 0.
uint32_t snorm16(float c) {
    const float s = gmin(gmax(c, -1.0f), 1.0f) * 32767.0f;
    if (s != s) return 0u;
    return uint32_t(uint16_t(int16_t(std::nearbyint(s))));
}
uint32_t pack_snorm2(float a, float b) { return snorm16(a) | (snorm16(b) << 16); }
float unsnorm16(uint32_t h) { return gmin(gmax(float(int16_t(uint16_t(h & 0xFFFFu))) / 32767.0f, -1.0f), 1.0f); }

inline float max3abs(V3 x) { return gmax(gmax(std::fabs(x.x), std::fabs(x.y)), std::fabs(x.z)); }

// PackSH: coefficients divided by the largest magnitude (starting from -1000), six snorm pairs,
// the scale's bits, 0.
void pack_sh(SH4 sh, uint32_t* w) {
    float m = -1000.0f;
    m = gmax(m, max3abs(sh.l00));
    m = gmax(m, max3abs(sh.l11));
    m = gmax(m, max3abs(sh.l10));
    m = gmax(m, max3abs(sh.l1_1));
    const V3 a = {sh.l00.x / m, sh.l00.y / m, sh.l00.z / m}, b = {sh.l11.x / m, sh.l11.y / m, sh.l11.z / m};
    const V3 c = {sh.l10.x / m, sh.l10.y / m, sh.l10.z / m}, d = {sh.l1_1.x / m, sh.l1_1.y / m, sh.l1_1.z / m};
    w[0] = pack_snorm2(a.x, a.y);
    w[1] = pack_snorm2(a.z, b.x);
    w[2] = pack_snorm2(b.y, b.z);
    w[3] = pack_snorm2(c.x, c.y);
    w[4] = pack_snorm2(c.z, d.x);
    w[5] = pack_snorm2(d.y, d.z);
    w[6] = f_bits(m);
    w[7] = 0u;
}

// UnpackSH: the snorm pairs times the scale stored in B.z.
SH4 unpack_sh(const uint32_t* w) {
    const float k = bits_f(w[6]);
    float u[12];
    for (int i = 0; i < 6; ++i) {
        u[2 * i] = unsnorm16(w[i]) * k;
        u[2 * i + 1] = unsnorm16(w[i] >> 16) * k;
    }
    return SH4{{u[0], u[1], u[2]}, {u[3], u[4], u[5]}, {u[6], u[7], u[8]}, {u[9], u[10], u[11]}};
}

// The previous volume's texel (x, y, z): 8 words, zeros outside the volume.
void load_texel(const ProbeGrid& g, const uint32_t* vol, int x, int y, int z, uint32_t* w) {
    if (!g.inside(x, y, z)) {
        for (int k = 0; k < 8; ++k) w[k] = 0u;
        return;
    }
    std::memcpy(w, vol + 8 * g.index(x, y, z), 32);
}

// GetVisibility (:176-188): clamp(dot(N, direction to the probe), 0, 1)^2, pow(x, 2) taken as x * x.
float probe_visibility(const ProbeGrid& g, int x, int y, int z, V3 wp, V3 n) {
    const V3 pp = probe_position(g, g.prev, x, y, z);
    V3 v = sub(pp, wp);
    const float len = std::sqrt(dot(v, v));
    v = {v.x / len, v.y / len, v.z / len};
    const float w = clamp01(dot(n, v));
    return w * w;
}

// SampleProbes (:190-237) over the previous volume.
V3 sample_probes(const ProbeGrid& g, const uint32_t* vol, V3 wp, V3 n) {
    wp = add(wp, muls(n, 0.45f));
    V3 sp = vdiv(sub(wp, g.prev), g.size);
    sp = vadds(muls(sp, 0.5f), 0.5f);
    if (!(sp.x == clamp01(sp.x) && sp.y == clamp01(sp.y) && sp.z == clamp01(sp.z))) return {0.0f, 0.0f, 0.0f};
    const V3 vc = mul(sp, g.res);
    const V3 mn = {std::floor(vc.x), std::floor(vc.y), std::floor(vc.z)};
    const V3 mx = {std::ceil(vc.x), std::ceil(vc.y), std::ceil(vc.z)};
    const V3 ext = sub(mx, mn);
    const float inv = 1.0f / (ext.x * ext.y * ext.z);
    const float ax = mx.x - vc.x, ay = mx.y - vc.y, az = mx.z - vc.z;  // Max - p
    const float bx = vc.x - mn.x, by = vc.y - mn.y, bz = vc.z - mn.z;  // p - Min
    float w[8] = {ax * ay * az * inv, ax * by * az * inv, bx * by * az * inv, bx * ay * az * inv,
                  ax * ay * bz * inv, ax * by * bz * inv, bx * by * bz * inv, bx * ay * bz * inv};
    const int x0 = int(mn.x), y0 = int(mn.y), z0 = int(mn.z), x1 = int(mx.x), y1 = int(mx.y), z1 = int(mx.z);
    const int tx[8] = {x0, x0, x1, x1, x0, x0, x1, x1}, ty[8] = {y0, y1, y1, y0, y0, y1, y1, y0};
    const int tz[8] = {z0, z0, z0, z0, z1, z1, z1, z1};
    SH4 sh[8];
    float alpha = 0.0f;
    for (int i = 0; i < 8; ++i) {
        uint32_t t[8];
        load_texel(g, vol, tx[i], ty[i], tz[i], t);
        sh[i] = unpack_sh(t);
        const float vis = probe_visibility(g, tx[i], ty[i], tz[i], wp, n);
        alpha = alpha + w[i] * (1.0f - vis);
        w[i] = w[i] * vis;
    }
    const float ws = 1.0f - alpha;
    SH4 f = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
    for (int i = 0; i < 8; ++i) {
        const float k = w[i] / gmax(ws, 0.000001f);
        f.l00 = add(f.l00, muls(sh[i].l00, k));
        f.l1_1 = add(f.l1_1, muls(sh[i].l1_1, k));
        f.l10 = add(f.l10, muls(sh[i].l10, k));
        f.l11 = add(f.l11, muls(sh[i].l11, k));
    }
    return vmaxs(sample_sh(f, n), 0.0f);
}

// Reproject (:298-313): the previous volume's texel under the world position, or false.
bool reproject(const ProbeGrid& g, V3 wp, int& x, int& y, int& z) {
    V3 sp = vdiv(sub(wp, g.prev), g.size);
    sp = vadds(muls(sp, 0.5f), 0.5f);
    if (!(sp.x > 0.0f && sp.x < 1.0f && sp.y > 0.0f && sp.y < 1.0f && sp.z > 0.0f && sp.z < 1.0f)) return false;
    sp = vadds(mul(sp, g.res), 0.5f);
    x = int(sp.x);
    y = int(sp.y);
    z = int(sp.z);
    return true;
}

}  // namespace

extern "C" {

void orc_probe_raygen(const orc_probe_params* p, int nthreads, orc_ray* out) {
    const ProbeGrid g = probe_grid(*p);
    parallel_for(g.count(), nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const int x = int(i % g.gx), y = int((i / g.gx) % g.gy), z = int(i / (int64_t(g.gx) * g.gy));
            const V3 o = probe_position(g, g.origin, x, y, z);
            const V3 d = probe_direction(p->seed, uint32_t(i));
            out[i] = orc_ray{{o.x, o.y, o.z}, 0.0f, {d.x, d.y, d.z}, p->ray_tmax};
        }
    });
}

void orc_probe_direction(uint32_t seed, const uint32_t* ids, int64_t n, float* out3) {
    for (int64_t i = 0; i < n; ++i) {
        const V3 d = probe_direction(seed, ids[i]);
        out3[3 * i] = d.x;
        out3[3 * i + 1] = d.y;
        out3[3 * i + 2] = d.z;
    }
}

// UpdateRadianceProbes.glsl main (:408-520) after the trace: shading, the bounce from the previous
// volume, SH encoding, temporal blend and packing; probe_map updated in place.  raw_r11: the raw
// radiance as the reference's r11f_g11f_b10f images (:17-18) hold it.
void orc_probe_shade(const orc_scene* sc, const orc_probe_params* p, const orc_ray* rays, const orc_hit* hits,
                     const uint8_t* lit, const orc_materials* mat, const uint32_t* prev_sh, const float* prev_raw,
                     float* probe_map, uint32_t* out_sh, float* out_raw, int raw_r11, int nthreads) {
    const Scene s = make_scene(sc);
    const ProbeGrid g = probe_grid(*p);
    const V3 sun = ld3(p->sun_color), sky = ld3(p->sky_color), sdir = ld3(p->sun_dir);
    parallel_for(g.count(), nthreads, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const V3 o = ld3(rays[i].o), d = ld3(rays[i].d);
            const orc_hit& h = hits[i];
            const float t = h.t;
            V3 N = {-1.0f, -1.0f, -1.0f}, alb = {0.0f, 0.0f, 0.0f};
            float em = 0.0f;
            if (t > 0.0f) {
                N = hit_normal(s, h, p->normal_mode);
                alb = hit_albedo(s, *mat, h);
                std::memcpy(&em, &s.ents[h.entity].data[0], 4);
            }
            if (dot(N, d) > 0.0001f) N = neg(N);
            const V3 wp = add(o, muls(d, t));
            const float lsky = clamp01(dot(d, V3{0.0f, 1.0f, 0.0f}));
            V3 fr;
            if (t < 0.0f) {
                fr = muls(muls(sky, 2.2f), lsky);
            } else {
                const float shadow = lit ? (lit[i] ? 1.0f : 0.0f) : 1.0f;
                const float ndl = clamp01(dot(N, neg(sdir)));
                fr = add(vmaxs(muls(muls(mul(alb, sun), shadow), ndl), 0.0f), muls(muls(alb, em), 1.0f));
            }
            if (t > 0.0f) fr = add(fr, mul(muls(sample_probes(g, prev_sh, add(wp, muls(N, 0.001f)), N), 0.999f), alb));
            float* px = probe_map + 128 * i + 2 * oct_pixel(d);
            const float depth = t < 0.0f ? 256.0f : t, depth2 = depth * depth;
            SH4 sh = encode_sh(fr, d);
            int32_t frames = 0;
            int rx, ry, rz;
            if (reproject(g, o, rx, ry, rz)) {
                uint32_t w[8];
                load_texel(g, prev_sh, rx, ry, rz, w);
                frames = int32_t(w[7] + 1u);
                const float ta = p->temporal ? gmin(1.0f - 1.0f / float(frames), 0.98f) : 0.0f;
                const float m0 = px[0], m1 = px[1];
                px[0] = mixf(depth, m0, ta);
                px[1] = mixf(depth2, m1, ta);
                const SH4 ps = unpack_sh(w);
                sh.l00 = vmix(sh.l00, ps.l00, ta);
                sh.l11 = vmix(sh.l11, ps.l11, ta);
                sh.l10 = vmix(sh.l10, ps.l10, ta);
                sh.l1_1 = vmix(sh.l1_1, ps.l1_1, ta);
                const V3 pr = g.inside(rx, ry, rz) ? ld3(prev_raw + 4 * g.index(rx, ry, rz)) : V3{0.0f, 0.0f, 0.0f};
                fr = vmix(fr, pr, ta);
            } else {
                px[0] = depth;
                px[1] = depth2;
            }
            uint32_t* w = out_sh + 8 * i;
            pack_sh(sh, w);
            w[7] = uint32_t(frames);
            float* r = out_raw + 4 * i;
            if (raw_r11) fr = V3{small_ufloat(fr.x, 6), small_ufloat(fr.y, 6), small_ufloat(fr.z, 5)};
            r[0] = fr.x;
            r[1] = fr.y;
            r[2] = fr.z;
            r[3] = 0.0f;
        }
    });
}

}  // extern "C"

// ---- RT second-bounce loop accumulation (DiffuseTrace.glsl:499-535) -----------------------

extern "C" {

// Per GI slot: fr = the first hit's radiance (FinalRadiance), thr0 = its albedo (Throughput);
// per bounce b < n_bounces of slot i, in = 12 floats {t (< 0: miss), albedo rgb, emissive,
// GetData normal xyz, direction xyz, sun visibility}.  Bounced starts at 0; a hit adds
// (GetDirect + albedo x emissive) x Throughput (:524) and multiplies Throughput by the albedo
// (:530); a miss adds nothing under ref_miss (the shader's GetDirect of a zero albedo) or
// 1.1 x sky x Throughput otherwise, and ends the path.  out = FinalRadiance + Bounced (:535).
void orc_bounce_accumulate(const float* fr, const float* thr0, const float* in, int64_t n, int32_t n_bounces,
                           const float sun_dir[3], const float sun_color[3], const float sky[3], int ref_miss,
                           float* out3) {
    const V3 sd = ld3(sun_dir), sun = ld3(sun_color), sk = ld3(sky);
    for (int64_t i = 0; i < n; ++i) {
        V3 b = {0.0f, 0.0f, 0.0f}, t = ld3(thr0 + 3 * i);
        for (int32_t k = 0; k < n_bounces; ++k) {
            const float* x = in + (i * n_bounces + k) * 12;
            if (!(x[0] > 0.0f)) {
                if (!ref_miss) b = add(b, mul(muls(sk, 1.1f), t));
                break;
            }
            const V3 alb = ld3(x + 1), d = ld3(x + 8);
            V3 nrm = ld3(x + 5);
            if (dot(nrm, d) > 0.0001f) nrm = neg(nrm);
            const float ndl = clamp01(dot(nrm, neg(sd)));
            const V3 v = add(muls(muls(mul(alb, sun), x[11]), ndl), muls(alb, x[4]));
            b = add(b, mul(v, t));
            t = mul(t, alb);
        }
        const V3 f = add(ld3(fr + 3 * i), b);
        out3[3 * i] = f.x;
        out3[3 * i + 1] = f.y;
        out3[3 * i + 2] = f.z;
    }
}


// Brute force over every triangle of every entity (no box tests): the lexicographic minimum of
// (t, triangle, entity) over tmin < t < tmax with the strict triangle test of RayTriangle
// (TraverseBVHStack.glsl:87-105) on the entity-transformed ray, barycentrics as IntersectScene
// reports them (:351-360).  A BVH walk can only lose hits to its box tests, so where a walk and
// this disagree the brute force says which answer the triangle test supports.  occluded (nullable)
// receives whether any such triangle exists.  flags: ORC_FLAG_IGNORE_TRANSPARENT.
void orc_brute_closest(const orc_scene* sc, const orc_ray* rays, int64_t n, orc_hit* hits, uint8_t* occluded,
                       int flags, int nthreads) {
    const Scene s = make_scene(sc);
    // leaf triangle ranges per entity, collected from every node of the entity's range
    std::vector<std::vector<std::pair<int32_t, int32_t>>> leaves(s.n_ents);
    for (int i = 0; i < s.n_ents; ++i) {
        const orc_entity& e = s.ents[i];
        for (int64_t k = e.node_offset; k < (int64_t)e.node_offset + e.node_count && k < s.n_nodes; ++k) {
            if (s.layout == ORC_STACK) {
                const float* nd = s.nodes + k * 16;
                for (int side = 0; side < 2; ++side) {
                    const int32_t kind = f2i(nd[side * 8 + 3]);
                    if (kind != -1 && (kind & 15) > 0) leaves[i].push_back({kind >> 4, kind & 15});
                }
            } else {
                const int32_t kind = f2i(s.nodes[k * 8 + 3]);
                if (kind != -1 && (kind & 15) > 0) leaves[i].push_back({kind >> 4, kind & 15});
            }
        }
    }
    parallel_for(n, nthreads, [&](int64_t b0, int64_t e0) {
        for (int64_t r = b0; r < e0; ++r) {
            const orc_ray& ray = rays[r];
            orc_hit& h = hits[r];
            h.t = h.u = h.v = h.w = -1.0f;
            h.tri = h.mesh = h.entity = -1;
            h.iters = 0;
            if (occluded) occluded[r] = 0;
            if (!(ray.tmax > ray.tmin)) continue;
            const V3 o = ld3(ray.o), d = ld3(ray.d);
            float bt = ray.tmax;
            int32_t btri = -1, bent = -1, bmesh = -1;
            bool any = false;
            for (int i = 0; i < s.n_ents; ++i) {
                const orc_entity& e = s.ents[i];
                if ((flags & ORC_FLAG_IGNORE_TRANSPARENT) && ent_alpha(e) < 0.99f) continue;
                const V3 ro = xform(e.inverse, o, 1.0f), rd = xform(e.inverse, d, 0.0f);
                for (const auto& lf : leaves[i]) {
                    for (int32_t idx = lf.first; idx < lf.first + lf.second; ++idx) {
                        const int32_t* tr = s.tris + (int64_t)idx * 4;
                        float t, u, v;
                        ray_triangle(ro, rd, vpos(s, tr[0]), vpos(s, tr[1]), vpos(s, tr[2]), t, u, v);
                        if (!(t > ray.tmin) || !(t < ray.tmax)) continue;
                        any = true;
                        if (t < bt || (t == bt && (idx < btri || (idx == btri && i < bent)))) {
                            bt = t;
                            btri = idx;
                            bent = i;
                            bmesh = tr[3];
                        }
                    }
                }
            }
            if (occluded) occluded[r] = any ? 1 : 0;
            if (btri < 0) continue;
            const orc_entity& e = s.ents[bent];
            const V3 ro = xform(e.inverse, o, 1.0f), rd = xform(e.inverse, d, 0.0f);
            const int32_t* tr = s.tris + (int64_t)btri * 4;
            float u, v, w;
            barycentrics(add(ro, muls(rd, bt)), vpos(s, tr[0]), vpos(s, tr[1]), vpos(s, tr[2]), u, v, w);
            h.t = bt;
            h.u = u;
            h.v = v;
            h.w = w;
            h.tri = btri;
            h.mesh = bmesh;
            h.entity = bent;
        }
    });
}

}  // extern "C"
