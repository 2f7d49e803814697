// BVH8 traversal with 8-bit quantised child boxes (closest hit and any hit).
//
// Box test: per node and axis the kernel forms inv_s = 2^(e-127) * inv (exact: a power-of-two
// scale) and o = (p - ro) * inv, so a child's slab distances are fma(q, inv_s, o).  The near and
// far planes are chosen per axis from the sign of the direction, so each child costs six FMAs and
// two 3-way min/max.  The FMA form rounds; its error is bounded by a few ulps of the node's extent
// in t plus half a grid step (from folding the 2^23 bias of the byte-to-float trick into o), so o
// is widened by that much on each side, which keeps the test conservative: every child box the ray
// meets in exact arithmetic is entered.  Zero direction
// components use a +-1e30 reciprocal for the boxes (the triangle test still uses the exact ray).
//
// Leaf test: the strict RayTriangle arithmetic (TraverseBVHStack.glsl:87-105) on precomputed
// records {v0, e1, e2, n} whose edges and normal were computed with the same IEEE operations, so
// t is bit-identical to the strict kernels; with the lower-index tie rule and inclusive box
// pruning (entry <= best t) the closest hit is the one the strict BVH2 traversal reports.
#pragma once
#include <cuda_runtime.h>

#include "rq_strict.cuh"

namespace rq {
namespace bvh8 {

using strict::f3;

constexpr int kStack = 48;         // group stack entries per lane (the default depth)
// Group-stack depths the launch variants are compiled for (the autotuner picks among them; a
// walk that would push beyond its depth sets kStatusStackOverflow, and the tuner rejects that
// variant).  A shallower stack is a smaller local-memory frame per lane.
constexpr int kStackDepths[3] = {48, 32, 24};
constexpr int kMaxVisits = 1 << 16;  // node visits per ray and entity before RQ_EBUDGET

enum : unsigned { kStatusStackOverflow = 1u, kStatusBudget = 2u };

__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
// Byte k of w as the float 2^23 + byte (one byte permute, no int-to-float conversion).
__device__ __forceinline__ float ubyte_biased(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | static_cast<unsigned>(k)));
}

struct Ray8 {
    f3 ro, rd;           // object-space ray (strict transform)
    f3 binv;             // reciprocal for box tests (zero components clamped)
    uint32_t oct;        // octant: bit a set when rd.a < 0
};

__device__ __forceinline__ Ray8 make_ray(f3 ro, f3 rd) {
    Ray8 r;
    r.ro = ro;
    r.rd = rd;
    auto safe = [](float x) { return fabsf(x) > 1e-30f ? x : copysignf(1e-30f, x); };
    r.binv = {__frcp_rn(safe(rd.x)), __frcp_rn(safe(rd.y)), __frcp_rn(safe(rd.z))};
    r.oct = (rd.x < 0.0f ? 1u : 0u) | (rd.y < 0.0f ? 2u : 0u) | (rd.z < 0.0f ? 4u : 0u);
    return r;
}

// Strict RayTriangle on a precomputed record.
__device__ __forceinline__ float ray_triangle_rec(const f3 ro, const f3 rd, const float4 a,
                                                  const float4 b, const float4 c, const float4 d) {
    const f3 v0 = strict::xyz(a), e1 = strict::xyz(b), e2 = strict::xyz(c), n = strict::xyz(d);
    const f3 rov0 = strict::sub(ro, v0);
    const f3 q = strict::cross(rov0, rd);
    const float dd = __fdiv_rn(1.0f, strict::dot(rd, n));
    const float u = __fmul_rn(dd, strict::dot(strict::neg(q), e2));
    const float v = __fmul_rn(dd, strict::dot(q, e1));
    float t = __fmul_rn(dd, strict::dot(strict::neg(n), rov0));
    if (u < 0.0f || v < 0.0f || __fadd_rn(u, v) > 1.0f) t = -1.0f;
    return t;
}

struct Hit8 {
    float tmax;     // running best t (closest) or the ray's tmax (any)
    float closest;  // -1 until a hit
    int32_t tri;    // reference triangle index of the best hit (tie seed on entry)
    int32_t mesh;
};

// Walk state of one ray through one BVH8: the node to visit next, the current group
// (child_base | (hit bits, octant order) << 32 | imask << 40), the group stack depth and the visit
// count.  The stack itself lives outside the struct so that the scalars stay in registers.
struct Walk {
    uint64_t group;
    int32_t node, sp, visits;
};

__device__ __forceinline__ Walk walk_begin(int32_t root) { return Walk{0ull, root, 0, 0}; }

// Visits node w.node (box tests of its eight children, then its leaf triangles) and selects the
// node after it.  Returns false when the walk has ended (stack empty, any-hit found, or an
// overflow/budget status bit set).  `stack` holds kDepth entries.
template <bool kAny, bool kTieLower, int kDepth = kStack>
__device__ __forceinline__ bool step(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                     const Ray8& r, float tmin, Hit8& h, Walk& w, uint64_t* stack,
                                     int32_t& tests, unsigned& status) {
    const float kUlp8 = 8.0f * 5.96046448e-08f;
    uint64_t group = w.group;
    int sp = w.sp;
    const int32_t node = w.node;
    {
        {
            if (++w.visits > kMaxVisits) {
                status |= kStatusBudget;
                return false;
            }
            const uint4* nd = nodes + 5 * static_cast<int64_t>(node);
            const uint4 w0 = __ldg(nd), w1 = __ldg(nd + 1), w2 = __ldg(nd + 2), w3 = __ldg(nd + 3),
                        w4 = __ldg(nd + 4);
            const f3 p = {__uint_as_float(w0.x), __uint_as_float(w0.y), __uint_as_float(w0.z)};
            const uint32_t imask = w0.w >> 24;
            const float sx = __uint_as_float((w0.w & 0xFFu) << 23);
            const float sy = __uint_as_float(((w0.w >> 8) & 0xFFu) << 23);
            const float sz = __uint_as_float(((w0.w >> 16) & 0xFFu) << 23);
            const float isx = sx * r.binv.x, isy = sy * r.binv.y, isz = sz * r.binv.z;
            const float ox = (p.x - r.ro.x) * r.binv.x;
            const float oy = (p.y - r.ro.y) * r.binv.y;
            const float oz = (p.z - r.ro.z) * r.binv.z;
            // Quantised coordinates arrive as 2^23 + q, so the origin term absorbs -2^23 * inv_s;
            // rounding that sum costs at most half a grid step, which the padding also covers.
            const float bx = ox - 8388608.0f * isx, by = oy - 8388608.0f * isy;
            const float bz = oz - 8388608.0f * isz;
            const float px = 0.5f * fabsf(isx) + kUlp8 * (255.0f * fabsf(isx) + fabsf(ox));
            const float py = 0.5f * fabsf(isy) + kUlp8 * (255.0f * fabsf(isy) + fabsf(oy));
            const float pz = 0.5f * fabsf(isz) + kUlp8 * (255.0f * fabsf(isz) + fabsf(oz));
            // near plane = lo for a positive direction, hi for a negative one
            const uint32_t loxy0 = w2.x, loxy1 = w2.y, loy0 = w2.z, loy1 = w2.w;
            const uint32_t loz0 = w3.x, loz1 = w3.y, hix0 = w3.z, hix1 = w3.w;
            const uint32_t hiy0 = w4.x, hiy1 = w4.y, hiz0 = w4.z, hiz1 = w4.w;
            const bool nx = r.oct & 1u, ny = r.oct & 2u, nz = r.oct & 4u;
            const uint32_t nX0 = nx ? hix0 : loxy0, nX1 = nx ? hix1 : loxy1;
            const uint32_t fX0 = nx ? loxy0 : hix0, fX1 = nx ? loxy1 : hix1;
            const uint32_t nY0 = ny ? hiy0 : loy0, nY1 = ny ? hiy1 : loy1;
            const uint32_t fY0 = ny ? loy0 : hiy0, fY1 = ny ? loy1 : hiy1;
            const uint32_t nZ0 = nz ? hiz0 : loz0, nZ1 = nz ? hiz1 : loz1;
            const uint32_t fZ0 = nz ? loz0 : hiz0, fZ1 = nz ? loz1 : hiz1;
            const float onx = bx - px, ofx = bx + px, ony = by - py, ofy = by + py;
            const float onz = bz - pz, ofz = bz + pz;
            const uint32_t meta0 = w1.z, meta1 = w1.w;
            uint32_t hitmask = 0;  // bit s: child slot s entered
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const int k = s & 3;
                const uint32_t a = s < 4 ? nX0 : nX1, b = s < 4 ? fX0 : fX1;
                const uint32_t c = s < 4 ? nY0 : nY1, d = s < 4 ? fY0 : fY1;
                const uint32_t e = s < 4 ? nZ0 : nZ1, f = s < 4 ? fZ0 : fZ1;
                const float tnx = fmaf(ubyte_biased(a, k), isx, onx);
                const float tfx = fmaf(ubyte_biased(b, k), isx, ofx);
                const float tny = fmaf(ubyte_biased(c, k), isy, ony);
                const float tfy = fmaf(ubyte_biased(d, k), isy, ofy);
                const float tnz = fmaf(ubyte_biased(e, k), isz, onz);
                const float tfz = fmaf(ubyte_biased(f, k), isz, ofz);
                const float tn = fmaxf(max3f(tnx, tny, tnz), tmin);
                const float tf = fminf(min3f(tfx, tfy, tfz), h.tmax);
                hitmask |= (tn <= tf ? 1u : 0u) << s;
            }
            // internal children in octant order: bit j of hits_oct = bit (j ^ oct) of the mask
            uint32_t hits_oct = hitmask & imask;
            {
                const uint32_t s1 = ((hits_oct & 0x55u) << 1) | ((hits_oct >> 1) & 0x55u);
                hits_oct = (r.oct & 1u) ? s1 : hits_oct;
                const uint32_t s2 = ((hits_oct & 0x33u) << 2) | ((hits_oct >> 2) & 0x33u);
                hits_oct = (r.oct & 2u) ? s2 : hits_oct;
                const uint32_t s4 = ((hits_oct & 0x0Fu) << 4) | ((hits_oct >> 4) & 0x0Fu);
                hits_oct = (r.oct & 4u) ? s4 : hits_oct;
            }
            uint32_t tmask = 0;  // triangles of the leaf children entered
            uint32_t lh = hitmask & ~imask;
            while (lh) {
                const int s = __ffs(lh) - 1;
                lh &= lh - 1;
                const uint32_t m = ((s < 4 ? meta0 : meta1) >> (8 * (s & 3))) & 0xFFu;
                if (m) tmask |= ((1u << (m >> 5)) - 1u) << (m & 31u);
            }
            // prefetch the node visited next while this node's triangles are tested
            if (tmask) {
                uint32_t gh = hits_oct ? hits_oct : static_cast<uint32_t>(group >> 32) & 0xFFu;
                if (gh) {
                    const uint64_t grp = hits_oct ? (static_cast<uint64_t>(w1.x) | (static_cast<uint64_t>(imask) << 40))
                                                  : group;
                    const uint32_t slot = static_cast<uint32_t>(__ffs(gh) - 1) ^ r.oct;
                    const uint32_t gim = static_cast<uint32_t>(grp >> 40) & 0xFFu;
                    const uint32_t nxt = static_cast<uint32_t>(grp) + __popc(gim & ((1u << slot) - 1u));
                    const char* pa = reinterpret_cast<const char*>(nodes + 5 * static_cast<int64_t>(nxt));
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(pa));
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(pa + 79));
                }
            }
            // leaf triangles of this node
            const int32_t tri_base = static_cast<int32_t>(w1.y);
            while (tmask) {
                const int i = __ffs(tmask) - 1;
                tmask &= tmask - 1;
                const float4* tr = tris + 4 * static_cast<int64_t>(tri_base + i);
                const float4 A = __ldg(tr), B = __ldg(tr + 1), C = __ldg(tr + 2), D = __ldg(tr + 3);
                ++tests;
                const float t = ray_triangle_rec(r.ro, r.rd, A, B, C, D);
                if (kAny) {
                    if (t > tmin && t < h.tmax) {  // first hit ends the walk
                        h.closest = t;
                        tmask = 0;
                        hits_oct = 0;
                        group = 0;
                        sp = 0;
                    }
                } else {
                    const int32_t idx = __float_as_int(A.w);
                    if (t > tmin && (t < h.tmax || (kTieLower && t == h.tmax && idx < h.tri))) {
                        h.tmax = t;
                        h.closest = t;
                        h.tri = idx;
                        h.mesh = __float_as_int(B.w);
                    }
                }
            }
            if (hits_oct) {
                if (static_cast<uint32_t>(group >> 32) & 0xFFu) {
                    if (sp >= kDepth) {
                        status |= kStatusStackOverflow;
                        return false;
                    }
                    stack[sp++] = group;
                }
                group = static_cast<uint64_t>(w1.x) | (static_cast<uint64_t>(hits_oct) << 32) |
                        (static_cast<uint64_t>(imask) << 40);
            }
        }
    }
    // next node: lowest remaining bit of the current group, else pop
    uint32_t gh = static_cast<uint32_t>(group >> 32) & 0xFFu;
    if (!gh) {
        if (sp == 0) return false;
        group = stack[--sp];
        gh = static_cast<uint32_t>(group >> 32) & 0xFFu;
    }
    const int j = __ffs(gh) - 1;
    gh &= gh - 1;
    const uint32_t slot = static_cast<uint32_t>(j) ^ r.oct;
    const uint32_t gim = static_cast<uint32_t>(group >> 40) & 0xFFu;
    w.node = static_cast<int32_t>(static_cast<uint32_t>(group) + __popc(gim & ((1u << slot) - 1u)));
    w.group = (group & ~(0xFFull << 32)) | (static_cast<uint64_t>(gh) << 32);
    w.sp = sp;
    return true;
}

// Visits the BVH8 rooted at `root`.  Returns the node-visit count; sets *status bits on overflow.
template <bool kAny, bool kTieLower, int kDepth = kStack>
__device__ int32_t traverse(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                            int32_t root, const Ray8& r, float tmin, Hit8& h, int32_t& tests,
                            unsigned& status) {
    uint64_t stack[kDepth];
    Walk w = walk_begin(root);
    while (step<kAny, kTieLower, kDepth>(nodes, tris, r, tmin, h, w, stack, tests, status)) {
    }
    return w.visits;
}

}  // namespace bvh8
}  // namespace rq
