// Refit of the BVH8 with quantised child boxes after the vertex positions change
// (rq_scene_update_positions), with its topology kept: the leaf triangle records are recomputed
// from the new positions with the strict arithmetic of the build ({v0, e1, e2, n}), then the nodes
// are refitted level by level from the deepest up.  Per node: each child's FP32 box (a leaf child:
// the min / max over its triangles' vertices; an internal child: that node's box, written when its
// level was refitted), the node box, a power-of-two grid step per axis and the child boxes rounded
// outward onto it, as the host build does (bvh8.cpp), so every decoded child box contains the
// triangles beneath it and no hit can be lost.  The host build checks the outward rounding in
// double precision; here it is checked exactly in binary32 with an error-free sum (Knuth's
// TwoSum: p + a = s + err exactly), which keeps FP64 off this path.
#include <cuda_runtime.h>

#include "bvh8.h"
#include "rq_objects.h"
#include "rq_strict.cuh"

namespace rq {
namespace {

using strict::f3;

// p + a <= x in real arithmetic (a = q * step is exact: q < 256 times a power of two).
__device__ __forceinline__ bool sum_le(float p, float a, float x) {
    const float s = __fadd_rn(p, a);
    const float bp = __fsub_rn(s, a), ap = __fsub_rn(s, bp);
    const float err = __fadd_rn(__fsub_rn(p, bp), __fsub_rn(a, ap));
    return s < x || (s == x && err <= 0.0f);
}
// p + a >= x in real arithmetic.
__device__ __forceinline__ bool sum_ge(float p, float a, float x) {
    const float s = __fadd_rn(p, a);
    const float bp = __fsub_rn(s, a), ap = __fsub_rn(s, bp);
    const float err = __fadd_rn(__fsub_rn(p, bp), __fsub_rn(a, ap));
    return s > x || (s == x && err >= 0.0f);
}

__device__ __forceinline__ f3 vert(const float4* verts, int32_t v) {
    return strict::xyz(__ldg(verts + 2 * static_cast<int64_t>(v)));
}

// Triangle records {v0, tri}, {e1, mesh}, {e2, 0}, {n, 0} from the current positions.
__global__ void k_b8_records(const int4* __restrict__ tris, const float4* __restrict__ verts,
                             float4* __restrict__ rec, int64_t n) {
    const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float4 A = rec[4 * r], B = rec[4 * r + 1];
    const int4 tr = __ldg(tris + __float_as_int(A.w));
    const f3 v0 = vert(verts, tr.x), v1 = vert(verts, tr.y), v2 = vert(verts, tr.z);
    const f3 e1 = strict::sub(v1, v0), e2 = strict::sub(v2, v0);
    const f3 nn = strict::cross(e1, e2);
    rec[4 * r] = make_float4(v0.x, v0.y, v0.z, A.w);
    rec[4 * r + 1] = make_float4(e1.x, e1.y, e1.z, B.w);
    rec[4 * r + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
    rec[4 * r + 3] = make_float4(nn.x, nn.y, nn.z, 0.0f);
}

// One level of nodes: child boxes, node box, grid and outward-rounded quantised boxes.
__global__ void k_b8_refit_level(uint32_t* __restrict__ nodes, const float4* __restrict__ rec,
                                 const int4* __restrict__ tris, const float4* __restrict__ verts,
                                 float* __restrict__ box, const int32_t* __restrict__ order, int64_t count) {
    const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int32_t me = order[k];
    uint32_t* nd = nodes + static_cast<int64_t>(me) * kBvh8NodeWords;
    const uint32_t imask = nd[3] >> 24;
    const uint32_t child_base = nd[4], tri_base = nd[5];
    uint8_t meta[8];
    for (int s = 0; s < 8; ++s) meta[s] = static_cast<uint8_t>((nd[6 + s / 4] >> (8 * (s % 4))) & 0xFFu);
    float clo[8][3], chi[8][3];
    bool used[8];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int s = 0; s < 8; ++s) {
        used[s] = false;
        for (int a = 0; a < 3; ++a) {
            clo[s][a] = INFINITY;
            chi[s][a] = -INFINITY;
        }
        if (imask & (1u << s)) {
            const int32_t c = static_cast<int32_t>(child_base + __popc(imask & ((1u << s) - 1u)));
            for (int a = 0; a < 3; ++a) {
                clo[s][a] = box[6 * static_cast<int64_t>(c) + a];
                chi[s][a] = box[6 * static_cast<int64_t>(c) + 3 + a];
            }
            used[s] = true;
        } else if (meta[s]) {
            const int cnt = meta[s] >> 5, off = meta[s] & 31;
            for (int i = 0; i < cnt; ++i) {
                const float4 A = __ldg(rec + 4 * (static_cast<int64_t>(tri_base) + off + i));
                const int4 tr = __ldg(tris + __float_as_int(A.w));
                const f3 v[3] = {vert(verts, tr.x), vert(verts, tr.y), vert(verts, tr.z)};
                for (int j = 0; j < 3; ++j) {
                    clo[s][0] = fminf(clo[s][0], v[j].x);
                    clo[s][1] = fminf(clo[s][1], v[j].y);
                    clo[s][2] = fminf(clo[s][2], v[j].z);
                    chi[s][0] = fmaxf(chi[s][0], v[j].x);
                    chi[s][1] = fmaxf(chi[s][1], v[j].y);
                    chi[s][2] = fmaxf(chi[s][2], v[j].z);
                }
            }
            used[s] = true;
        }
        if (used[s])
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], clo[s][a]);
                hi[a] = fmaxf(hi[a], chi[s][a]);
            }
    }
    for (int a = 0; a < 3; ++a) {
        box[6 * static_cast<int64_t>(me) + a] = lo[a];
        box[6 * static_cast<int64_t>(me) + 3 + a] = hi[a];
    }
    uint32_t ebyte[3];
    float step[3];
    bool coarse[3];
    for (int a = 0; a < 3; ++a) {
        // the smallest power-of-two step whose 255 steps from lo reach hi (frexp start, then up)
        const float ext = __fsub_rn(hi[a], lo[a]);
        int e = -126;
        if (ext > 0.0f) {
            int x;
            frexpf(__fdiv_rn(ext, 255.0f), &x);
            e = max(x - 1, -126);
        }
        while (e < 127 && !sum_ge(lo[a], __fmul_rn(255.0f, ldexpf(1.0f, e)), hi[a])) ++e;
        ebyte[a] = static_cast<uint32_t>(e + 127);
        step[a] = ldexpf(1.0f, e);
        coarse[a] = __fdiv_rn(fabsf(lo[a]), step[a]) > 1048576.0f;
        nd[a] = __float_as_uint(lo[a]);
    }
    uint8_t qb[48];
    for (int s = 0; s < 8; ++s)
        for (int a = 0; a < 3; ++a) {
            if (!used[s]) {
                qb[a * 8 + s] = 255;
                qb[24 + a * 8 + s] = 0;
                continue;
            }
            const float p = lo[a];
            float ql = floorf(__fdiv_rn(__fsub_rn(clo[s][a], p), step[a]));
            float qh = ceilf(__fdiv_rn(__fsub_rn(chi[s][a], p), step[a]));
            ql = fminf(fmaxf(ql, 0.0f), 255.0f);
            qh = fminf(fmaxf(qh, 0.0f), 255.0f);
            while (ql > 0.0f && !sum_le(p, __fmul_rn(ql, step[a]), clo[s][a])) ql -= 1.0f;
            while (qh < 255.0f && !sum_ge(p, __fmul_rn(qh, step[a]), chi[s][a])) qh += 1.0f;
            if (coarse[a]) {
                ql = fmaxf(ql - 1.0f, 0.0f);
                qh = fminf(qh + 1.0f, 255.0f);
            }
            qb[a * 8 + s] = static_cast<uint8_t>(ql);
            qb[24 + a * 8 + s] = static_cast<uint8_t>(qh);
        }
    nd[3] = ebyte[0] | (ebyte[1] << 8) | (ebyte[2] << 16) | (imask << 24);
    for (int w = 0; w < 12; ++w)
        nd[8 + w] = static_cast<uint32_t>(qb[4 * w]) | (static_cast<uint32_t>(qb[4 * w + 1]) << 8) |
                    (static_cast<uint32_t>(qb[4 * w + 2]) << 16) | (static_cast<uint32_t>(qb[4 * w + 3]) << 24);
}

inline unsigned grid_of(int64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace

rq_status refit_bvh8(rq_scene* sc, cudaStream_t st) {
    rq_ctx* ctx = sc->ctx;
    if (!sc->bvh8 || !sc->d_b8_order) return RQ_OK;
    k_b8_records<<<grid_of(sc->b8_tris, 256), 256, 0, st>>>(sc->d_tris, sc->d_verts, sc->d_b8tris, sc->b8_tris);
    RQ_CUDA(ctx, cudaGetLastError());
    for (size_t L = sc->b8_level_off.size() - 1; L-- > 0;) {  // deepest level first
        const int64_t b = sc->b8_level_off[L], e = sc->b8_level_off[L + 1];
        if (e > b)
            k_b8_refit_level<<<grid_of(e - b, 128), 128, 0, st>>>(
                reinterpret_cast<uint32_t*>(sc->d_b8nodes), sc->d_b8tris, sc->d_tris, sc->d_verts, sc->d_b8box,
                sc->d_b8_order + b, e - b);
        RQ_CUDA(ctx, cudaGetLastError());
    }
    sc->b8_bounds_stale = true;
    return RQ_OK;
}

}  // namespace rq
