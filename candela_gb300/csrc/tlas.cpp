// Top-level BVH over entities: world boxes with a rounding margin, a range-split SAH tree in
// pre-order with skip links (leaves in ascending entity order), prefix counts for the skipped
// entities' iterations.
#include "tlas.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace rq {
namespace {

constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr int kSahDepth = 24;  // deeper ranges split at the midpoint (depth <= 24 + log2 n)

struct Box {
    float lo[3], hi[3];
};

float round_down(double x) {
    float f = static_cast<float>(x);
    if (static_cast<double>(f) > x) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
    return f;
}
float round_up(double x) {
    float f = static_cast<float>(x);
    if (static_cast<double>(f) < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

double norm_inf(const double m[3][3]) {
    double r = 0.0;
    for (int i = 0; i < 3; ++i) r = std::max(r, std::fabs(m[i][0]) + std::fabs(m[i][1]) + std::fabs(m[i][2]));
    return r;
}

bool invert3(const double m[3][3], double a[3][3]) {
    const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    const double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
    const double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    if (!std::isfinite(det) || det == 0.0) return false;
    const double id = 1.0 / det;
    a[0][0] = c00 * id;
    a[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
    a[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
    a[1][0] = c01 * id;
    a[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    a[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
    a[2][0] = c02 * id;
    a[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
    a[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (!std::isfinite(a[i][j])) return false;
    return true;
}

// World box of one entity; false when it must never be skipped.  The object-space ray is
// L * o + c (the entity's inverse matrix); the world box is the image of the object box under
// the exact inverse of that affine map, widened by kTlasMargin * (cond * |box| + |L^-1| *
// (|c| + |object box|)).  Together with the per-ray widening kTlasMargin * cond_max * |o| this
// covers the rounding of the transformed ray (a few ulps of |L||o| + |c| in the origin, of
// t|L||d| along the ray) and of the object-space slab test, about 2^-20 of those magnitudes.
bool world_box(const TlasEntity& e, Box& out, double& cond) {
    if (!e.cullable) return false;
    double L[3][3], c[3];
    for (int r = 0; r < 3; ++r) {
        for (int k = 0; k < 3; ++k) L[r][k] = e.inverse[k * 4 + r];
        c[r] = e.inverse[12 + r];
    }
    for (int r = 0; r < 3; ++r) {
        if (!std::isfinite(c[r])) return false;
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(L[r][k])) return false;
        if (!(e.lo[r] <= e.hi[r]) || !std::isfinite(e.lo[r]) || !std::isfinite(e.hi[r])) return false;
    }
    double A[3][3];
    if (!invert3(L, A)) return false;
    const double nl = norm_inf(L), na = norm_inf(A);
    cond = nl * na;
    if (!std::isfinite(cond) || cond > 1e6) return false;
    double lo[3] = {kInf, kInf, kInf}, hi[3] = {-kInf, -kInf, -kInf};
    for (int k = 0; k < 8; ++k) {
        const double p[3] = {(k & 1) ? e.hi[0] : e.lo[0], (k & 2) ? e.hi[1] : e.lo[1], (k & 4) ? e.hi[2] : e.lo[2]};
        const double q[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
        for (int r = 0; r < 3; ++r) {
            const double w = A[r][0] * q[0] + A[r][1] * q[1] + A[r][2] * q[2];
            lo[r] = std::min(lo[r], w);
            hi[r] = std::max(hi[r], w);
        }
    }
    double pmax = 0.0, bmax = 0.0, cmax = 0.0;
    for (int r = 0; r < 3; ++r) {
        pmax = std::max({pmax, std::fabs(lo[r]), std::fabs(hi[r])});
        bmax = std::max({bmax, std::fabs(e.lo[r]), std::fabs(e.hi[r])});
        cmax = std::max(cmax, std::fabs(c[r]));
    }
    const double m = kTlasMargin * (cond * pmax + na * (cmax + bmax));
    for (int r = 0; r < 3; ++r) {
        out.lo[r] = round_down(lo[r] - m);
        out.hi[r] = round_up(hi[r] + m);
        if (!std::isfinite(out.lo[r]) || !std::isfinite(out.hi[r])) return false;
    }
    return true;
}

// SAH weight of a box: half surface area, with infinite extents clamped so that costs stay
// comparable.
double half_area(const Box& b) {
    double d[3];
    for (int r = 0; r < 3; ++r) d[r] = std::min(static_cast<double>(b.hi[r]) - b.lo[r], 1e30);
    return d[0] * d[1] + d[1] * d[2] + d[2] * d[0];
}

void grow(Box& a, const Box& b) {
    for (int r = 0; r < 3; ++r) {
        a.lo[r] = std::min(a.lo[r], b.lo[r]);
        a.hi[r] = std::max(a.hi[r], b.hi[r]);
    }
}

Box empty_box() {
    const float inf = std::numeric_limits<float>::infinity();
    return Box{{inf, inf, inf}, {-inf, -inf, -inf}};
}

struct Builder {
    const std::vector<Box>& boxes;
    std::vector<float>& nodes;
    std::vector<Box> pre, suf;

    void put(int32_t idx, const Box& b, int32_t ent, int32_t skip) {
        float* n = nodes.data() + 8 * static_cast<size_t>(idx);
        n[0] = b.lo[0];
        n[1] = b.lo[1];
        n[2] = b.lo[2];
        std::memcpy(&n[3], &ent, 4);
        n[4] = b.hi[0];
        n[5] = b.hi[1];
        n[6] = b.hi[2];
        std::memcpy(&n[7], &skip, 4);
    }

    // Range split [lo, hi): the first position with the smallest SAH cost, or the midpoint.
    int32_t split(int32_t lo, int32_t hi, int depth) {
        const int32_t n = hi - lo;
        if (depth >= kSahDepth) return lo + n / 2;
        pre.resize(n);
        suf.resize(n);
        Box acc = empty_box();
        for (int32_t i = 0; i < n; ++i) {
            grow(acc, boxes[lo + i]);
            pre[i] = acc;
        }
        acc = empty_box();
        for (int32_t i = n - 1; i >= 0; --i) {
            grow(acc, boxes[lo + i]);
            suf[i] = acc;
        }
        double best = kInf;
        int32_t k = lo + n / 2;
        for (int32_t i = 1; i < n; ++i) {
            const double cost = half_area(pre[i - 1]) * i + half_area(suf[i]) * (n - i);
            if (cost < best) {
                best = cost;
                k = lo + i;
            }
        }
        return k;
    }

    // Emits the subtree of [lo, hi) in pre-order; returns its box.
    Box build(int32_t lo, int32_t hi, int depth) {
        const int32_t idx = static_cast<int32_t>(nodes.size() / 8);
        nodes.resize(nodes.size() + 8);
        if (hi - lo == 1) {
            put(idx, boxes[lo], lo, idx + 1);
            return boxes[lo];
        }
        const int32_t k = split(lo, hi, depth);
        Box b = build(lo, k, depth + 1);
        grow(b, build(k, hi, depth + 1));
        put(idx, b, -1, static_cast<int32_t>(nodes.size() / 8));
        return b;
    }
};

}  // namespace

bool build_tlas(const std::vector<TlasEntity>& ents, TlasOut& out, std::string& why) {
    out = TlasOut{};
    const int32_t n = static_cast<int32_t>(ents.size());
    if (n <= 0) {
        why = "no entities";
        return false;
    }
    std::vector<Box> boxes(n);
    double cond_max = 1.0;
    const float inf = std::numeric_limits<float>::infinity();
    for (int32_t i = 0; i < n; ++i) {
        double cond = 1.0;
        if (world_box(ents[i], boxes[i], cond)) {
            cond_max = std::max(cond_max, cond);
            ++out.n_cullable;
        } else {
            boxes[i] = Box{{-inf, -inf, -inf}, {inf, inf, inf}};
        }
    }
    out.ray_margin = round_up(kTlasMargin * cond_max);
    out.nodes.reserve(static_cast<size_t>(2 * n) * 8);
    Builder b{boxes, out.nodes, {}, {}};
    b.build(0, n, 0);
    out.n_nodes = static_cast<int32_t>(out.nodes.size() / 8);
    for (int32_t i = 0; i < out.n_nodes; ++i) {  // the node after the last subtree ends the walk
        int32_t skip;
        std::memcpy(&skip, &out.nodes[8 * static_cast<size_t>(i) + 7], 4);
        if (skip >= out.n_nodes) {
            skip = -1;
            std::memcpy(&out.nodes[8 * static_cast<size_t>(i) + 7], &skip, 4);
        }
    }
    out.prefix.assign(4 * static_cast<size_t>(n + 1), 0);
    for (int32_t i = 0; i < n; ++i) {
        const int32_t* p = &out.prefix[4 * static_cast<size_t>(i)];
        int32_t* q = &out.prefix[4 * static_cast<size_t>(i + 1)];
        q[0] = p[0] + (ents[i].opaque ? 1 : 0);
        q[1] = p[1] + (ents[i].b8 ? 1 : 0);
        q[2] = p[2] + (ents[i].b8 && ents[i].opaque ? 1 : 0);
        q[3] = 0;
    }
    return true;
}

}  // namespace rq
