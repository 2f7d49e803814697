// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// A sequential CPU restatement of the reference SAH BVH constructor (swr06/Candela,
// Source/Core/BVH/BVHConstructor.cpp), for where the reference tree is not mounted (the GPU hosts):
// the CPU reference arm of the benchmark builds its BVHs with it, so that nothing of the product is
// loaded there, and tests pin it against the reference constructor compiled here and against the
// committed hashes of that constructor's output (tests/golden/builder.json).  The product's own
// builder (candela_gb300/csrc/bvh_build.cpp) is a separate, task-parallel design.
//
// Followed step by step, in the reference's order and float arithmetic (no contraction):
//   ConstructTree (:385-627): per-triangle bounds and centroids, a LIFO stack of nodes (the right
//     child is pushed last, so processed first), leaves when len <= MAX_TRIANGLES_PER_LEAF or len <= 1
//     (their triangle references appended in stack order, start = position + triangle offset);
//   SearchSAHPlaneBinned (:276-363): 64 bins per axis, flat axes skipped, bin = min(63, (int)((c -
//     min) * (64 / extent))), prefix / suffix boxes and counts, cost nL * areaL + nR * areaR, the
//     first strictly smaller cost wins, border = min + step * (i + 1) with step = extent / 64;
//   the Lomuto partition by centroid < border (:532-550) and the midpoint fallback (:553-556);
//   child bounds from the triangle bounds (:574-593); the stackless child swap drawn from
//     uniform_int_distribution(1, 4) over mt19937 (:389-391, :599-609), seeded by the caller where
//     the reference seeds from std::random_device;
//   FlattenBVHRecursive / FlattenBVH (:783-845) and FlattenStackBVH (:847-930); GenerateTriangles
//     (:630-650).
// glm::min(x, y) is x < y ? x : y and glm::max(x, y) is x > y ? x : y (the reference's vendored GLM);
// the argument order of each call is kept, since it decides which of two equal values (+0 / -0)
// survives.
// One case the reference leaves undefined is given a value: a node whose bounds are flat on every
// axis (or whose costs are all NaN) finds no split plane, and the reference then partitions with
// uninitialised axis and border; here axis 0 and border = min.x are used, so the partition finds
// nothing and the midpoint fallback splits the node (as the product builder does).
#include <cstdint>
#include <cstring>
#include <random>
#include <stack>
#include <queue>
#include <vector>

#include "rq_oracle.h"

namespace {

constexpr int kBins = 64;                 // BIN_COUNT (:46)
constexpr float kInfCost = 1e29f;         // INF_COST (:56)
constexpr float kArbMax = 10000000.0f;    // ARBITRARY_MAX (BVHConstructor.h:20)
constexpr float kArbMin = -10000000.0f;   // ARBITRARY_MIN (BVHConstructor.h:21)

// glm::min / glm::max of the reference's vendored GLM (Source/Dependencies/glm/glm/detail/
// func_common.inl:15-28), applied per component by its vector forms
inline float gmin(float x, float y) { return x < y ? x : y; }
inline float gmax(float x, float y) { return x > y ? x : y; }

struct Bounds {  // BVH::Bounds (BVHConstructor.h:23-45)
    float mn[3] = {kArbMax, kArbMax, kArbMax};
    float mx[3] = {kArbMin, kArbMin, kArbMin};
    float area() const {
        const float ex = mx[0] - mn[0], ey = mx[1] - mn[1], ez = mx[2] - mn[2];
        float a = ex * ey;
        a = a + ey * ez;
        a = a + ez * ex;
        return a;
    }
};

struct BNode {
    Bounds b;
    int64_t start = 0, len = 0;
    bool leaf = false;
    int64_t left = -1, right = -1;
};

inline float ibits(int32_t i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

struct Builder {
    const float* verts;  // 8 floats per vertex, position first
    const uint32_t* idx;
    int64_t n_tris;
    int leaf_size;
    int32_t tri_offset;
    bool swaps;
    uint32_t seed;
    std::vector<BNode> nodes;
    std::vector<int64_t> refs, sorted;
    std::vector<Bounds> tb;
    std::vector<float> cen;  // 3 per triangle
    int64_t last_node_index = 0, leaf_count = 0, split_fails = 0;

    void pos(uint32_t v, float p[3]) const {
        for (int k = 0; k < 3; ++k) p[k] = verts[(int64_t)v * 8 + k];
    }

    // SearchSAHPlaneBinned (:276-363).  Returns false when no plane was found.
    bool find_split(const BNode& nd, int& o_axis, float& o_border) const {
        float best = kInfCost;
        bool found = false;
        for (int axis = 0; axis < 3; ++axis) {
            const float mn = nd.b.mn[axis], mx = nd.b.mx[axis];
            if (mn == mx) continue;
            Bounds bins[kBins];
            int count[kBins] = {};
            float larea[kBins - 1], rarea[kBins - 1];
            int lcount[kBins - 1], rcount[kBins - 1];
            const float extent = mx - mn;
            const float scale = static_cast<float>(kBins) / extent;
            for (int64_t i = nd.start; i < nd.start + nd.len; ++i) {
                const int64_t r = refs[i];
                const float c = cen[r * 3 + axis];
                int bin = static_cast<int>((c - mn) * scale);
                bin = (bin < kBins - 1) ? bin : kBins - 1;  // glm::min(BIN_COUNT - 1, ...)
                count[bin]++;
                for (int k = 0; k < 3; ++k) {
                    bins[bin].mn[k] = gmin(bins[bin].mn[k], tb[r].mn[k]);
                    bins[bin].mx[k] = gmax(bins[bin].mx[k], tb[r].mx[k]);
                }
            }
            Bounds lb, rb;
            int lsum = 0, rsum = 0;
            for (int i = 0; i < kBins - 1; ++i) {
                lsum += count[i];
                lcount[i] = lsum;
                for (int k = 0; k < 3; ++k) {
                    lb.mn[k] = gmin(lb.mn[k], bins[i].mn[k]);
                    lb.mx[k] = gmax(lb.mx[k], bins[i].mx[k]);
                }
                larea[i] = lb.area();
                const int ir = kBins - 1 - i;
                rsum += count[ir];
                rcount[ir - 1] = rsum;
                for (int k = 0; k < 3; ++k) {
                    rb.mn[k] = gmin(rb.mn[k], bins[ir].mn[k]);
                    rb.mx[k] = gmax(rb.mx[k], bins[ir].mx[k]);
                }
                rarea[ir - 1] = rb.area();
            }
            const float step = extent / static_cast<float>(kBins);
            for (int i = 0; i < kBins - 1; ++i) {
                float cost = static_cast<float>(lcount[i]) * larea[i];
                cost = cost + static_cast<float>(rcount[i]) * rarea[i];
                if (cost < best) {
                    best = cost;
                    o_axis = axis;
                    o_border = mn + step * static_cast<float>(i + 1);
                    found = true;
                }
            }
        }
        return found;
    }

    // ConstructTree (:385-627).
    void construct() {
        refs.resize(n_tris);
        for (int64_t i = 0; i < n_tris; ++i) refs[i] = i;
        tb.resize(n_tris);
        cen.resize(n_tris * 3);
        Bounds root;
        for (int64_t t = 0; t < n_tris; ++t) {
            Bounds cb;
            for (int c = 0; c < 3; ++c) {
                float p[3];
                pos(idx[t * 3 + c], p);
                for (int k = 0; k < 3; ++k) {
                    cb.mn[k] = gmin(cb.mn[k], p[k]);
                    cb.mx[k] = gmax(cb.mx[k], p[k]);
                }
            }
            for (int k = 0; k < 3; ++k) {
                root.mn[k] = gmin(root.mn[k], cb.mn[k]);
                root.mx[k] = gmax(root.mx[k], cb.mx[k]);
                cen[t * 3 + k] = (cb.mn[k] + cb.mx[k]) / 2.0f;  // GetCenter
            }
            tb[t] = cb;
        }
        nodes.reserve(2 * n_tris + 1);
        nodes.push_back(BNode{});
        nodes[0].b = root;
        nodes[0].len = n_tris;
        std::mt19937 rng(seed);
        std::uniform_int_distribution<std::mt19937::result_type> dist(1, 4);
        std::stack<int64_t> work;
        work.push(0);
        while (!work.empty()) {
            const int64_t id = work.top();
            work.pop();
            if (nodes[id].len <= leaf_size || nodes[id].len <= 1) {
                BNode& nd = nodes[id];
                nd.leaf = true;
                ++leaf_count;
                const int64_t fin = static_cast<int64_t>(sorted.size());
                for (int64_t i = nd.start; i < nd.start + nd.len; ++i) sorted.push_back(refs[i]);
                nd.start = fin + tri_offset;
                continue;
            }
            int axis = 0;
            float border = nodes[id].b.mn[0];
            find_split(nodes[id], axis, border);
            const int64_t start = nodes[id].start, len = nodes[id].len;
            int64_t mid = start;
            for (int64_t i = start; i < start + len; ++i) {
                if (cen[refs[i] * 3 + axis] < border) {
                    std::swap(refs[i], refs[mid]);
                    ++mid;
                }
            }
            if (mid == start || mid == start + len) {
                mid = start + len / 2;
                ++split_fails;
            }
            last_node_index += 2;
            BNode ln, rn;
            ln.start = start;
            ln.len = mid - start;
            rn.start = mid;
            rn.len = start + len - mid;
            for (BNode* ch : {&ln, &rn}) {
                float cmn[3] = {kArbMax, kArbMax, kArbMax}, cmx[3] = {kArbMin, kArbMin, kArbMin};
                for (int64_t x = 0; x < ch->len; ++x) {
                    const Bounds& bb = tb[refs[ch->start + x]];
                    for (int k = 0; k < 3; ++k) {
                        cmn[k] = gmin(bb.mn[k], cmn[k]);  // glm::min(bounds.Min, LeftMin)
                        cmx[k] = gmax(bb.mx[k], cmx[k]);  // glm::max(bounds.Max, LeftMax)
                    }
                }
                for (int k = 0; k < 3; ++k) {
                    ch->b.mn[k] = cmn[k];
                    ch->b.mx[k] = cmx[k];
                }
            }
            const int64_t L = static_cast<int64_t>(nodes.size());
            nodes.push_back(ln);
            const int64_t R = static_cast<int64_t>(nodes.size());
            nodes.push_back(rn);
            // the swap exchanges the child pointers only; the stack still receives the nodes as
            // they were split (LeftNode / RightNode are bound before the swap, :558-570, :611-625)
            int64_t cl = L, cr = R;
            if (swaps) {
                const uint32_t h = static_cast<uint32_t>(dist(rng));
                if (h <= 2) std::swap(cl, cr);
            }
            nodes[id].len = 0;
            nodes[id].left = cl;
            nodes[id].right = cr;
            work.push(L);
            work.push(R);
        }
    }

    // FlattenBVHRecursive (:801-822): pre-order, cache.x = index of the right child (or -1 for a
    // leaf), cache.y = packed leaf data.
    int64_t flatten_rec(int64_t id, float* out, std::vector<int32_t>& cx, std::vector<int32_t>& cy,
                        int64_t& processed) {
        const int64_t at = processed;
        const BNode& nd = nodes[id];
        for (int k = 0; k < 3; ++k) {
            out[at * 8 + k] = nd.b.mn[k];
            out[at * 8 + 4 + k] = nd.b.mx[k];
        }
        out[at * 8 + 3] = 0.0f;
        out[at * 8 + 7] = 0.0f;
        ++processed;
        if (nd.leaf) {
            cy[at] = static_cast<int32_t>((nd.start << 4) | (nd.len & 0xF));
            cx[at] = -1;
        } else {
            flatten_rec(nd.left, out, cx, cy, processed);
            cx[at] = static_cast<int32_t>(flatten_rec(nd.right, out, cx, cy, processed));
        }
        return at;
    }

    // FlattenBVH (:824-845).
    void flatten_stackless(float* out, int64_t n) {
        std::vector<int32_t> cx(n, 0), cy(n, 0);
        int64_t processed = 0;
        flatten_rec(0, out, cx, cy, processed);
        out[7] = ibits(-1);
        for (int64_t i = 0; i < n; ++i) {
            if (cx[i] != -1) {
                out[(i + 1) * 8 + 7] = ibits(cx[i]);
                out[static_cast<int64_t>(cx[i]) * 8 + 7] = out[i * 8 + 7];
            }
        }
        for (int64_t i = 0; i < n; ++i) out[i * 8 + 3] = (cx[i] == -1) ? ibits(cy[i]) : ibits(-1);
    }

    // FlattenStackBVH (:847-930): breadth first; the link of an internal child is written when the
    // child itself is dequeued.
    void flatten_stack(float* out) {
        int64_t counter = 0;
        std::queue<std::pair<int64_t, int64_t>> q;
        q.push({0, 0});
        while (!q.empty()) {
            const auto cur = q.front();
            q.pop();
            float* nd = out + (counter++) * 16;
            const BNode& p = nodes[cur.first];
            const int64_t ch[2] = {p.left, p.right};
            for (int side = 0; side < 2; ++side) {
                const BNode& c = nodes[ch[side]];
                float* f = nd + side * 8;
                for (int k = 0; k < 3; ++k) {
                    f[k] = c.b.mn[k];
                    f[4 + k] = c.b.mx[k];
                }
                f[7] = 0.0f;
                if (!c.leaf) {
                    f[3] = ibits(-1);
                    q.push({ch[side], side == 0 ? counter : -counter});
                } else {
                    f[3] = ibits(static_cast<int32_t>((c.start << 4) | (c.len & 0xF)));
                }
            }
            if (cur.second > 0)
                out[(cur.second - 1) * 16 + 7] = ibits(static_cast<int32_t>(counter - 1));
            else if (cur.second < 0)
                out[(-cur.second - 1) * 16 + 8 + 7] = ibits(static_cast<int32_t>(counter - 1));
        }
    }
};

}  // namespace

extern "C" {

struct orc_bvh {
    std::vector<float> nodes;
    std::vector<int32_t> tris;
    int64_t n_nodes = 0, leaf_count = 0, split_fails = 0;
    int32_t stackless = 0;
};

orc_bvh* orc_build_bvh(const void* verts, int64_t n_verts, const uint32_t* indices, int64_t n_indices,
                       const int32_t* mesh_ids, int32_t tri_offset, int32_t stackless, int32_t leaf_size,
                       int32_t swap_children, uint32_t swap_seed) {
    const int64_t nt = n_indices / 3;
    if (!verts || !indices || nt <= 0 || leaf_size < 1 || leaf_size > 15) return nullptr;
    if (!stackless && nt <= leaf_size) return nullptr;  // the reference dereferences a null child
    for (int64_t i = 0; i < n_indices; ++i)
        if (static_cast<int64_t>(indices[i]) >= n_verts) return nullptr;
    Builder b{static_cast<const float*>(verts), indices, nt, leaf_size, tri_offset,
              stackless != 0 && swap_children != 0, swap_seed};
    b.construct();
    auto* out = new orc_bvh;
    out->n_nodes = b.last_node_index + 1;
    out->leaf_count = b.leaf_count;
    out->split_fails = b.split_fails;
    out->stackless = stackless;
    out->nodes.assign(out->n_nodes * (stackless ? 8 : 16), 0.0f);
    if (stackless)
        b.flatten_stackless(out->nodes.data(), out->n_nodes);
    else
        b.flatten_stack(out->nodes.data());
    out->tris.resize(nt * 4);
    for (int64_t i = 0; i < nt; ++i) {
        const int64_t t = b.sorted[i];
        out->tris[i * 4 + 0] = static_cast<int32_t>(indices[t * 3 + 0]);
        out->tris[i * 4 + 1] = static_cast<int32_t>(indices[t * 3 + 1]);
        out->tris[i * 4 + 2] = static_cast<int32_t>(indices[t * 3 + 2]);
        out->tris[i * 4 + 3] = mesh_ids ? mesh_ids[t] : 0;
    }
    return out;
}

void orc_bvh_info(const orc_bvh* b, int64_t* n_nodes, int64_t* leaf_count, int64_t* split_fails) {
    *n_nodes = b->n_nodes;
    *leaf_count = b->leaf_count;
    *split_fails = b->split_fails;
}

void orc_bvh_copy(const orc_bvh* b, float* nodes, int32_t* tris) {
    std::memcpy(nodes, b->nodes.data(), b->nodes.size() * sizeof(float));
    std::memcpy(tris, b->tris.data(), b->tris.size() * sizeof(int32_t));
}

void orc_bvh_free(orc_bvh* b) { delete b; }

}  // extern "C"
