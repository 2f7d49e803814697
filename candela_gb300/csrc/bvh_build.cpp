// Host SAH BVH builder.
//
// Produces the reference constructor's flattened buffers byte for byte
// (Source/Core/BVH/BVHConstructor.cpp), so that a scene built here and a scene built by the
// reference traverse identically.  The reference's split rule, partition and output numbering are
// reproduced step for step, because the buffers are the interface:
//   * binned SAH, 64 bins per axis, cost nL*areaL + nR*areaR with area = xy + yz + zx,
//     border = min + (extent/64)*(i+1)                      (BVHConstructor.cpp:276-363, .h:41-44)
//   * Lomuto partition by `centroid < border`, midpoint fallback           (:532-556)
//   * leaf when length <= MAX_TRIANGLES_PER_LEAF                           (:81-87, :456)
//   * leaves are numbered in the order of a LIFO walk that visits the upper (right) half first
//     (:443-470, :624-625); stackless child swaps use an mt19937 drawing uniform{1..4}
//     per split, in that same walk order                                   (:389-391, :599-609)
//   * stackless nodes in DFS pre-order with escape links                   (:783-845)
//   * stack nodes in BFS order, one per internal node                      (:847-930)
//   * triangles permuted into leaf order {i0, i1, i2, mesh}                (:630-650)
// glm's min/max return their second argument on ties (glm 0.9.8 func_common.inl:15-27); every
// call below keeps the reference's argument order because that decides which of +0/-0 survives.
//
// What differs is how the work is scheduled: the tree is built by a task-parallel recursion over
// disjoint triangle ranges (each node only touches its own range), large nodes bin their
// triangles with several threads and merge the per-thread bins in range order (which preserves
// the sequential tie behaviour), and all three axes are binned in one pass.  Leaf numbering and
// the random child swaps, which depend on the reference's sequential walk order, are assigned in a
// separate sequential pass over the finished tree.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <deque>
#include <random>
#include <thread>
#include <utility>

namespace rq {
namespace {

constexpr int kBins = 64;
constexpr float kArbMax = 10000000.0f;   // ARBITRARY_MAX (BVHConstructor.h:21)
constexpr float kArbMin = -10000000.0f;  // ARBITRARY_MIN (BVHConstructor.h:22)
constexpr float kInfCost = 1e29f;        // INF_COST (BVHConstructor.cpp:56)

inline float gmin(float x, float y) { return x < y ? x : y; }  // glm::min
inline float gmax(float x, float y) { return x > y ? x : y; }  // glm::max

struct Box {
    float mn[3], mx[3];
    void reset() {
        mn[0] = mn[1] = mn[2] = kArbMax;
        mx[0] = mx[1] = mx[2] = kArbMin;
    }
    // Accumulator-first argument order: glm::min(acc, x) keeps x on ties.
    void grow_acc_first(const float* bmn, const float* bmx) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = gmin(mn[k], bmn[k]);
            mx[k] = gmax(mx[k], bmx[k]);
        }
    }
    // New-first argument order: glm::min(x, acc) keeps acc on ties (child bounds, :573-597).
    void grow_new_first(const float* bmn, const float* bmx) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = gmin(bmn[k], mn[k]);
            mx[k] = gmax(bmx[k], mx[k]);
        }
    }
    float area() const {  // Bounds::GetArea, BVHConstructor.h:41-44
        const float ex = mx[0] - mn[0], ey = mx[1] - mn[1], ez = mx[2] - mn[2];
        float a = ex * ey;
        a = a + ey * ez;
        a = a + ez * ex;
        return a;
    }
};

struct Node {
    Box box;
    uint32_t start = 0, len = 0;
    int32_t left = -1, right = -1;  // indices into the node arena (after swaps: left/right ptrs)
    int32_t orig_left = -1, orig_right = -1;
    bool leaf = false;
};

struct Bins {
    int32_t count[3][kBins];
    Box box[3][kBins];
    void reset() {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < kBins; ++b) {
                count[a][b] = 0;
                box[a][b].reset();
            }
    }
};

struct Builder {
    const BuildInput& in;
    int64_t n;
    std::vector<float> tmn[3], tmx[3], cen[3];  // per-triangle bounds and centroid (SoA)
    std::vector<int32_t> refs;                  // TriangleReferences
    std::vector<Node> nodes;
    std::atomic<int64_t> next_node{0};
    std::atomic<int64_t> split_fails{0};
    int n_threads = 1;
    std::atomic<int> live_threads{1};
    int64_t max_depth = 0;
    std::atomic<int64_t> depth_seen{0};

    explicit Builder(const BuildInput& i) : in(i), n(i.n_tris) {}

    int32_t alloc_node() { return static_cast<int32_t>(next_node.fetch_add(1)); }

    void bin_range(const Node& nd, uint32_t b, uint32_t e, Bins& bins, const float* scale,
                   const bool* active) const {
        for (uint32_t i = b; i < e; ++i) {
            const int32_t r = refs[i];
            const float bmn[3] = {tmn[0][r], tmn[1][r], tmn[2][r]};
            const float bmx[3] = {tmx[0][r], tmx[1][r], tmx[2][r]};
            for (int a = 0; a < 3; ++a) {
                if (!active[a]) continue;
                int bi = static_cast<int>((cen[a][r] - nd.box.mn[a]) * scale[a]);
                bi = kBins - 1 < bi ? kBins - 1 : bi;  // glm::min(BIN_COUNT - 1, idx)
                ++bins.count[a][bi];
                bins.box[a][bi].grow_acc_first(bmn, bmx);
            }
        }
    }

    // SearchSAHPlaneBinned, BVHConstructor.cpp:276-363.  Returns false when every axis is flat.
    bool find_split(const Node& nd, int& axis, float& border) {
        bool active[3];
        float scale[3], extent[3];
        for (int a = 0; a < 3; ++a) {
            active[a] = !(nd.box.mn[a] == nd.box.mx[a]);
            extent[a] = nd.box.mx[a] - nd.box.mn[a];
            scale[a] = static_cast<float>(kBins) / extent[a];
        }
        Bins bins;
        bins.reset();
        const uint32_t b0 = nd.start, e0 = nd.start + nd.len;
        const int par = (nd.len >= (1u << 17)) ? std::min(n_threads, 16) : 1;
        if (par <= 1) {
            bin_range(nd, b0, e0, bins, scale, active);
        } else {
            std::vector<Bins> part(par);
            std::vector<std::thread> th;
            const uint32_t chunk = (nd.len + par - 1) / par;
            for (int t = 0; t < par; ++t) {
                part[t].reset();
                const uint32_t b = b0 + t * chunk, e = std::min(e0, b + chunk);
                if (b >= e) continue;
                th.emplace_back([&, t, b, e] { bin_range(nd, b, e, part[t], scale, active); });
            }
            for (auto& x : th) x.join();
            // Merge in range order: glm::min(acc, chunk) keeps the later chunk on ties, which is
            // what the sequential loop keeps.  Empty chunk bins hold the sentinel and are skipped.
            for (int t = 0; t < par; ++t)
                for (int a = 0; a < 3; ++a)
                    for (int k = 0; k < kBins; ++k) {
                        if (part[t].count[a][k] == 0) continue;
                        bins.count[a][k] += part[t].count[a][k];
                        bins.box[a][k].grow_acc_first(part[t].box[a][k].mn, part[t].box[a][k].mx);
                    }
        }
        float best = kInfCost;
        bool found = false;
        for (int a = 0; a < 3; ++a) {
            if (!active[a]) continue;
            float larea[kBins - 1], rarea[kBins - 1];
            int lcount[kBins - 1], rcount[kBins - 1];
            Box lb, rb;
            lb.reset();
            rb.reset();
            int lsum = 0, rsum = 0;
            for (int i = 0; i < kBins - 1; ++i) {
                lsum += bins.count[a][i];
                lcount[i] = lsum;
                lb.grow_acc_first(bins.box[a][i].mn, bins.box[a][i].mx);
                larea[i] = lb.area();
                const int ir = kBins - 1 - i;
                rsum += bins.count[a][ir];
                rcount[ir - 1] = rsum;
                rb.grow_acc_first(bins.box[a][ir].mn, bins.box[a][ir].mx);
                rarea[ir - 1] = rb.area();
            }
            const float step = extent[a] / static_cast<float>(kBins);
            for (int i = 0; i < kBins - 1; ++i) {
                float c = static_cast<float>(lcount[i]) * larea[i];
                c = c + static_cast<float>(rcount[i]) * rarea[i];
                if (c < best) {
                    best = c;
                    axis = a;
                    border = nd.box.mn[a] + step * static_cast<float>(i + 1);
                    found = true;
                }
            }
        }
        return found;
    }

    void process(int32_t id, int depth) {
        int64_t d = depth_seen.load();
        while (depth > d && !depth_seen.compare_exchange_weak(d, depth)) {
        }
        Node& nd = nodes[id];
        const uint32_t cap = static_cast<uint32_t>(in.leaf_size);
        if (nd.len <= cap || nd.len <= 1) {
            nd.leaf = true;
            return;
        }
        int axis = 0;
        float border = nd.box.mn[0];
        find_split(nd, axis, border);  // all-flat node: partition below finds nothing -> midpoint
        // Lomuto partition (BVHConstructor.cpp:532-550).
        uint32_t mid = nd.start;
        const std::vector<float>& c = cen[axis];
        for (uint32_t i = nd.start; i < nd.start + nd.len; ++i) {
            if (c[refs[i]] < border) {
                std::swap(refs[i], refs[mid]);
                ++mid;
            }
        }
        if (mid == nd.start || mid == nd.start + nd.len) {
            mid = nd.start + nd.len / 2;
            split_fails.fetch_add(1);
        }
        const int32_t L = alloc_node(), R = alloc_node();
        Node& ln = nodes[L];
        Node& rn = nodes[R];
        ln.start = nd.start;
        ln.len = mid - nd.start;
        rn.start = mid;
        rn.len = nd.start + nd.len - mid;
        for (Node* ch : {&ln, &rn}) {
            ch->box.reset();
            for (uint32_t i = ch->start; i < ch->start + ch->len; ++i) {
                const int32_t r = refs[i];
                const float bmn[3] = {tmn[0][r], tmn[1][r], tmn[2][r]};
                const float bmx[3] = {tmx[0][r], tmx[1][r], tmx[2][r]};
                ch->box.grow_new_first(bmn, bmx);
            }
        }
        nd.left = nd.orig_left = L;
        nd.right = nd.orig_right = R;
        // Recurse; large halves run on their own thread while threads are available.
        const bool spawn = rn.len >= 4096 && ln.len >= 4096 &&
                           live_threads.fetch_add(1) < n_threads;
        if (spawn) {
            std::thread t([this, R, depth] { process(R, depth + 1); });
            process(L, depth + 1);
            t.join();
            live_threads.fetch_sub(1);
        } else {
            if (rn.len >= 4096 && ln.len >= 4096) live_threads.fetch_sub(1);
            process(R, depth + 1);
            process(L, depth + 1);
        }
    }
};

inline float i2f(int32_t i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

}  // namespace

int build_bvh(const BuildInput& in, BuildOutput& out) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!in.vert_records || !in.indices || in.n_tris <= 0 || in.n_verts <= 0) return -1;
    if (in.leaf_size < 1 || in.leaf_size > 15) return -1;
    if (in.layout != 0 && in.layout != 1) return -1;
    if (in.n_tris + static_cast<int64_t>(in.tri_offset) >= (int64_t(1) << 27)) return -1;
    if (in.layout == 0 && in.n_tris <= in.leaf_size) return -1;  // stack layout needs a split root
    for (int64_t i = 0; i < in.n_tris * 3; ++i)
        if (static_cast<int64_t>(in.indices[i]) >= in.n_verts) return -1;

    Builder b(in);
    const int64_t n = in.n_tris;
    b.n_threads = in.n_threads > 0 ? in.n_threads
                                   : std::max(1u, std::thread::hardware_concurrency());
    for (int a = 0; a < 3; ++a) {
        b.tmn[a].resize(n);
        b.tmx[a].resize(n);
        b.cen[a].resize(n);
    }
    b.refs.resize(n);
    // Per-triangle bounds and centroids (BVHConstructor.cpp:406-424), in parallel over triangles.
    auto tri_bounds = [&](int64_t lo, int64_t hi) {
        for (int64_t t = lo; t < hi; ++t) {
            float mn[3] = {kArbMax, kArbMax, kArbMax}, mx[3] = {kArbMin, kArbMin, kArbMin};
            for (int v = 0; v < 3; ++v) {
                const float* p = in.vert_records + static_cast<int64_t>(in.indices[t * 3 + v]) * 8;
                for (int k = 0; k < 3; ++k) {
                    mn[k] = gmin(mn[k], p[k]);
                    mx[k] = gmax(mx[k], p[k]);
                }
            }
            for (int k = 0; k < 3; ++k) {
                b.tmn[k][t] = mn[k];
                b.tmx[k][t] = mx[k];
                b.cen[k][t] = (mn[k] + mx[k]) / 2.0f;
            }
            b.refs[t] = static_cast<int32_t>(t);
        }
    };
    {
        std::vector<std::thread> th;
        const int T = n >= 65536 ? b.n_threads : 1;
        const int64_t chunk = (n + T - 1) / T;
        for (int t = 0; t < T; ++t) {
            const int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
            if (lo < hi) th.emplace_back(tri_bounds, lo, hi);
        }
        for (auto& x : th) x.join();
    }
    b.nodes.resize(static_cast<size_t>(2 * n + 1));
    const int32_t root = b.alloc_node();
    Node& rn = b.nodes[root];
    rn.start = 0;
    rn.len = static_cast<uint32_t>(n);
    rn.box.reset();
    for (int64_t t = 0; t < n; ++t) {  // MinInitial/MaxInitial (:420-421): glm::min(acc, tri)
        const float bmn[3] = {b.tmn[0][t], b.tmn[1][t], b.tmn[2][t]};
        const float bmx[3] = {b.tmx[0][t], b.tmx[1][t], b.tmx[2][t]};
        rn.box.grow_acc_first(bmn, bmx);
    }
    b.process(root, 1);
    const int64_t total = b.next_node.load();
    std::vector<Node>& N = b.nodes;

    // Sequential walk in the reference's processing order: leaf numbering and child swaps.
    std::vector<int32_t> sorted;
    sorted.reserve(n);
    {
        const bool swaps = in.layout == 1 && in.swap_children;
        std::mt19937 rng(in.swap_seed);
        std::uniform_int_distribution<std::mt19937::result_type> dist(1, 4);
        std::vector<int32_t> st;
        st.push_back(root);
        while (!st.empty()) {
            const int32_t id = st.back();
            st.pop_back();
            Node& nd = N[id];
            if (nd.leaf) {
                const int64_t fin = static_cast<int64_t>(sorted.size());
                for (uint32_t i = nd.start; i < nd.start + nd.len; ++i) sorted.push_back(b.refs[i]);
                nd.start = static_cast<uint32_t>(fin + in.tri_offset);
                ++out.leaf_count;
                continue;
            }
            if (swaps && dist(rng) <= 2) std::swap(nd.left, nd.right);
            st.push_back(nd.orig_left);
            st.push_back(nd.orig_right);
        }
    }
    out.split_fails = b.split_fails.load();
    out.max_depth = b.depth_seen.load();

    // Triangles in leaf order (GenerateTriangles, :630-650).
    out.tris.resize(static_cast<size_t>(n) * 4);
    for (int64_t i = 0; i < n; ++i) {
        const int32_t t = sorted[i];
        out.tris[i * 4 + 0] = static_cast<int32_t>(in.indices[t * 3 + 0]);
        out.tris[i * 4 + 1] = static_cast<int32_t>(in.indices[t * 3 + 1]);
        out.tris[i * 4 + 2] = static_cast<int32_t>(in.indices[t * 3 + 2]);
        out.tris[i * 4 + 3] = in.mesh_ids ? in.mesh_ids[t] : 0;
    }

    auto packed = [](const Node& nd) {
        return static_cast<int32_t>((nd.start << 4) | (nd.len & 0xFu));
    };
    out.n_nodes = total;  // LastNodeIndex + 1
    if (in.layout == 1) {
        // DFS pre-order (FlattenBVHRecursive, :795-819) and link pass (:821-845).
        out.nodes.assign(static_cast<size_t>(total) * 8, 0.0f);
        std::vector<int32_t> order(total), right_of(total, -1), flat_of(total, -1);
        std::vector<int32_t> st;
        st.push_back(root);
        int32_t next = 0;
        while (!st.empty()) {
            const int32_t id = st.back();
            st.pop_back();
            flat_of[id] = next;
            order[next++] = id;
            if (!N[id].leaf) {
                st.push_back(N[id].right);
                st.push_back(N[id].left);
            }
        }
        float* F = out.nodes.data();
        for (int64_t i = 0; i < total; ++i) {
            const Node& nd = N[order[i]];
            for (int k = 0; k < 3; ++k) {
                F[i * 8 + k] = nd.box.mn[k];
                F[i * 8 + 4 + k] = nd.box.mx[k];
            }
        }
        F[7] = i2f(-1);
        for (int64_t i = 0; i < total; ++i) {
            const Node& nd = N[order[i]];
            if (!nd.leaf) {
                const int32_t r = flat_of[nd.right];
                F[(i + 1) * 8 + 7] = i2f(r);
                F[static_cast<int64_t>(r) * 8 + 7] = F[i * 8 + 7];
            }
        }
        for (int64_t i = 0; i < total; ++i) {
            const Node& nd = N[order[i]];
            F[i * 8 + 3] = nd.leaf ? i2f(packed(nd)) : i2f(-1);
        }
        out.n_nodes_used = total;
    } else {
        // BFS over internal nodes (FlattenStackBVH, :847-930).
        out.nodes.assign(static_cast<size_t>(total) * 16, 0.0f);
        float* F = out.nodes.data();
        std::deque<std::pair<int32_t, int32_t>> q;
        q.emplace_back(root, 0);
        int32_t counter = 0;
        while (!q.empty()) {
            const auto cur = q.front();
            q.pop_front();
            const int64_t me = counter++;
            const Node& nd = N[cur.first];
            const int32_t kids[2] = {nd.left, nd.right};
            for (int s = 0; s < 2; ++s) {
                const Node& ch = N[kids[s]];
                float* bnd = F + me * 16 + s * 8;
                for (int k = 0; k < 3; ++k) {
                    bnd[k] = ch.box.mn[k];
                    bnd[4 + k] = ch.box.mx[k];
                }
                bnd[7] = 0.0f;
                if (!ch.leaf) {
                    bnd[3] = i2f(-1);
                    q.emplace_back(kids[s], s == 0 ? counter : -counter);
                } else {
                    bnd[3] = i2f(packed(ch));
                }
            }
            if (cur.second > 0)
                F[static_cast<int64_t>(cur.second - 1) * 16 + 7] = i2f(counter - 1);
            else if (cur.second < 0)
                F[static_cast<int64_t>(-cur.second - 1) * 16 + 15] = i2f(counter - 1);
        }
        out.n_nodes_used = counter;
    }
    out.build_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

}  // namespace rq
