// BVH2 -> BVH8 collapse and 8-bit child-box quantisation (the compressed wide BVH of Ylitie,
// Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs",
// HPG 2017), built from the reference's flattened BVH2 buffers.
//
// Collapse: the SAH-optimal assignment of that paper.  A bottom-up dynamic programme over the
// BVH2 gives, for every node n and slot budget i = 1..8, the cheapest way to place n's subtree in
// at most i child slots of one BVH8 node: as one leaf child (all triangles of the subtree, at most
// kLeafMax, or a BVH2 leaf as given), as one internal child (a new BVH8 node whose 8 slots hold n's
// subtree), or split between its two BVH2 children.  Cost = surface area x (kNodeCost for a node
// visit, kTriCost per triangle test).  A top-down pass then emits the chosen BVH8.
// Quantisation: per node, a grid origin p (the node's min corner) and a power-of-two step per
// axis; child boxes are rounded outward (floor / ceil) and then checked in double precision so that
// every decoded child box contains the child's FP32 box.
#include "bvh8.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <limits>
#include <unordered_map>

namespace rq {
namespace {

struct TNode {
    float lo[3], hi[3];
    int32_t a = -1, b = -1;      // children (temp indices) when internal
    int32_t tri_start = 0, tri_count = 0;
    bool leaf = false;
};

inline int32_t bits(float f) {
    int32_t i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline float fbits(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

float half_area(const TNode& n) {
    const float x = n.hi[0] - n.lo[0], y = n.hi[1] - n.lo[1], z = n.hi[2] - n.lo[2];
    return x * y + y * z + z * x;
}

// Rebuilds the pointer tree of one object's BVH2 from the flattened buffer.
bool recover_tree(int32_t layout, const float* nodes, int32_t off, int32_t cnt, int64_t n_tris,
                  std::vector<TNode>& T, std::string& why) {
    T.clear();
    std::vector<uint8_t> seen(static_cast<size_t>(cnt), 0);
    auto leaf_node = [&](const float* lo, const float* hi, int32_t packed, TNode& t) -> bool {
        t.leaf = true;
        for (int k = 0; k < 3; ++k) {
            t.lo[k] = lo[k];
            t.hi[k] = hi[k];
        }
        t.tri_start = packed >> 4;
        t.tri_count = packed & 0xF;
        if (packed < 0 || t.tri_start + t.tri_count > n_tris) {
            why = "leaf range out of bounds";
            return false;
        }
        if (t.tri_count > 4) {
            why = "BVH8 needs BVH2 leaves of at most 4 triangles";
            return false;
        }
        return true;
    };
    if (layout == 1) {
        // Stack layout: node j holds both children's boxes; the object root's box is their union.
        struct Work {
            int32_t tnode;  // temp node to fill (internal)
            int32_t j;      // flattened node holding its two children
        };
        T.emplace_back();
        std::vector<Work> st{{0, 0}};
        while (!st.empty()) {
            const Work w = st.back();
            st.pop_back();
            if (w.j < 0 || w.j >= cnt || seen[w.j]) {
                why = "stack BVH is not a tree";
                return false;
            }
            seen[w.j] = 1;
            const float* nd = nodes + static_cast<int64_t>(off + w.j) * 16;
            int32_t kids[2];
            for (int s = 0; s < 2; ++s) {
                const float* lo = nd + s * 8;
                const float* hi = nd + s * 8 + 4;
                const int32_t kind = bits(lo[3]);
                TNode c;
                if (kind != -1) {
                    if (!leaf_node(lo, hi, kind, c)) return false;
                } else {
                    for (int k = 0; k < 3; ++k) {
                        c.lo[k] = lo[k];
                        c.hi[k] = hi[k];
                    }
                }
                kids[s] = static_cast<int32_t>(T.size());
                T.push_back(c);
                if (kind == -1) st.push_back({kids[s], bits(hi[3])});
            }
            TNode& p = T[w.tnode];
            p.a = kids[0];
            p.b = kids[1];
            if (w.tnode == 0) {
                for (int k = 0; k < 3; ++k) {
                    p.lo[k] = std::min(T[kids[0]].lo[k], T[kids[1]].lo[k]);
                    p.hi[k] = std::max(T[kids[0]].hi[k], T[kids[1]].hi[k]);
                }
            }
        }
        return true;
    }
    // Stackless layout: DFS pre-order; left child = j + 1, right child = escape link of j + 1.
    struct Work {
        int32_t tnode, j;
    };
    T.emplace_back();
    std::vector<Work> st{{0, 0}};
    while (!st.empty()) {
        const Work w = st.back();
        st.pop_back();
        if (w.j < 0 || w.j >= cnt || seen[w.j]) {
            why = "stackless BVH is not a tree";
            return false;
        }
        seen[w.j] = 1;
        const float* nd = nodes + static_cast<int64_t>(off + w.j) * 8;
        const int32_t kind = bits(nd[3]);
        if (kind != -1) {
            TNode c;
            if (!leaf_node(nd, nd + 4, kind, c)) return false;
            T[w.tnode] = c;
            continue;
        }
        TNode& p = T[w.tnode];
        for (int k = 0; k < 3; ++k) {
            p.lo[k] = nd[k];
            p.hi[k] = nd[4 + k];
        }
        const int32_t left = w.j + 1;
        if (left >= cnt) {
            why = "internal node without children";
            return false;
        }
        const int32_t right = bits(nodes[static_cast<int64_t>(off + left) * 8 + 7]);
        const int32_t ta = static_cast<int32_t>(T.size());
        T.emplace_back();
        T.emplace_back();
        T[w.tnode].a = ta;
        T[w.tnode].b = ta + 1;
        st.push_back({ta, left});
        st.push_back({ta + 1, right});
    }
    return true;
}

// One strict triangle test with its 64-byte record costs about as much as a node visit in the
// GB300 walk.  C2 GI pass by triangle cost / leaf size: 0.15/3 1.053 ms, 0.3/3 1.044, 0.6/3 1.020,
// 1.0/3 1.019, 2.0/3 1.021, 0.3/2 1.020, 0.3/4 1.054, 0.15/4 1.091 (same hit records); from 0.6 up
// the collapse keeps the BVH2 leaves as they are.
constexpr float kNodeCost = 1.0f;  // one BVH8 node visit (eight child box tests)
constexpr float kTriCost = 1.0f;   // one triangle test, relative to a node visit
constexpr int kLeafMax = 3;        // triangles merged into one leaf child

// Dynamic-programme tables of one BVH2 tree (index = temp node).
struct Collapse {
    std::vector<float> cost;     // cost[8n + i - 1] = C(n, i)
    std::vector<int8_t> split;   // split[8n + i - 1] = k of the best split of n into i slots
    std::vector<uint16_t> flag;  // bit 0: C(n, 1) is a leaf child; bit i-1 (i >= 2): C(n, i) = C(n, i-1)
    std::vector<int32_t> ntris;  // triangles below n
};

void collapse_costs(const std::vector<TNode>& T, Collapse& D) {
    const size_t n = T.size();
    D.cost.assign(8 * n, 0.0f);
    D.split.assign(8 * n, 0);
    D.flag.assign(n, 0);
    D.ntris.assign(n, 0);
    const float inf = std::numeric_limits<float>::infinity();
    // children have larger temp indices than their parent (both recoveries append them later)
    for (size_t j = n; j-- > 0;) {
        const TNode& t = T[j];
        const float area = std::max(half_area(t), 0.0f);
        float* c = &D.cost[8 * j];
        if (t.leaf) {
            D.ntris[j] = t.tri_count;
            for (int i = 0; i < 8; ++i) c[i] = area * kTriCost * static_cast<float>(t.tri_count);
            D.flag[j] = 1;
            continue;
        }
        D.ntris[j] = D.ntris[t.a] + D.ntris[t.b];
        const float* ca = &D.cost[8 * static_cast<size_t>(t.a)];
        const float* cb = &D.cost[8 * static_cast<size_t>(t.b)];
        float dist[9];
        for (int i = 2; i <= 8; ++i) {
            float best = inf;
            int bk = 1;
            for (int k = 1; k < i; ++k) {
                const float v = ca[k - 1] + cb[i - k - 1];
                if (v < best) {
                    best = v;
                    bk = k;
                }
            }
            dist[i] = best;
            D.split[8 * j + i - 1] = static_cast<int8_t>(bk);
        }
        const float internal = area * kNodeCost + dist[8];
        const float leaf = D.ntris[j] <= kLeafMax ? area * kTriCost * static_cast<float>(D.ntris[j]) : inf;
        uint16_t f = 0;
        if (leaf <= internal) {
            c[0] = leaf;
            f |= 1;
        } else {
            c[0] = internal;
        }
        for (int i = 2; i <= 8; ++i) {
            if (c[i - 2] <= dist[i]) {
                c[i - 1] = c[i - 2];
                f |= static_cast<uint16_t>(1u << (i - 1));
            } else {
                c[i - 1] = dist[i];
            }
        }
        D.flag[j] = f;
    }
}

struct Slot {
    int32_t tnode;
    bool leaf;
};

// The child slots that subtree x takes with a budget of i slots.
void collect(const std::vector<TNode>& T, const Collapse& D, int32_t x, int i, std::vector<Slot>& out) {
    while (true) {
        if (T[x].leaf) {
            out.push_back({x, true});
            return;
        }
        if (i == 1) {
            out.push_back({x, (D.flag[x] & 1u) != 0});
            return;
        }
        if (D.flag[x] & (1u << (i - 1))) {
            --i;
            continue;
        }
        const int k = D.split[8 * static_cast<size_t>(x) + i - 1];
        collect(T, D, T[x].a, k, out);
        x = T[x].b;
        i -= k;
    }
}

// The eight-slot children of internal node x (its BVH8 node).
void node_slots(const std::vector<TNode>& T, const Collapse& D, int32_t x, std::vector<Slot>& out) {
    out.clear();
    const int k = D.split[8 * static_cast<size_t>(x) + 7];
    collect(T, D, T[x].a, k, out);
    collect(T, D, T[x].b, 8 - k, out);
}

// Triangles of the subtree x in BVH2 leaf order (left before right).
void subtree_tris(const std::vector<TNode>& T, int32_t x, std::vector<int32_t>& out) {
    std::vector<int32_t> st{x};
    while (!st.empty()) {
        const int32_t y = st.back();
        st.pop_back();
        if (T[y].leaf) {
            for (int32_t i = 0; i < T[y].tri_count; ++i) out.push_back(T[y].tri_start + i);
        } else {
            st.push_back(T[y].b);
            st.push_back(T[y].a);
        }
    }
}

// Greedy octant slot assignment: slot bit i set = child centroid toward +axis i.
void assign_slots(const std::vector<TNode>& T, const std::vector<int32_t>& kids, const float* lo,
                  const float* hi, int32_t slot_of[8]) {
    const int k = static_cast<int>(kids.size());
    double c[3], ext[3];
    for (int a = 0; a < 3; ++a) {
        c[a] = 0.5 * (double(lo[a]) + double(hi[a]));
        ext[a] = std::max(1e-30, double(hi[a]) - double(lo[a]));
    }
    struct Pair {
        double score;
        int child, slot;
    };
    std::vector<Pair> pairs;
    for (int i = 0; i < k; ++i) {
        const TNode& n = T[kids[i]];
        double off[3];
        for (int a = 0; a < 3; ++a) off[a] = (0.5 * (double(n.lo[a]) + double(n.hi[a])) - c[a]) / ext[a];
        for (int s = 0; s < 8; ++s) {
            double sc = 0;
            for (int a = 0; a < 3; ++a) sc += ((s >> a) & 1) ? off[a] : -off[a];
            pairs.push_back({sc, i, s});
        }
    }
    std::stable_sort(pairs.begin(), pairs.end(),
                     [](const Pair& x, const Pair& y) { return x.score > y.score; });
    bool child_done[8] = {}, slot_used[8] = {};
    for (int i = 0; i < 8; ++i) slot_of[i] = -1;
    for (const Pair& p : pairs) {
        if (child_done[p.child] || slot_used[p.slot]) continue;
        child_done[p.child] = slot_used[p.slot] = true;
        slot_of[p.child] = p.slot;
    }
}

}  // namespace

void bvh8_decode_child(const uint32_t* node, int s, float lo[3], float hi[3]) {
    const uint8_t* q = reinterpret_cast<const uint8_t*>(node + 8);
    for (int a = 0; a < 3; ++a) {
        const uint32_t e = (node[3] >> (8 * a)) & 0xFFu;
        const double step = std::ldexp(1.0, static_cast<int>(e) - 127);
        const double p = fbits(node[a]);
        lo[a] = static_cast<float>(p + q[a * 8 + s] * step);
        hi[a] = static_cast<float>(p + q[24 + a * 8 + s] * step);
    }
}

bool build_bvh8(int32_t layout, const float* nodes, int64_t n_nodes, const int32_t* tris,
                int64_t n_tris, const float* verts, int64_t n_verts,
                const std::vector<Bvh8Range>& ranges, Bvh8Out& out, std::string& why) {
    const auto t0 = std::chrono::steady_clock::now();
    if (layout != 1 && layout != 2) {
        why = "BVH8 is derived from a BVH2 stack or stackless buffer";
        return false;
    }
    out = Bvh8Out{};
    std::unordered_map<int64_t, int32_t> done;
    std::vector<TNode> T;
    Collapse D;
    std::vector<Slot> slots;
    std::vector<int32_t> leaf_tris;
    for (const Bvh8Range& r : ranges) {
        const int64_t key = (static_cast<int64_t>(r.node_offset) << 32) | uint32_t(r.node_count);
        auto it = done.find(key);
        if (it != done.end()) {
            out.roots.push_back(it->second);
            continue;
        }
        if (r.node_offset < 0 || r.node_count < 1 || r.node_offset + int64_t(r.node_count) > n_nodes) {
            why = "node range outside the node buffer";
            return false;
        }
        if (!recover_tree(layout, nodes, r.node_offset, r.node_count, n_tris, T, why)) return false;
        out.bvh2_nodes += static_cast<int64_t>(T.size());
        const int32_t root = static_cast<int32_t>(out.nodes.size() / kBvh8NodeWords);
        done[key] = root;
        out.roots.push_back(root);
        collapse_costs(T, D);
        // BFS emission: internal children of a node get consecutive node indices.
        std::deque<std::pair<int32_t, int32_t>> q;  // (temp node, bvh8 index)
        out.nodes.resize(out.nodes.size() + kBvh8NodeWords, 0u);
        q.emplace_back(0, root);
        while (!q.empty()) {
            const auto [tn, me] = q.front();
            q.pop_front();
            if (T[tn].leaf) {
                slots.assign(1, Slot{tn, true});  // single-leaf object
            } else {
                node_slots(T, D, tn, slots);
            }
            std::vector<int32_t> kids;
            for (const Slot& sl : slots) kids.push_back(sl.tnode);
            float lo[3], hi[3];
            for (int a = 0; a < 3; ++a) {
                lo[a] = T[kids[0]].lo[a];
                hi[a] = T[kids[0]].hi[a];
                for (size_t i = 1; i < kids.size(); ++i) {
                    lo[a] = std::min(lo[a], T[kids[i]].lo[a]);
                    hi[a] = std::max(hi[a], T[kids[i]].hi[a]);
                }
            }
            int32_t slot_of[8];
            assign_slots(T, kids, lo, hi, slot_of);
            int32_t child_at[8];
            bool leaf_at[8] = {};
            for (int s = 0; s < 8; ++s) child_at[s] = -1;
            for (size_t i = 0; i < kids.size(); ++i) {
                child_at[slot_of[i]] = kids[i];
                leaf_at[slot_of[i]] = slots[i].leaf;
            }

            uint32_t* nd = out.nodes.data() + static_cast<int64_t>(me) * kBvh8NodeWords;
            uint8_t qb[48];
            uint8_t meta[8] = {};
            uint32_t imask = 0;
            uint32_t e_byte[3];
            double step[3];
            for (int a = 0; a < 3; ++a) {
                const double ext = double(hi[a]) - double(lo[a]);
                int e = -126;  // smallest normal step for flat axes
                if (ext > 0) {
                    int x;
                    std::frexp(ext / 255.0, &x);  // ext/255 < 2^x
                    e = std::max(x, -126);
                }
                while (double(lo[a]) + 255.0 * std::ldexp(1.0, e) < double(hi[a])) ++e;
                e_byte[a] = static_cast<uint32_t>(e + 127);
                step[a] = std::ldexp(1.0, e);
                std::memcpy(&nd[a], &lo[a], 4);
            }
            // Large origin relative to the step: the double checks below may round; widen by one.
            bool coarse[3];
            for (int a = 0; a < 3; ++a) coarse[a] = std::fabs(double(lo[a])) / step[a] > 1048576.0;
            // internal children first get consecutive indices (slot order)
            const int32_t child_base = static_cast<int32_t>(out.nodes.size() / kBvh8NodeWords);
            int32_t n_int = 0;
            const int32_t tri_base = static_cast<int32_t>(out.tris.size() / kBvh8TriWords);
            int32_t tri_off = 0;
            std::vector<int32_t> new_internal;
            for (int s = 0; s < 8; ++s) {
                const int32_t c = child_at[s];
                for (int a = 0; a < 3; ++a) {
                    if (c < 0) {
                        qb[a * 8 + s] = 255;
                        qb[24 + a * 8 + s] = 0;
                        continue;
                    }
                    const double p = lo[a];
                    double ql = std::floor((double(T[c].lo[a]) - p) / step[a]);
                    double qh = std::ceil((double(T[c].hi[a]) - p) / step[a]);
                    while (ql > 0 && p + ql * step[a] > double(T[c].lo[a])) ql -= 1;
                    while (qh < 255 && p + qh * step[a] < double(T[c].hi[a])) qh += 1;
                    if (coarse[a]) {
                        ql -= 1;
                        qh += 1;
                    }
                    ql = std::min(255.0, std::max(0.0, ql));
                    qh = std::min(255.0, std::max(0.0, qh));
                    qb[a * 8 + s] = static_cast<uint8_t>(ql);
                    qb[24 + a * 8 + s] = static_cast<uint8_t>(qh);
                }
                if (c < 0) continue;
                if (!leaf_at[s]) {
                    imask |= 1u << s;
                    new_internal.push_back(c);
                    ++n_int;
                } else {
                    leaf_tris.clear();
                    subtree_tris(T, c, leaf_tris);
                    const int32_t cnt = static_cast<int32_t>(leaf_tris.size());
                    if (tri_off + cnt > 32 || cnt > 7) {
                        why = "more than 32 triangles under one BVH8 node";
                        return false;
                    }
                    if (cnt > 0) meta[s] = static_cast<uint8_t>((cnt << 5) | tri_off);
                    for (int32_t i = 0; i < cnt; ++i) {
                        const int32_t t = leaf_tris[i];
                        const int32_t* tr = tris + static_cast<int64_t>(t) * 4;
                        for (int k = 0; k < 3; ++k)
                            if (tr[k] < 0 || tr[k] >= n_verts) {
                                why = "vertex index out of range";
                                return false;
                            }
                        const float* v0 = verts + static_cast<int64_t>(tr[0]) * 8;
                        const float* v1 = verts + static_cast<int64_t>(tr[1]) * 8;
                        const float* v2 = verts + static_cast<int64_t>(tr[2]) * 8;
                        const float e1[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
                        const float e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
                        const float nx = e1[1] * e2[2] - e1[2] * e2[1];
                        const float ny = e1[2] * e2[0] - e1[0] * e2[2];
                        const float nz = e1[0] * e2[1] - e1[1] * e2[0];
                        const float rec[16] = {v0[0], v0[1], v0[2], fbits(uint32_t(t)),
                                               e1[0], e1[1], e1[2], fbits(uint32_t(tr[3])),
                                               e2[0], e2[1], e2[2], 0.0f,
                                               nx, ny, nz, 0.0f};
                        out.tris.insert(out.tris.end(), rec, rec + 16);
                    }
                    tri_off += cnt;
                }
            }
            nd[3] = e_byte[0] | (e_byte[1] << 8) | (e_byte[2] << 16) | (imask << 24);
            nd[4] = static_cast<uint32_t>(n_int ? child_base : 0);
            nd[5] = static_cast<uint32_t>(tri_base);
            std::memcpy(&nd[6], meta, 8);
            std::memcpy(&nd[8], qb, 48);
            out.nodes.resize(out.nodes.size() + static_cast<size_t>(n_int) * kBvh8NodeWords, 0u);
            for (int32_t i = 0; i < n_int; ++i) q.emplace_back(new_internal[i], child_base + i);
        }
    }
    out.n_nodes = static_cast<int64_t>(out.nodes.size() / kBvh8NodeWords);
    out.n_tris = static_cast<int64_t>(out.tris.size() / kBvh8TriWords);
    out.build_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return true;
}

}  // namespace rq
