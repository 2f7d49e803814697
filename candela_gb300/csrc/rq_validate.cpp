#include "rq_validate.h"

#include <cstring>
#include <set>
#include <utility>

namespace rq {
namespace {

inline int32_t bits(float f) {
    int32_t i;
    std::memcpy(&i, &f, 4);
    return i;
}

bool leaf_ok(int32_t w, int64_t n_tris) {
    if (w < 0) return false;
    const int64_t start = w >> 4, len = w & 0xF;
    return start + len <= n_tris;
}

}  // namespace

bool validate_entities(int32_t layout, const float* nodes, int64_t n_nodes, int64_t n_tris,
                       const rq_entity* ents, int32_t n_ents, std::string& why) {
    if (n_ents < 0 || (n_ents > 0 && !ents)) {
        why = "entity array is NULL or n_ents < 0";
        return false;
    }
    std::set<std::pair<int32_t, int32_t>> done;
    const int stride = layout == RQ_LAYOUT_BVH2_STACK ? 16 : 8;
    for (int32_t e = 0; e < n_ents; ++e) {
        const int32_t off = ents[e].node_offset, cnt = ents[e].node_count;
        if (off < 0 || cnt < 1 || static_cast<int64_t>(off) + cnt > n_nodes) {
            why = "entity " + std::to_string(e) + ": node range outside the node buffer";
            return false;
        }
        if (!done.insert({off, cnt}).second) continue;
        for (int32_t j = 0; j < cnt; ++j) {
            const float* nd = nodes + static_cast<int64_t>(off + j) * stride;
            const std::string where =
                "entity " + std::to_string(e) + " node " + std::to_string(j) + ": ";
            if (layout == RQ_LAYOUT_BVH2_STACK) {
                for (int s = 0; s < 2; ++s) {
                    const int32_t w = bits(nd[s * 8 + 3]);
                    if (w == -1) {
                        const int32_t link = bits(nd[s * 8 + 7]);
                        if (link < 0 || link >= cnt) {
                            why = where + "child link out of range";
                            return false;
                        }
                    } else if (!leaf_ok(w, n_tris)) {
                        why = where + "leaf triangle range out of bounds";
                        return false;
                    }
                }
            } else {
                const int32_t w = bits(nd[3]);
                const int32_t esc = bits(nd[7]);
                if (w == -1) {
                    if (j + 1 >= cnt) {
                        why = where + "internal node has no successor";
                        return false;
                    }
                } else if (!leaf_ok(w, n_tris)) {
                    why = where + "leaf triangle range out of bounds";
                    return false;
                }
                if (esc != -1 && (esc < 0 || esc >= cnt)) {
                    why = where + "escape link out of range";
                    return false;
                }
            }
        }
    }
    return true;
}

bool validate_scene(int32_t layout, const rq_vertex* verts, int64_t n_verts, const rq_triangle* tris,
                    int64_t n_tris, const void* nodes, int64_t n_nodes, const rq_entity* ents,
                    int32_t n_ents, std::string& why) {
    if (layout != RQ_LAYOUT_BVH2_STACK && layout != RQ_LAYOUT_BVH2_STACKLESS) {
        why = "layout must be BVH2_STACK or BVH2_STACKLESS";
        return false;
    }
    if (!verts || !tris || !nodes || n_verts <= 0 || n_tris <= 0 || n_nodes <= 0) {
        why = "empty or NULL vertex/triangle/node buffer";
        return false;
    }
    if (n_tris >= (int64_t(1) << 27) || n_verts >= (int64_t(1) << 31) ||
        n_nodes >= (int64_t(1) << 31)) {
        why = "buffer too large for 32-bit packed indices";
        return false;
    }
    for (int64_t t = 0; t < n_tris; ++t)
        for (int k = 0; k < 3; ++k) {
            const int32_t v = tris[t].packed[k];
            if (v < 0 || v >= n_verts) {
                why = "triangle " + std::to_string(t) + ": vertex index out of range";
                return false;
            }
        }
    return validate_entities(layout, static_cast<const float*>(nodes), n_nodes, n_tris, ents,
                             n_ents, why);
}

}  // namespace rq
