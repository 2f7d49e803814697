// Host-side SAH BVH construction (native C++, multi-threaded) producing the reference's flattened
// buffer formats byte for byte.  See bvh_build.cpp for the algorithm and its reference lines.
#pragma once
#include <cstdint>
#include <vector>

namespace rq {

struct BuildInput {
    const float* vert_records;  // 8 words per vertex (32-byte Candela::Vertex); xyz = position
    int64_t n_verts;
    const uint32_t* indices;    // 3 per triangle
    int64_t n_tris;
    const int32_t* mesh_ids;    // one per triangle (nullable -> 0)
    int32_t tri_offset;         // TriangleOffset_: global index of this object's first triangle
    int32_t leaf_size;          // MAX_TRIANGLES_PER_LEAF (reference: 2; 1..15)
    int32_t layout;             // 0 = stack (64 B nodes), 1 = stackless (32 B nodes)
    int32_t swap_children;      // stackless only: reference OPTIMIZE_FOR_AVERAGE_CASE child swap
    uint32_t swap_seed;         // seed of the mt19937 that drives the swap
    int32_t n_threads;          // 0 = hardware concurrency
};

struct BuildOutput {
    std::vector<float> nodes;      // 16 (stack) or 8 (stackless) floats per node
    int64_t n_nodes = 0;           // array length (the reference's LastNodeIndex + 1)
    int64_t n_nodes_used = 0;      // stack layout: internal-node count; stackless: n_nodes
    std::vector<int32_t> tris;     // 4 ints per triangle {i0, i1, i2, mesh}
    int64_t leaf_count = 0;
    int64_t split_fails = 0;
    int64_t max_depth = 0;         // deepest tree level
    double build_ms = 0.0;
};

// Returns 0 on success, or a negative code: -1 invalid arguments.
int build_bvh(const BuildInput& in, BuildOutput& out);

}  // namespace rq
