// BVH8 with 8-bit quantised child boxes, derived from the reference's flattened BVH2 buffers.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace rq {

// One BVH8 node = 80 bytes = 5 x uint4 (20 words):
//   w[0..2]  origin p (float), w[3] = ex | ey << 8 | ez << 16 | imask << 24
//            (e* = biased float exponents of the per-axis grid step 2^(e-127); imask bit s = slot
//            s holds an internal child)
//   w[4]     child_base: node index of the first internal child (internal children contiguous,
//            in slot order)
//   w[5]     tri_base: first record of this node's leaf triangles (contiguous, slot order)
//   w[6..7]  meta[8]: slot s: 0 = empty or internal, else leaf = count << 5 | offset with
//            offset < 32 relative to tri_base and 1 <= count <= 4 (never 0 for a leaf)
//   w[8..19] quantised boxes: qlo_x[8] qlo_y[8] qlo_z[8] qhi_x[8] qhi_y[8] qhi_z[8] (bytes);
//            child box = p + q * 2^(e-127) per axis, rounded outward so it contains the FP32 box
// Children are placed in slots by octant (slot bit i set = child lies toward +axis i), so a ray
// visits slots in the order slot ^ octant(dir) for an approximately front-to-back walk.
constexpr int kBvh8NodeWords = 20;

// Triangle record (64 bytes = 4 x float4) in BVH8 leaf order:
//   {v0.xyz, tri}, {e1.xyz, mesh}, {e2.xyz, 0}, {n.xyz, 0}
// e1 = v1 - v0, e2 = v2 - v0, n = cross(e1, e2) computed with the same IEEE binary32 operations as
// RayTriangle (TraverseBVHStack.glsl:89-93), so a test on these records gives bit-identical t, u, v;
// `tri` is the triangle's index in the reference triangle buffer.
constexpr int kBvh8TriWords = 16;

struct Bvh8Range {
    int32_t node_offset, node_count;  // an object's BVH2 node range (BVHEntity.NodeOffset/Count)
};

struct Bvh8Out {
    std::vector<uint32_t> nodes;     // kBvh8NodeWords per node
    std::vector<float> tris;         // kBvh8TriWords per record
    std::vector<int32_t> roots;      // BVH8 root node per input range (-1: empty object)
    int64_t n_nodes = 0, n_tris = 0;
    int64_t bvh2_nodes = 0;          // BVH2 nodes collapsed
    double build_ms = 0.0;
};

// layout: 1 = stack (64 B nodes), 2 = stackless (32 B nodes), as in rq_layout.
// Returns false with `why` set on malformed input or leaves with more than 4 triangles.
bool build_bvh8(int32_t layout, const float* nodes, int64_t n_nodes, const int32_t* tris,
                int64_t n_tris, const float* vert_records, int64_t n_verts,
                const std::vector<Bvh8Range>& ranges, Bvh8Out& out, std::string& why);

// Decodes child slot s of node `node` (20 words) into the float box the kernels test against.
void bvh8_decode_child(const uint32_t* node, int s, float lo[3], float hi[3]);

}  // namespace rq
