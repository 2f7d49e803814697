// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference SAH BVH constructor (Source/Core/BVH/BVHConstructor.cpp of swr06/Candela)
// unmodified, by #including it into this translation unit, and exposes a C entry point that runs
// it on caller-supplied vertex/index arrays.  Only tests/ and the bench's CPU-baseline leg load the
// resulting library (oracle/_ref/librefbvh*.so); the product never does.
//
// The recipe that builds this file is oracle/Makefile.  It needs the reference tree, so it only
// runs where the reference is mounted; the library is a checker, not a product dependency.
//
// What the harness does around the reference code:
//  * resets the reference's file-static counters (BVHConstructor.cpp:58-66) before each build,
//    exactly as BVH::BuildBVH does (BVHConstructor.cpp:955-961, 1036-1042);
//  * calls ConstructHierarchy (stackless, BVHConstructor.cpp:702) or ConstructHierarchy_StackBVH
//    (stack, BVHConstructor.cpp:748) directly, because BuildBVH takes an Object whose Mesh
//    constructor issues OpenGL calls (Mesh.cpp:5-23);
//  * optionally replaces std::random_device (used only for the stackless child swap,
//    BVHConstructor.cpp:389-391, 599-609) by a fixed-seed device so that the swap sequence is
//    reproducible; with UsesStackless = false no random number is drawn at all;
//  * silences the reference's progress printing on std::cout;
//  * frees the pointer tree the reference leaks.
#include <cstdint>
#include <cstring>
#include <random>
#include <sstream>
#include <vector>

// Fixed-seed stand-in for std::random_device.  Declared before the reference TU is included so
// that its `std::random_device dev;` (BVHConstructor.cpp:389) picks this type up.  (The leaf-4
// recipe in oracle/Makefile declares it itself, ahead of the piped reference source.)
#ifndef HARNESS_DEVICE_DECLARED
namespace std {
struct harness_seeded_device {
    static unsigned seed;
    unsigned operator()() { return seed; }
};
}  // namespace std
#define random_device harness_seeded_device
#endif
namespace std {
unsigned harness_seeded_device::seed = 0u;
}  // namespace std

#ifndef REF_BVH_INCLUDED
#include REF_BVH_CPP
#endif

#undef random_device

namespace {

using Candela::Vertex;
namespace RB = Candela::BVH;

void free_tree(RB::Node* n, bool is_root) {
    // Iterative: the reference allocates every child with `new` (BVHConstructor.cpp:558, 566).
    std::vector<RB::Node*> work;
    if (n->LeftChildPtr) work.push_back(n->LeftChildPtr);
    if (n->RightChildPtr) work.push_back(n->RightChildPtr);
    while (!work.empty()) {
        RB::Node* c = work.back();
        work.pop_back();
        if (c->LeftChildPtr) work.push_back(c->LeftChildPtr);
        if (c->RightChildPtr) work.push_back(c->RightChildPtr);
        delete c;
    }
    if (!is_root) delete n;
}

struct RefBuild {
    std::vector<RB::FlattenedNode> stackless;
    std::vector<RB::FlattenedStackNode> stack;
    std::vector<RB::Triangle> tris;
    uint64_t last_node_index = 0;
    uint64_t leaf_count = 0;
    uint64_t split_fails = 0;
    uint32_t max_depth = 0;
};

}  // namespace

extern "C" {

// Runs the reference constructor.
//   layout     : 0 = stack (FlattenedStackNode, 64 B), 1 = stackless (FlattenedNode, 32 B)
//   verts      : n_verts records of 32 bytes (Candela::Vertex, Utils/Vertex.h:7-12)
//   indices    : n_indices vertex indices (3 per triangle); n_indices/3 must be >= 100 because the
//                reference computes `TotalIterations % (n_indices/300)` (BVHConstructor.cpp:387,445)
//   mesh_ids   : one mesh id per triangle (the reference's MeshReferences, BVHConstructor.cpp:983-998)
//   tri_offset : TriangleOffset_ (global triangle index of this object's first triangle)
//   swap_mode  : stackless only.  0 = UsesStackless=false (no random swaps, deterministic);
//                1 = UsesStackless=true with std::random_device seeded by `swap_seed`.
// Returns an opaque handle (nullptr on invalid input).
void* refbvh_build(int layout, const void* verts, int64_t n_verts, const uint32_t* indices,
                   int64_t n_indices, const int32_t* mesh_ids, int32_t tri_offset, int swap_mode,
                   uint32_t swap_seed) {
    if (n_indices % 3 != 0 || n_indices / 3 < 100 || n_verts <= 0) return nullptr;
    const int64_t n_tris = n_indices / 3;
    std::vector<Vertex> V(static_cast<size_t>(n_verts));
    std::memcpy(V.data(), verts, sizeof(Vertex) * static_cast<size_t>(n_verts));
    std::vector<GLuint> I(indices, indices + n_indices);
    std::vector<int> M(static_cast<size_t>(n_tris));
    for (int64_t i = 0; i < n_tris; ++i) M[i] = mesh_ids ? mesh_ids[i] : 0;

    // State reset as in BuildBVH (BVHConstructor.cpp:955-961 / 1036-1042).
    RB::TotalIterations = 0;
    RB::LastNodeIndex = 0;
    RB::LeafNodeCount = 0;
    RB::SplitFails = 0;
    RB::MaxBVHDepth = 0;
    RB::TriangleOffset_ = tri_offset;
    RB::UsesStackless = (layout == 1 && swap_mode == 1);
    std::harness_seeded_device::seed = swap_seed;

    RB::Node* root = new RB::Node;
    root->LeftChildPtr = nullptr;
    root->RightChildPtr = nullptr;
    root->StartIndex = 0;
    root->Length = static_cast<RB::uint>(n_tris);

    auto* out = new RefBuild;
    std::stringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    if (layout == 0) {
        if (n_tris <= 2) {  // the stack flattener dereferences a null child for a leaf root
            std::cout.rdbuf(old);
            delete root;
            delete out;
            return nullptr;
        }
        RB::ConstructHierarchy_StackBVH(V, I, out->stack, out->tris, M, root);
    } else {
        RB::ConstructHierarchy(V, I, out->stackless, out->tris, M, root);
    }
    std::cout.rdbuf(old);
    out->last_node_index = RB::LastNodeIndex;
    out->leaf_count = RB::LeafNodeCount;
    out->split_fails = RB::SplitFails;
    out->max_depth = RB::MaxBVHDepth;
    free_tree(root, false);
    return out;
}

// Sizes of the buffers held by a handle.  node_bytes is 64 (stack) or 32 (stackless).
void refbvh_info(void* h, int64_t* n_nodes, int64_t* n_tris, int64_t* last_node_index,
                 int64_t* leaf_count, int64_t* split_fails, int64_t* max_depth) {
    auto* b = static_cast<RefBuild*>(h);
    *n_nodes = b->stack.empty() ? static_cast<int64_t>(b->stackless.size())
                                : static_cast<int64_t>(b->stack.size());
    *n_tris = static_cast<int64_t>(b->tris.size());
    *last_node_index = static_cast<int64_t>(b->last_node_index);
    *leaf_count = static_cast<int64_t>(b->leaf_count);
    *split_fails = static_cast<int64_t>(b->split_fails);
    *max_depth = static_cast<int64_t>(b->max_depth);
}

void refbvh_copy(void* h, void* nodes_out, void* tris_out) {
    auto* b = static_cast<RefBuild*>(h);
    if (!b->stack.empty())
        std::memcpy(nodes_out, b->stack.data(), b->stack.size() * sizeof(RB::FlattenedStackNode));
    else
        std::memcpy(nodes_out, b->stackless.data(),
                    b->stackless.size() * sizeof(RB::FlattenedNode));
    std::memcpy(tris_out, b->tris.data(), b->tris.size() * sizeof(RB::Triangle));
}

void refbvh_free(void* h) { delete static_cast<RefBuild*>(h); }

int refbvh_leaf_cap() { return RB::MAX_TRIANGLES_PER_LEAF; }

}  // extern "C"
