// Top-level BVH over a scene's entities (host build).
//
// The reference intersects every entity in turn (IntersectScene, Shaders/Intersectors/Include/
// TraverseBVHStack.glsl:337-349): world ray -> object space by the entity's inverse matrix, walk
// of the entity's BVH with the running TMax.  The top level here keeps that loop exactly and only
// skips entities that the ray provably cannot touch:
//
//  * every entity gets a world-space box that encloses everything its object-space walk can
//    touch, widened by a margin that covers the rounding of the object-space ray transform and of
//    the walk's own slab tests (so a ray that misses the widened box has its object-space walk
//    end at the root with nothing found);
//  * the top-level tree splits the entity index range (left child = lower indices) and is stored
//    in pre-order with skip links, so its leaves come out in ascending entity order: candidates
//    are walked in the loop's order, each with the loop's TMax, and results (hits, ties, the
//    any-hit early exit) are those of the plain loop;
//  * a skipped entity's walk would have visited exactly its root node, so its iteration is added
//    to the count (per-entity prefix counts give the number skipped between two candidates);
//  * entities whose walk tests triangles without a box test first (a stack-layout root with a
//    leaf child) or whose transform is singular or not finite are never skipped.
// BVH8 closest-hit queries walk the same tree nearest box first instead (rq_tlas.cuh, near_next):
// their hit is the lexicographic minimum of (t, triangle, entity), which no walk order changes.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace rq {

struct TlasEntity {
    float inverse[16];    // rq_entity.inverse, column-major
    double lo[3], hi[3];  // object-space bounds of everything the entity's walk can box-test
    bool cullable;        // false: always a candidate (infinite box)
    bool opaque;          // alpha >= 0.99 (kept by the ignore-transparent loop)
    bool b8;              // has a BVH8 root (kept by the BVH8 loop)
};

struct TlasOut {
    // 8 floats per node, pre-order: {min.xyz, entity index or -1 (int bits)},
    // {max.xyz, skip link: the node after this subtree, -1 at the end (int bits)}
    std::vector<float> nodes;
    // 4 ints per entity index e in [0, n_ents]: entities before e that are opaque, that have a
    // BVH8 root, that are both; 0
    std::vector<int32_t> prefix;
    float ray_margin = 0.0f;  // per-ray widening = ray_margin * max |origin component|
    int32_t n_nodes = 0, n_cullable = 0;
};

// The margin factor: 2^-14, about 100 times the worst rounding of the transform and slab test.
constexpr double kTlasMargin = 1.0 / 16384.0;
// Scenes with fewer entities keep the plain loop.
constexpr int32_t kTlasMinEntities = 4;

bool build_tlas(const std::vector<TlasEntity>& ents, TlasOut& out, std::string& why);

}  // namespace rq
