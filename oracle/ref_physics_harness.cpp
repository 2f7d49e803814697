// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's host collision walk (Source/Core/Physics.cpp of swr06/Candela:
// AABBAABBOverlap, BoxTriangleOverlap, CollideBVH, CollidePoint, CollideBox) and exposes
// Physics::CollideBox to the tests, which pin the collision restatement in rq_oracle.cpp against it.
//
// The recipe is oracle/Makefile: it pipes Physics.cpp without its first line (`#include
// "Physics.h"`) into the compiler after this file, so nothing is copied or modified on disk.
// Physics.h would pull in BVH/Intersector.h, whose RayIntersector<T> owns OpenGL objects; the
// walk only reads the intersector's four host buffers, so this file declares a RayIntersector<T>
// holding exactly those (m_BVHNodes, m_BVHVertices, m_BVHTriangles, m_BVHEntities) and the
// BVHEntity record and StacklessTraversalNode alias of Intersector.h:39-49, with the reference
// types (FlattenedNode, Triangle, Vertex) from BVH/BVHConstructor.h.
#include <cstdint>
#include <cstring>
#include <functional>
#include <vector>

#include "BVH/BVHConstructor.h"

namespace Candela {
namespace BVH {
typedef FlattenedNode StacklessTraversalNode;  // Intersector.h:39
}

struct BVHEntity {  // Intersector.h:43-49
    glm::mat4 ModelMatrix;
    glm::mat4 InverseMatrix;
    int NodeOffset;
    int NodeCount;
    int Data[14];
};

template <typename T>
class RayIntersector {
public:
    std::vector<T> m_BVHNodes;
    std::vector<Vertex> m_BVHVertices;
    std::vector<BVH::Triangle> m_BVHTriangles;
    std::vector<BVHEntity> m_BVHEntities;
};

namespace Physics {
bool CollideBox(const glm::vec3& Min, const glm::vec3& Max, RayIntersector<BVH::StacklessTraversalNode>& Intersector);
}
}  // namespace Candela

static_assert(sizeof(Candela::BVH::FlattenedNode) == 32, "FlattenedNode layout");
static_assert(sizeof(Candela::BVH::Triangle) == 16, "Triangle layout");
static_assert(sizeof(Candela::Vertex) == 32, "Vertex layout");
static_assert(sizeof(Candela::BVHEntity) == 192, "BVHEntity layout");

// Physics::CollideBox for n world-space boxes ({min.xyzw, max.xyzw} floats) over a stackless scene
// given as the reference's global buffers; out[i] = 1 when box i collides.  (CollideBox itself is
// compiled from Physics.cpp, which the recipe appends to this file.)
extern "C" void ref_collide_boxes(const void* nodes, int64_t n_nodes, const void* tris, int64_t n_tris,
                                  const void* verts, int64_t n_verts, const void* ents, int32_t n_ents,
                                  const float* boxes, int64_t n, uint8_t* out) {
    Candela::RayIntersector<Candela::BVH::StacklessTraversalNode> ri;
    ri.m_BVHNodes.resize(n_nodes);
    std::memcpy(static_cast<void*>(ri.m_BVHNodes.data()), nodes, 32 * n_nodes);
    ri.m_BVHTriangles.resize(n_tris);
    std::memcpy(static_cast<void*>(ri.m_BVHTriangles.data()), tris, 16 * n_tris);
    ri.m_BVHVertices.resize(n_verts);
    std::memcpy(static_cast<void*>(ri.m_BVHVertices.data()), verts, 32 * n_verts);
    ri.m_BVHEntities.resize(n_ents);
    std::memcpy(static_cast<void*>(ri.m_BVHEntities.data()), ents, 192 * static_cast<size_t>(n_ents));
    for (int64_t i = 0; i < n; ++i) {
        const float* b = boxes + 8 * i;
        out[i] = Candela::Physics::CollideBox(glm::vec3(b[0], b[1], b[2]), glm::vec3(b[4], b[5], b[6]), ri) ? 1 : 0;
    }
}

#line 2 "Physics.cpp"
