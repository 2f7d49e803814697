// rq_intersector.hpp — C++ host mirror of Candela's RayIntersector<T> over the C ABI (rq.h).
//
// Replaces Source/Core/BVH/Intersector.h:60-451 for the ray-query path: the same member names and
// call order (AddObject -> PushEntity/PushEntities -> BufferEntities -> BufferData -> queries),
// the same global buffers (m_BVHNodes, m_BVHVertices, m_BVHTriangles, m_BVHEntities), the same
// object bookkeeping (node / triangle / vertex offsets per object id), with the OpenGL SSBO upload
// replaced by a device scene and the GLSL dispatch by rq_closest / rq_anyhit / rq_gi_frame.
// Errors throw rq::Error (the reference throws C strings, Intersector.h:147, 204).
//
// NodeT is rq_node_stack (RayIntersector<FlattenedStackNode>) or rq_node_stackless
// (RayIntersector<FlattenedNode>).  Header-only; link with librq.so.
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "rq.h"

namespace rq {

struct Error : std::runtime_error {
    rq_status status;
    Error(rq_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(rq_status s, const rq_ctx* ctx = nullptr) {
    if (s != RQ_OK) {
        const char* m = rq_last_error(ctx);
        throw Error(s, std::string(rq_status_string(s)) + ": " + (m ? m : ""));
    }
}

// One mesh of an object: vertices, vertex indices (3 per triangle), global mesh number
// (Mesh::GlobalMeshNumber).
struct Mesh {
    std::vector<rq_vertex> vertices;
    std::vector<uint32_t> indices;
    int32_t mesh_number = 0;
};

// An object (Candela::Object): an id and its meshes.
struct Object {
    int32_t id = 0;
    std::vector<Mesh> meshes;
};

// The reference's _ObjectData (Intersector.h:51-56).
struct ObjectData {
    int32_t triangle_offset = 0, vertices_offset = 0, node_offset = 0, node_count = 0;
};

// A column-major 4x4 matrix (glm::mat4 memory layout).
struct Mat4 {
    float m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
};

// Inverse of a column-major 4x4 matrix (cofactor expansion, double precision).
inline Mat4 inverse(const Mat4& a) {
    const float* m = a.m;
    double inv[16];
    inv[0] = double(m[5]) * m[10] * m[15] - double(m[5]) * m[11] * m[14] - double(m[9]) * m[6] * m[15] +
             double(m[9]) * m[7] * m[14] + double(m[13]) * m[6] * m[11] - double(m[13]) * m[7] * m[10];
    inv[4] = -double(m[4]) * m[10] * m[15] + double(m[4]) * m[11] * m[14] + double(m[8]) * m[6] * m[15] -
             double(m[8]) * m[7] * m[14] - double(m[12]) * m[6] * m[11] + double(m[12]) * m[7] * m[10];
    inv[8] = double(m[4]) * m[9] * m[15] - double(m[4]) * m[11] * m[13] - double(m[8]) * m[5] * m[15] +
             double(m[8]) * m[7] * m[13] + double(m[12]) * m[5] * m[11] - double(m[12]) * m[7] * m[9];
    inv[12] = -double(m[4]) * m[9] * m[14] + double(m[4]) * m[10] * m[13] + double(m[8]) * m[5] * m[14] -
              double(m[8]) * m[6] * m[13] - double(m[12]) * m[5] * m[10] + double(m[12]) * m[6] * m[9];
    inv[1] = -double(m[1]) * m[10] * m[15] + double(m[1]) * m[11] * m[14] + double(m[9]) * m[2] * m[15] -
             double(m[9]) * m[3] * m[14] - double(m[13]) * m[2] * m[11] + double(m[13]) * m[3] * m[10];
    inv[5] = double(m[0]) * m[10] * m[15] - double(m[0]) * m[11] * m[14] - double(m[8]) * m[2] * m[15] +
             double(m[8]) * m[3] * m[14] + double(m[12]) * m[2] * m[11] - double(m[12]) * m[3] * m[10];
    inv[9] = -double(m[0]) * m[9] * m[15] + double(m[0]) * m[11] * m[13] + double(m[8]) * m[1] * m[15] -
             double(m[8]) * m[3] * m[13] - double(m[12]) * m[1] * m[11] + double(m[12]) * m[3] * m[9];
    inv[13] = double(m[0]) * m[9] * m[14] - double(m[0]) * m[10] * m[13] - double(m[8]) * m[1] * m[14] +
              double(m[8]) * m[2] * m[13] + double(m[12]) * m[1] * m[10] - double(m[12]) * m[2] * m[9];
    inv[2] = double(m[1]) * m[6] * m[15] - double(m[1]) * m[7] * m[14] - double(m[5]) * m[2] * m[15] +
             double(m[5]) * m[3] * m[14] + double(m[13]) * m[2] * m[7] - double(m[13]) * m[3] * m[6];
    inv[6] = -double(m[0]) * m[6] * m[15] + double(m[0]) * m[7] * m[14] + double(m[4]) * m[2] * m[15] -
             double(m[4]) * m[3] * m[14] - double(m[12]) * m[2] * m[7] + double(m[12]) * m[3] * m[6];
    inv[10] = double(m[0]) * m[5] * m[15] - double(m[0]) * m[7] * m[13] - double(m[4]) * m[1] * m[15] +
              double(m[4]) * m[3] * m[13] + double(m[12]) * m[1] * m[7] - double(m[12]) * m[3] * m[5];
    inv[14] = -double(m[0]) * m[5] * m[14] + double(m[0]) * m[6] * m[13] + double(m[4]) * m[1] * m[14] -
              double(m[4]) * m[2] * m[13] - double(m[12]) * m[1] * m[6] + double(m[12]) * m[2] * m[5];
    inv[3] = -double(m[1]) * m[6] * m[11] + double(m[1]) * m[7] * m[10] + double(m[5]) * m[2] * m[11] -
             double(m[5]) * m[3] * m[10] - double(m[9]) * m[2] * m[7] + double(m[9]) * m[3] * m[6];
    inv[7] = double(m[0]) * m[6] * m[11] - double(m[0]) * m[7] * m[10] - double(m[4]) * m[2] * m[11] +
             double(m[4]) * m[3] * m[10] + double(m[8]) * m[2] * m[7] - double(m[8]) * m[3] * m[6];
    inv[11] = -double(m[0]) * m[5] * m[11] + double(m[0]) * m[7] * m[9] + double(m[4]) * m[1] * m[11] -
              double(m[4]) * m[3] * m[9] - double(m[8]) * m[1] * m[7] + double(m[8]) * m[3] * m[5];
    inv[15] = double(m[0]) * m[5] * m[10] - double(m[0]) * m[6] * m[9] - double(m[4]) * m[1] * m[10] +
              double(m[4]) * m[2] * m[9] + double(m[8]) * m[1] * m[6] - double(m[8]) * m[2] * m[5];
    const double det = double(m[0]) * inv[0] + double(m[1]) * inv[4] + double(m[2]) * inv[8] +
                       double(m[3]) * inv[12];
    if (det == 0.0) throw Error(RQ_EINVAL, "singular entity matrix");
    Mat4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = static_cast<float>(inv[i] / det);
    return r;
}

// Owns an rq_ctx (one per host thread).
class Context {
  public:
    explicit Context(int device = 0) { check(rq_create(device, &ctx_)); }
    ~Context() { rq_destroy(ctx_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    rq_ctx* get() const { return ctx_; }

  private:
    rq_ctx* ctx_ = nullptr;
};

template <typename NodeT>
class RayIntersector {
    static_assert(std::is_same<NodeT, rq_node_stack>::value || std::is_same<NodeT, rq_node_stackless>::value,
                  "RayIntersector<T>: T must be rq_node_stack or rq_node_stackless");

  public:
    static constexpr rq_layout kLayout =
        std::is_same<NodeT, rq_node_stack>::value ? RQ_LAYOUT_BVH2_STACK : RQ_LAYOUT_BVH2_STACKLESS;

    explicit RayIntersector(rq_build_opts opts = rq_build_opts{}) : opts_(opts) {}
    ~RayIntersector() {
        if (scene_) rq_scene_destroy(scene_);
    }
    RayIntersector(const RayIntersector&) = delete;
    RayIntersector& operator=(const RayIntersector&) = delete;

    // AddObject (Intersector.h:169-198): merges the object's meshes (BVHConstructor.cpp:981-1002),
    // builds its BVH with rq_build_bvh, appends the buffers and rebases vertex indices.
    void AddObject(const Object& object) {
        std::vector<rq_vertex> verts;
        std::vector<uint32_t> idx;
        std::vector<int32_t> mesh_ids;
        uint32_t offset = 0;
        for (const Mesh& m : object.meshes) {
            for (size_t x = 0; x < m.indices.size(); ++x) {
                idx.push_back(m.indices[x] + offset);
                if (x % 3 == 0) mesh_ids.push_back(m.mesh_number);
            }
            verts.insert(verts.end(), m.vertices.begin(), m.vertices.end());
            offset += static_cast<uint32_t>(m.vertices.size());
        }
        ObjectData& od = m_ObjectData[object.id];
        od.node_offset = static_cast<int32_t>(m_BVHNodes.size());
        od.triangle_offset = static_cast<int32_t>(m_BVHTriangles.size());
        od.vertices_offset = static_cast<int32_t>(m_BVHVertices.size());
        rq_bvh* bvh = nullptr;
        check(rq_build_bvh(verts.data(), static_cast<int64_t>(verts.size()), idx.data(),
                           static_cast<int64_t>(idx.size()), mesh_ids.data(),
                           static_cast<int32_t>(m_BVHTriangles.size()), kLayout, &opts_, &bvh));
        const void* nodes = nullptr;
        const rq_triangle* tris = nullptr;
        int64_t n_nodes = 0, n_tris = 0;
        check(rq_bvh_nodes(bvh, &nodes, &n_nodes));
        check(rq_bvh_triangles(bvh, &tris, &n_tris));
        const NodeT* nb = static_cast<const NodeT*>(nodes);
        m_BVHNodes.insert(m_BVHNodes.end(), nb, nb + n_nodes);
        od.node_count = static_cast<int32_t>(n_nodes);
        for (int64_t i = 0; i < n_tris; ++i) {
            rq_triangle t = tris[i];
            for (int k = 0; k < 3; ++k) t.packed[k] += static_cast<int32_t>(m_IndexOffset);
            m_BVHTriangles.push_back(t);
        }
        rq_bvh_free(bvh);
        m_BVHVertices.insert(m_BVHVertices.end(), verts.begin(), verts.end());
        m_IndexOffset += static_cast<uint32_t>(verts.size());
    }

    // PushEntity (Intersector.h:200-216).
    void PushEntity(int32_t object_id, const Mat4& model = Mat4{}, float emissive = 0.0f,
                    float translucency = 0.0f) {
        auto it = m_ObjectData.find(object_id);
        if (it == m_ObjectData.end())
            throw Error(RQ_EINVAL, "Trying to push entity whose parent object hasn't been added to global BVH");
        rq_entity e{};
        std::memcpy(e.model, model.m, sizeof(e.model));
        const Mat4 inv = inverse(model);
        std::memcpy(e.inverse, inv.m, sizeof(e.inverse));
        e.node_offset = it->second.node_offset;
        e.node_count = it->second.node_count;
        const float alpha = 1.0f - translucency;
        std::memcpy(&e.data[0], &emissive, 4);
        std::memcpy(&e.data[1], &alpha, 4);
        m_Entities.push_back(e);
    }

    // BufferEntities (Intersector.h:226-239).
    void BufferEntities() {
        m_BVHEntities = m_Entities;
        m_Entities.clear();
        if (scene_)
            check(rq_scene_set_entities(scene_, m_BVHEntities.data(),
                                        static_cast<int32_t>(m_BVHEntities.size())),
                  ctx_);
    }

    // BufferData (Intersector.h:321-351): uploads the global buffers to the device.
    void BufferData(Context& ctx, bool clear_cpu_data = false) {
        if (scene_) rq_scene_destroy(scene_);
        scene_ = nullptr;
        ctx_ = ctx.get();
        check(rq_scene_create(ctx_, kLayout, m_BVHVertices.data(), static_cast<int64_t>(m_BVHVertices.size()),
                              m_BVHTriangles.data(), static_cast<int64_t>(m_BVHTriangles.size()),
                              m_BVHNodes.data(), static_cast<int64_t>(m_BVHNodes.size()), m_BVHEntities.data(),
                              static_cast<int32_t>(m_BVHEntities.size()), &scene_),
              ctx_);
        if (clear_cpu_data) {
            m_BVHNodes.clear();
            m_BVHVertices.clear();
            m_BVHTriangles.clear();
        }
    }

    // Closest hit for a batch (the GLSL IntersectRay(o, d, out TUVW, ...)); host vectors.
    std::vector<rq_hit> Intersect(const std::vector<rq_ray>& rays, rq_opts opts = rq_opts{}) const {
        std::vector<rq_hit> hits(rays.size());
        opts.flags |= RQ_FLAG_HOST_BUFFERS;
        check(rq_closest(ctx_, need_scene(), rays.data(), static_cast<int64_t>(rays.size()), hits.data(), &opts,
                         nullptr),
              ctx_);
        return hits;
    }

    // Any hit (float IntersectRay(o, d)).
    std::vector<uint8_t> Occluded(const std::vector<rq_ray>& rays, rq_opts opts = rq_opts{}) const {
        std::vector<uint8_t> occ(rays.size());
        opts.flags |= RQ_FLAG_HOST_BUFFERS;
        check(rq_anyhit(ctx_, need_scene(), rays.data(), static_cast<int64_t>(rays.size()), occ.data(), &opts,
                        nullptr),
              ctx_);
        return occ;
    }

    // Collision queries (Collide.comp): the first {collided, entity, mesh, triangle} per box.
    std::vector<rq_collision> Collide(const std::vector<rq_box>& boxes, rq_opts opts = rq_opts{}) const {
        std::vector<rq_collision> out(boxes.size());
        opts.flags |= RQ_FLAG_HOST_BUFFERS;
        check(rq_collide(ctx_, need_scene(), boxes.data(), static_cast<int64_t>(boxes.size()), out.data(), &opts,
                         nullptr),
              ctx_);
        return out;
    }

    // Physics::CollideBox (Physics.cpp:203-228).
    bool CollideBox(const float min[3], const float max[3]) const {
        rq_box b = {{min[0], min[1], min[2], 1.0f}, {max[0], max[1], max[2], 1.0f}};
        return Collide({b})[0].collided != 0;
    }

    // Physics::CollidePoint (Physics.cpp:176-201): the box point -/+ 0.01.
    bool CollidePoint(const float p[3]) const {
        const float lo[3] = {p[0] - 0.01f, p[1] - 0.01f, p[2] - 0.01f};
        const float hi[3] = {p[0] + 0.01f, p[1] + 0.01f, p[2] + 0.01f};
        return CollideBox(lo, hi);
    }

    rq_scene* scene() const { return scene_; }
    const std::unordered_map<int32_t, ObjectData>& objects() const { return m_ObjectData; }

    std::vector<NodeT> m_BVHNodes;
    std::vector<rq_vertex> m_BVHVertices;
    std::vector<rq_triangle> m_BVHTriangles;
    std::vector<rq_entity> m_BVHEntities;

  private:
    rq_scene* need_scene() const {
        if (!scene_) throw Error(RQ_ESTATE, "BufferData has not been called");
        return scene_;
    }

    rq_build_opts opts_;
    std::vector<rq_entity> m_Entities;
    uint32_t m_IndexOffset = 0;
    std::unordered_map<int32_t, ObjectData> m_ObjectData;
    rq_ctx* ctx_ = nullptr;
    rq_scene* scene_ = nullptr;
};

}  // namespace rq
