// Example host program for the C++ mirror of Candela's RayIntersector<T> (include/rq_intersector.hpp).
//
// Reads objects (raw vertex / index files), adds them with AddObject, pushes translated entities,
// and writes the global buffers the reference would upload to its SSBOs.  With --gpu it uploads the
// scene (BufferData) and writes the closest-hit and any-hit results for a ray file, and the
// collision records for a box file when one is present.
//
//   rq_intersector_example <stack|stackless> <input dir> <output dir> [--gpu]
//
// Input dir: objects.txt ("<count>" then per object "<id> <mesh number>"), verts_<k>.bin
// (32-byte rq_vertex records), idx_<k>.bin (uint32, 3 per triangle), entities.txt (per line
// "<object id> <tx> <ty> <tz> <translucency>"), rays.bin (32-byte rq_ray records, --gpu only),
// boxes.bin (optional, 32-byte rq_box records, --gpu only).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "rq_intersector.hpp"

namespace {

template <class T>
std::vector<T> read_raw(const std::string& path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) throw std::runtime_error("cannot open " + path);
    const std::streamsize n = f.tellg();
    f.seekg(0);
    std::vector<T> v(static_cast<size_t>(n) / sizeof(T));
    f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
    return v;
}

template <class T>
void write_raw(const std::string& path, const std::vector<T>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}

template <class NodeT>
int run(const std::string& in, const std::string& out, bool gpu) {
    rq::RayIntersector<NodeT> ri;
    std::ifstream objs(in + "/objects.txt");
    int count = 0;
    objs >> count;
    for (int k = 0; k < count; ++k) {
        rq::Object o;
        rq::Mesh m;
        objs >> o.id >> m.mesh_number;
        m.vertices = read_raw<rq_vertex>(in + "/verts_" + std::to_string(k) + ".bin");
        m.indices = read_raw<uint32_t>(in + "/idx_" + std::to_string(k) + ".bin");
        o.meshes.push_back(std::move(m));
        ri.AddObject(o);
    }
    std::ifstream ents(in + "/entities.txt");
    std::string line;
    while (std::getline(ents, line)) {
        if (line.empty()) continue;
        std::istringstream ls(line);
        int id;
        float tx, ty, tz, tr;
        ls >> id >> tx >> ty >> tz >> tr;
        rq::Mat4 model;
        model.m[12] = tx;
        model.m[13] = ty;
        model.m[14] = tz;
        ri.PushEntity(id, model, 0.0f, tr);
    }
    ri.BufferEntities();
    write_raw(out + "/nodes.bin", ri.m_BVHNodes);
    write_raw(out + "/tris.bin", ri.m_BVHTriangles);
    write_raw(out + "/verts.bin", ri.m_BVHVertices);
    write_raw(out + "/ents.bin", ri.m_BVHEntities);
    if (gpu) {
        rq::Context ctx(0);
        ri.BufferData(ctx);
        const std::vector<rq_ray> rays = read_raw<rq_ray>(in + "/rays.bin");
        write_raw(out + "/hits.bin", ri.Intersect(rays));
        write_raw(out + "/occ.bin", ri.Occluded(rays));
        if (std::ifstream(in + "/boxes.bin").good())
            write_raw(out + "/coll.bin", ri.Collide(read_raw<rq_box>(in + "/boxes.bin")));
    }
    std::cout << "objects " << count << " nodes " << ri.m_BVHNodes.size() << " triangles "
              << ri.m_BVHTriangles.size() << " entities " << ri.m_BVHEntities.size() << "\n";
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::cerr << "usage: rq_intersector_example <stack|stackless> <in> <out> [--gpu]\n";
        return 2;
    }
    const std::string layout = argv[1], in = argv[2], out = argv[3];
    const bool gpu = argc > 4 && std::string(argv[4]) == "--gpu";
    try {
        return layout == "stack" ? run<rq_node_stack>(in, out, gpu) : run<rq_node_stackless>(in, out, gpu);
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
}
