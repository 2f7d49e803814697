// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Entry points around the reference's traversal shaders compiled as C++.  The recipe in
// oracle/Makefile builds one translation unit from ref_glsl_prologue.h, then, in namespace
// glsl_stack, the struct declarations and traversal functions of
// Shaders/Intersectors/Include/TraverseBVHStack.glsl (lines 14-52, 75-414, 505-683: RayTriangle,
// RayBounds, ComputeBarycentrics, IntersectBVHStack, IntersectScene, IntersectSceneIgnoreTransparent,
// the occlusion walk, IntersectSceneOcclusion, IntersectRay), then likewise in namespace
// glsl_stackless for TraverseBVHStackless.glsl (lines 14-46, 67-368, 461-580),
// the collision shaders CollideBVHStack.glsl (14-48, 67-326) and CollideBVHStackless.glsl (11-32,
// 51-54, 56-248) in namespaces glsl_collide_stack / glsl_collide_stackless, CosWeightedHemisphere
// of Shaders/Include/Sampling.glsl (lines 1-12) in namespace glsl_sampling, and finally this file.  The shader text is piped through sed (`.xyz` -> `.xyz()`, `out T` /
// `inout T` -> `T&`) and compiled with `in` defined empty; nothing is written to disk but the library
// (oracle/_ref/librefglsl.so).  The SSBOs and uniforms the shaders read become the namespace
// globals below, set per call.  The tests compare the CPU restatement (rq_oracle.cpp) with it.
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// Copies the caller's buffers into arrays with one zero node of padding: the shaders guard the
// node index with `> u_TotalNodes`, so an index equal to the node count passes the guard.
template <class NS_Node, class NS_Tri, class NS_Vert, class NS_Ent>
struct Buffers {
    std::vector<NS_Node> nodes;
    std::vector<NS_Tri> tris;
    std::vector<NS_Vert> verts;
    std::vector<NS_Ent> ents;
    Buffers(const void* n, int64_t nn, const void* t, int64_t nt, const void* v, int64_t nv, const void* e,
            int32_t ne)
        : nodes(nn + 1), tris(nt), verts(nv), ents(ne) {
        std::memset(static_cast<void*>(nodes.data()), 0, sizeof(NS_Node) * (nn + 1));
        std::memcpy(static_cast<void*>(nodes.data()), n, sizeof(NS_Node) * nn);
        std::memcpy(static_cast<void*>(tris.data()), t, sizeof(NS_Tri) * nt);
        std::memcpy(static_cast<void*>(verts.data()), v, sizeof(NS_Vert) * nv);
        std::memcpy(static_cast<void*>(ents.data()), e, sizeof(NS_Ent) * ne);
    }
};

void put_hit(float* o, const glsl::vec4& tuvw, int tri, int mesh, int ent, int iters) {
    o[0] = tuvw.x;
    o[1] = tuvw.y;
    o[2] = tuvw.z;
    o[3] = tuvw.w;
    std::memcpy(o + 4, &tri, 4);
    std::memcpy(o + 5, &mesh, 4);
    std::memcpy(o + 6, &ent, 4);
    std::memcpy(o + 7, &iters, 4);
}

}  // namespace

static_assert(sizeof(glsl_stack::Node) == 64 && sizeof(glsl_stackless::Node) == 32, "node layouts");
static_assert(sizeof(glsl_stack::BVHEntity) == 192 && sizeof(glsl_stack::Vertex) == 32, "record layouts");

// IntersectScene (closest hit; ignore_transparent: IntersectSceneIgnoreTransparent) per ray of
// `rays` (8 floats: origin, tmin, direction, tmax; the shaders use tmin 0 and TMax 1e6 whatever
// the ray says).  out: 8 words per ray, TUVW then the Triangle, Mesh, Entity and Iters outputs
// (-1 where the shader leaves an output unwritten).  stackless selects the shader file.
extern "C" void ref_glsl_closest(int stackless, int ignore_transparent, const void* nodes, int64_t n_nodes,
                                 const void* tris, int64_t n_tris, const void* verts, int64_t n_verts,
                                 const void* ents, int32_t n_ents, const float* rays, int64_t n, float* out) {
    if (!stackless) {
        namespace G = glsl_stack;
        Buffers<G::Node, G::Triangle, G::Vertex, G::BVHEntity> b(nodes, n_nodes, tris, n_tris, verts, n_verts,
                                                                  ents, n_ents);
        G::BVHNodes = b.nodes.data();
        G::BVHTris = b.tris.data();
        G::BVHVertices = b.verts.data();
        G::BVHEntities = b.ents.data();
        G::u_EntityCount = n_ents;
        G::u_TotalNodes = static_cast<int>(n_nodes);
        for (int64_t i = 0; i < n; ++i) {
            const float* r = rays + 8 * i;
            int mesh = -1, tri = -1, ent = -1, iters = -1;
            const glsl::vec4 h = ignore_transparent
                                     ? G::IntersectSceneIgnoreTransparent(glsl::vec3(r[0], r[1], r[2]),
                                                                          glsl::vec3(r[4], r[5], r[6]), mesh, tri, ent,
                                                                          iters)
                                     : G::IntersectScene(glsl::vec3(r[0], r[1], r[2]), glsl::vec3(r[4], r[5], r[6]),
                                                         mesh, tri, ent, iters);
            put_hit(out + 8 * i, h, tri, mesh, ent, iters);
        }
    } else {
        namespace G = glsl_stackless;
        Buffers<G::Node, G::Triangle, G::Vertex, G::BVHEntity> b(nodes, n_nodes, tris, n_tris, verts, n_verts,
                                                                  ents, n_ents);
        G::BVHNodes = b.nodes.data();
        G::BVHTris = b.tris.data();
        G::BVHVertices = b.verts.data();
        G::BVHEntities = b.ents.data();
        G::u_EntityCount = n_ents;
        G::u_TotalNodes = static_cast<int>(n_nodes);
        for (int64_t i = 0; i < n; ++i) {
            const float* r = rays + 8 * i;
            int mesh = -1, tri = -1, ent = -1, iters = -1;
            const glsl::vec4 h = ignore_transparent
                                     ? G::IntersectSceneIgnoreTransparent(glsl::vec3(r[0], r[1], r[2]),
                                                                          glsl::vec3(r[4], r[5], r[6]), mesh, tri, ent,
                                                                          iters)
                                     : G::IntersectScene(glsl::vec3(r[0], r[1], r[2]), glsl::vec3(r[4], r[5], r[6]),
                                                         mesh, tri, ent, iters);
            put_hit(out + 8 * i, h, tri, mesh, ent, iters);
        }
    }
}

// CollideScene (Collide.comp's query; CollideBVHStack.glsl / CollideBVHStackless.glsl) per box
// ({min.xyzw, max.xyzw}): out 4 ints {collided, entity, mesh, triangle}, -1 where unwritten.
template <class NS_Node, class NS_Tri, class NS_Vert, class NS_Ent, class Scene>
static void collide_all(const void* nodes, int64_t n_nodes, const void* tris, int64_t n_tris, const void* verts,
                        int64_t n_verts, const void* ents, int32_t n_ents, const float* boxes, int64_t n,
                        int32_t* out, NS_Node** gn, NS_Tri** gt, NS_Vert** gv, NS_Ent** ge, int* gcount, int* gtotal,
                        Scene scene) {
    Buffers<NS_Node, NS_Tri, NS_Vert, NS_Ent> b(nodes, n_nodes, tris, n_tris, verts, n_verts, ents, n_ents);
    *gn = b.nodes.data();
    *gt = b.tris.data();
    *gv = b.verts.data();
    *ge = b.ents.data();
    *gcount = n_ents;
    *gtotal = static_cast<int>(n_nodes);
    for (int64_t i = 0; i < n; ++i) {
        const float* x = boxes + 8 * i;
        int mesh = -1, tri = -1, ent = -1;
        const bool hit = scene(glsl::vec3(x[0], x[1], x[2]), glsl::vec3(x[4], x[5], x[6]), mesh, tri, ent);
        out[4 * i] = hit ? 1 : 0;
        out[4 * i + 1] = ent;
        out[4 * i + 2] = mesh;
        out[4 * i + 3] = tri;
    }
}

extern "C" void ref_glsl_collide(int stackless, const void* nodes, int64_t n_nodes, const void* tris, int64_t n_tris,
                                 const void* verts, int64_t n_verts, const void* ents, int32_t n_ents,
                                 const float* boxes, int64_t n, int32_t* out) {
    if (!stackless) {
        namespace G = glsl_collide_stack;
        collide_all(nodes, n_nodes, tris, n_tris, verts, n_verts, ents, n_ents, boxes, n, out, &G::BVHNodes,
                    &G::BVHTris, &G::BVHVertices, &G::BVHEntities, &G::u_EntityCount, &G::u_TotalNodes,
                    [](glsl::vec3 a, glsl::vec3 b, int& m, int& t, int& e) { return G::CollideScene(a, b, m, t, e); });
    } else {
        namespace G = glsl_collide_stackless;
        collide_all(nodes, n_nodes, tris, n_tris, verts, n_verts, ents, n_ents, boxes, n, out, &G::BVHNodes,
                    &G::BVHTris, &G::BVHVertices, &G::BVHEntities, &G::u_EntityCount, &G::u_TotalNodes,
                    [](glsl::vec3 a, glsl::vec3 b, int& m, int& t, int& e) { return G::CollideScene(a, b, m, t, e); });
    }
}

// GetData (TraverseBVHStack.glsl:422-455) per hit record (t, u, v, w, tri, mesh, entity, iters)
// with the texture table `refs` (32 bytes per mesh: ModelColor, Albedo texture index, ...): out 8
// floats per hit, Normal, Albedo, Emissivity, Alpha.  texture() is replaced by (u, v, texture
// index), so Albedo reports the UV GetData samples at for textured meshes.
extern "C" void ref_glsl_getdata(const void* tris, int64_t n_tris, const void* verts, int64_t n_verts,
                                 const void* ents, int32_t n_ents, const void* refs, int32_t n_refs,
                                 const float* hits, int64_t n, float* out) {
    namespace G = glsl_stack;
    std::vector<G::Triangle> t(n_tris);
    std::vector<G::Vertex> v(n_verts);
    std::vector<G::BVHEntity> e(n_ents);
    std::vector<G::TextureReferences> r(n_refs);
    std::memcpy(static_cast<void*>(t.data()), tris, sizeof(G::Triangle) * n_tris);
    std::memcpy(static_cast<void*>(v.data()), verts, sizeof(G::Vertex) * n_verts);
    std::memcpy(static_cast<void*>(e.data()), ents, sizeof(G::BVHEntity) * n_ents);
    std::memcpy(static_cast<void*>(r.data()), refs, sizeof(G::TextureReferences) * n_refs);
    G::BVHTris = t.data();
    G::BVHVertices = v.data();
    G::BVHEntities = e.data();
    G::BVHTextureReferences = r.data();
    for (int k = 0; k < 512; ++k) G::Textures[k].id = k;
    for (int64_t i = 0; i < n; ++i) {
        const float* h = hits + 8 * i;
        int tri, mesh, ent;
        std::memcpy(&tri, h + 4, 4);
        std::memcpy(&mesh, h + 5, 4);
        std::memcpy(&ent, h + 6, 4);
        glsl::vec3 normal(0.0f), albedo(0.0f);
        float em = 0.0f, alpha = 0.0f;
        G::GetData(glsl::vec4(h[0], h[1], h[2], h[3]), mesh, tri, ent, normal, albedo, em, alpha);
        float* o = out + 8 * i;
        o[0] = normal.x;
        o[1] = normal.y;
        o[2] = normal.z;
        o[3] = albedo.x;
        o[4] = albedo.y;
        o[5] = albedo.z;
        o[6] = em;
        o[7] = alpha;
    }
}

// hash2() of the specular shader (SpecularTrace.glsl:71-75) is a fract(sin) sequence whose values
// depend on the driver's sin; here it draws the engine's counter-based samples instead (pcg_hash,
// Jarzynski & Olano 2020: key = hash(hash(hash(seed) + sample) + dimension), u = (key >> 8) / 2^24),
// dimensions 2k and 2k+1 on the k-th call, so both sides consume the same numbers.
namespace glsl_specular {
uint32_t g_seed = 0, g_sample = 0, g_dim = 0;
static uint32_t pcg(uint32_t x) {
    const uint32_t state = x * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
static float u01(uint32_t dim) {
    return static_cast<float>(pcg(pcg(pcg(g_seed) + g_sample) + dim) >> 8) * (1.0f / 16777216.0f);
}
glsl::vec2 hash2() {
    const glsl::vec2 r{u01(g_dim), u01(g_dim + 1)};
    g_dim += 2;
    return r;
}
}  // namespace glsl_specular

// StochasticReflectionDirection(I, N, PBR.x * 0.9) as SpecularTrace.glsl:513 calls it.
extern "C" void ref_glsl_spec_direction(const float* incident, const float* normals, int64_t n, float roughness,
                                        uint32_t seed, const uint32_t* rid, float* out) {
    namespace G = glsl_specular;
    for (int64_t i = 0; i < n; ++i) {
        G::g_seed = seed;
        G::g_sample = rid[i];
        G::g_dim = 0;
        const glsl::vec3 d = G::StochasticReflectionDirection(
            glsl::vec3(incident[3 * i], incident[3 * i + 1], incident[3 * i + 2]),
            glsl::vec3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]), roughness * 0.9f);
        out[3 * i] = d.x;
        out[3 * i + 1] = d.y;
        out[3 * i + 2] = d.z;
    }
}

// The diffuse pass's hit shading (DiffuseTrace.glsl:486-494 with GetDirect :368-372) and the
// specular pass's (SpecularTrace.glsl:554-563, 588-596 with SampleLighting :420-425, Sky :435-437,
// IsValid Utility.glsl:117-125 and TransformReflectionTransversal SpatialUtility.glsl:12-14), per
// ray.  in: 18 floats {origin, direction, TUVW, Albedo (rgb, emissive), the normal GetData returns
// (not yet faced), sun visibility (0 or 1, what GetDirectShadow returns)}; out: 4 floats, the
// diffuse statements' {FinalRadiance, AO} or the specular pass's stored texel.  sun_dir, sun
// colour, sky (what the sky textures return), probe (what SampleProbes returns) and roughness
// (PBR.x) are the renderer state the statements read.
extern "C" void ref_glsl_shade(int specular, const float* in, int64_t n, const float* sun_dir, const float* sun,
                               const float* sky, const float* probe, float roughness, float* out) {
    const glsl::vec3 sd(sun_dir[0], sun_dir[1], sun_dir[2]), sc(sun[0], sun[1], sun[2]);
    const glsl::vec3 sk(sky[0], sky[1], sky[2]), pr(probe[0], probe[1], probe[2]);
    for (int64_t i = 0; i < n; ++i) {
        const float* x = in + 18 * i;
        const glsl::vec3 o(x[0], x[1], x[2]), d(x[3], x[4], x[5]), nrm(x[14], x[15], x[16]);
        const glsl::vec4 tuvw(x[6], x[7], x[8], x[9]), alb(x[10], x[11], x[12], x[13]);
        glsl::vec4 r;
        if (!specular) {
            namespace G = glsl_diffuse_shade;
            G::g_shadow = x[17];
            G::g_sun = sc;
            G::u_SunDirection = sd;
            G::g_sky = sk;
            G::shade(o, d, tuvw, alb, nrm, r);
        } else {
            namespace G = glsl_specular_shade;
            G::g_shadow = x[17];
            G::g_sun = sc;
            G::g_sky = sk;
            G::g_probe = pr;
            G::shade(o, d, tuvw, alb, nrm, glsl::vec4(roughness, 0.0f, 0.0f, 0.0f));
            r = G::g_out;
        }
        out[4 * i] = r.x;
        out[4 * i + 1] = r.y;
        out[4 * i + 2] = r.z;
        out[4 * i + 3] = r.w;
    }
}

// UpdateRadianceProbes.glsl main (:408-520 with the functions it calls, SphericalHarmonics.glsl
// and Octahedral.glsl) for every probe of a gx x gy x gz grid, in probe order.  Per probe `in`
// holds 16 floats: the ray direction ImportanceSample returns, the TUVW, Albedo (rgb, emissive) and
// normal IntersectRay returns, and what GetDirectShadow returns.  prev_sh (8 words per probe:
// the u_PrevFrameSH / u_PreviousSH A and B texels), prev_raw (4 floats, u_PrevRaw), map (128
// floats, MapData, updated in place), out_sh and out_raw (o_SHOutputA/B, o_CurrentRaw).
extern "C" void ref_glsl_probe(const int32_t* grid, const float* origin, const float* prev_origin, const float* size,
                               int temporal, const float* sun_dir, const float* sun, const float* sky, const float* in,
                               const uint32_t* prev_sh, const float* prev_raw, float* map, uint32_t* out_sh,
                               float* out_raw) {
    namespace G = glsl_probe;
    G::u_Resolution = glsl::vec3(float(grid[0]), float(grid[1]), float(grid[2]));
    G::u_BoxOrigin = glsl::vec3(origin[0], origin[1], origin[2]);
    G::u_PreviousOrigin = glsl::vec3(prev_origin[0], prev_origin[1], prev_origin[2]);
    G::u_Size = glsl::vec3(size[0], size[1], size[2]);
    G::u_Temporal = temporal != 0;
    G::u_SunDirection = glsl::vec3(sun_dir[0], sun_dir[1], sun_dir[2]);
    G::g_sun = glsl::vec3(sun[0], sun[1], sun[2]);
    G::g_sky = glsl::vec3(sky[0], sky[1], sky[2]);
    G::u_Time = 0.0f;
    G::u_PrevFrameSHA = G::u_PreviousSHA = G::SHImage{prev_sh, 0};
    G::u_PrevFrameSHB = G::u_PreviousSHB = G::SHImage{prev_sh, 1};
    G::o_SHOutputA = G::SHOut{out_sh, 0};
    G::o_SHOutputB = G::SHOut{out_sh, 1};
    G::u_PrevRaw = G::RawImage{prev_raw};
    G::o_CurrentRaw = G::RawOut{out_raw};
    G::MapData = reinterpret_cast<G::ProbeMapPixel*>(map);
    static_assert(sizeof(G::ProbeMapPixel) == 8, "ProbeMapPixel layout");
    int64_t i = 0;
    for (int z = 0; z < grid[2]; ++z)
        for (int y = 0; y < grid[1]; ++y)
            for (int x = 0; x < grid[0]; ++x, ++i) {
                const float* v = in + 16 * i;
                G::gl_GlobalInvocationID = glsl::uvec3{uint32_t(x), uint32_t(y), uint32_t(z)};
                G::g_dir = glsl::vec3(v[0], v[1], v[2]);
                G::g_tuvw = glsl::vec4(v[3], v[4], v[5], v[6]);
                G::g_alb = glsl::vec4(v[7], v[8], v[9], v[10]);
                G::g_nrm = glsl::vec3(v[11], v[12], v[13]);
                G::g_shadow = v[14];
                G::probe_main();
            }
}

// The unit vector LambertBRDF (UpdateRadianceProbes.glsl:351-362) gives for hash values (h.x, h.y,
// h.z), normalised as ImportanceSample does (:370-372).
extern "C" void ref_glsl_lambert_direction(const float* h, int64_t n, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        const glsl::vec3 d =
            glsl::normalize(glsl_probe::LambertBRDF(glsl::vec3(h[3 * i], h[3 * i + 1], h[3 * i + 2])));
        out[3 * i] = d.x;
        out[3 * i + 1] = d.y;
        out[3 * i + 2] = d.z;
    }
}

// SUN_COLOR_PROBES as the shader evaluates it.
extern "C" void ref_glsl_probe_sun_color(float* out3) {
    const glsl::vec3 c = glsl_probe::sun_color_constant();
    out3[0] = c.x;
    out3[1] = c.y;
    out3[2] = c.z;
}

// The RT second-bounce loop (DiffuseTrace.glsl:499-535) per GI slot.  slot: 20 floats {GI ray
// origin, direction, TUVW, Albedo (rgb, emissive), faced normal, FinalRadiance before the loop};
// per bounce (n_bounces <= 8): 15 floats {direction, TUVW, Albedo, normal as GetData returns it,
// sun visibility}.  out_fr: FinalRadiance after the loop; out_org: the origin of each bounce ray.
extern "C" void ref_glsl_bounce(int32_t n_bounces, const float* slot, const float* per_bounce, int64_t n,
                                const float* sun_dir, const float* sun, const float* sky, float* out_fr,
                                float* out_org) {
    namespace G = glsl_bounce;
    G::u_SunDirection = glsl::vec3(sun_dir[0], sun_dir[1], sun_dir[2]);
    G::g_sun = glsl::vec3(sun[0], sun[1], sun[2]);
    G::g_sky = glsl::vec3(sky[0], sky[1], sky[2]);
    G::u_SecondaryBounces = n_bounces;
    for (int64_t i = 0; i < n; ++i) {
        const float* x = slot + 20 * i;
        for (int k = 0; k < n_bounces; ++k) {
            const float* y = per_bounce + (i * n_bounces + k) * 15;
            G::g_dir[k] = glsl::vec3(y[0], y[1], y[2]);
            G::g_tuvw[k] = glsl::vec4(y[3], y[4], y[5], y[6]);
            G::g_alb[k] = glsl::vec4(y[7], y[8], y[9], y[10]);
            G::g_nrm[k] = glsl::vec3(y[11], y[12], y[13]);
            G::g_lit[k] = y[14];
            G::g_org[k] = glsl::vec3(0.0f);
        }
        G::g_k = 0;
        glsl::vec3 fr(x[17], x[18], x[19]);
        G::bounce(glsl::vec3(x[0], x[1], x[2]), glsl::vec3(x[3], x[4], x[5]), glsl::vec4(x[6], x[7], x[8], x[9]),
                  glsl::vec4(x[10], x[11], x[12], x[13]), glsl::vec3(x[14], x[15], x[16]), fr);
        out_fr[3 * i] = fr.x;
        out_fr[3 * i + 1] = fr.y;
        out_fr[3 * i + 2] = fr.z;
        for (int k = 0; k < n_bounces; ++k) {
            out_org[(i * n_bounces + k) * 3] = G::g_org[k].x;
            out_org[(i * n_bounces + k) * 3 + 1] = G::g_org[k].y;
            out_org[(i * n_bounces + k) * 3 + 2] = G::g_org[k].z;
        }
    }
}

// SUN_COLOR_DIFF and SUN_COLOR_SPEC of ColorConstants.h as the shaders evaluate them.
extern "C" void ref_glsl_sun_colors(float* out6) {
    const glsl::vec3 a = glsl_diffuse_shade::sun_color_constant(), b = glsl_specular_shade::sun_color_constant();
    out6[0] = a.x;
    out6[1] = a.y;
    out6[2] = a.z;
    out6[3] = b.x;
    out6[4] = b.y;
    out6[5] = b.z;
}

// CosWeightedHemisphere (Shaders/Include/Sampling.glsl:1-12) for n normals / sample pairs.
extern "C" void ref_glsl_cos_hemisphere(const float* normals, const float* r, int64_t n, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        const glsl::vec3 d = glsl_sampling::CosWeightedHemisphere(
            glsl::vec3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]), glsl::vec2{r[2 * i], r[2 * i + 1]});
        out[3 * i] = d.x;
        out[3 * i + 1] = d.y;
        out[3 * i + 2] = d.z;
    }
}

// float IntersectRay(o, d) (the occlusion query): out[i] = 1 when it returns a value > 0.
extern "C" void ref_glsl_occluded(int stackless, const void* nodes, int64_t n_nodes, const void* tris, int64_t n_tris,
                                  const void* verts, int64_t n_verts, const void* ents, int32_t n_ents,
                                  const float* rays, int64_t n, uint8_t* out) {
    if (!stackless) {
        namespace G = glsl_stack;
        Buffers<G::Node, G::Triangle, G::Vertex, G::BVHEntity> b(nodes, n_nodes, tris, n_tris, verts, n_verts,
                                                                  ents, n_ents);
        G::BVHNodes = b.nodes.data();
        G::BVHTris = b.tris.data();
        G::BVHVertices = b.verts.data();
        G::BVHEntities = b.ents.data();
        G::u_EntityCount = n_ents;
        G::u_TotalNodes = static_cast<int>(n_nodes);
        for (int64_t i = 0; i < n; ++i) {
            const float* r = rays + 8 * i;
            out[i] = G::IntersectRay(glsl::vec3(r[0], r[1], r[2]), glsl::vec3(r[4], r[5], r[6])) > 0.0f ? 1 : 0;
        }
    } else {
        namespace G = glsl_stackless;
        Buffers<G::Node, G::Triangle, G::Vertex, G::BVHEntity> b(nodes, n_nodes, tris, n_tris, verts, n_verts,
                                                                  ents, n_ents);
        G::BVHNodes = b.nodes.data();
        G::BVHTris = b.tris.data();
        G::BVHVertices = b.verts.data();
        G::BVHEntities = b.ents.data();
        G::u_EntityCount = n_ents;
        G::u_TotalNodes = static_cast<int>(n_nodes);
        for (int64_t i = 0; i < n; ++i) {
            const float* r = rays + 8 * i;
            out[i] = G::IntersectRay(glsl::vec3(r[0], r[1], r[2]), glsl::vec3(r[4], r[5], r[6])) > 0.0f ? 1 : 0;
        }
    }
}
