// ORACLE / TEST INFRASTRUCTURE ONLY.  C declarations of the CPU restatement in rq_oracle.cpp.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Buffers use the reference's byte layouts (see include/rq.h for the product-side names):
//   vertex   32 B  {float pos[4]; uint32 packed[4]}              Utils/Vertex.h:7-12
//   triangle 16 B  {int32 i0,i1,i2,mesh}                          BVHConstructor.h:78-83
//   node     64 B  stack  {Lmin,Lmax,Rmin,Rmax} (float4 each)     BVHConstructor.h:72-76
//            32 B  stackless {min,max}                            BVHConstructor.h:66-70
//   entity  192 B  {mat4 model; mat4 inverse; int node_offset, node_count; int data[14]}
//                                                                 BVH/Intersector.h:43-49
typedef struct {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} orc_ray;

typedef struct {
    float t, u, v, w;
    int32_t tri, mesh, entity, iters;
} orc_hit;

typedef struct {
    float model[16];
    float inverse[16];
    int32_t node_offset, node_count;
    int32_t data[14];
} orc_entity;

enum { ORC_STACK = 0, ORC_STACKLESS = 1 };
enum { ORC_TIE_FIRST_FOUND = 0, ORC_TIE_LOWER_INDEX = 1 };
enum { ORC_FLAG_REF_COMPAT = 1, ORC_FLAG_IGNORE_TRANSPARENT = 2 };

typedef struct {
    const void* nodes;
    int64_t n_nodes;
    const int32_t* tris;  // 4 ints per triangle
    const void* verts;    // 32-byte records
    const orc_entity* ents;
    int32_t n_ents;
    int32_t layout;
} orc_scene;

// Closest hit for n rays (IntersectScene / IntersectSceneIgnoreTransparent).
// tri_tests (nullable) receives the number of ray/triangle tests per ray.
void orc_closest(const orc_scene* s, const orc_ray* rays, int64_t n, orc_hit* hits, int tie,
                 int flags, int nthreads, int32_t* tri_tests);

// Any hit (IntersectSceneOcclusion with per-ray TMax).  occluded[i] = 1 when a triangle with
// tmin < t < tmax exists on the traversal path.  iters/tri_tests (nullable) receive counters.
void orc_anyhit(const orc_scene* s, const orc_ray* rays, int64_t n, uint8_t* occluded,
                int nthreads, int32_t* iters, int32_t* tri_tests);

// Single primitives, exposed for known-answer tests.
void orc_ray_triangle(const float ro[3], const float rd[3], const float v0[3], const float v1[3],
                      const float v2[3], float out_tuv[3]);
float orc_ray_bounds_stack(const float ro[3], const float invdir[3], const float bmin[3],
                           const float bmax[3], float maxt);
float orc_ray_bounds_stackless(const float bmin[3], const float bmax[3], const float ro[3],
                               const float invdir[3], float t_min, float t_max);
void orc_barycentrics(const float p[3], const float a[3], const float b[3], const float c[3],
                      float out_uvw[3]);

// Diffuse-GI / RTAO ray generation from primary hits (DiffuseTrace.glsl:439-446,
// Sampling.glsl:1-12).  For every primary ray i with a hit and every k < spp, writes ray
// out[i*spp + k]; rays of missed pixels get tmax = -1 (inactive).  normal_mode 0 = interpolated
// half-packed vertex normal (GetData), 1 = geometric normal.
void orc_gi_raygen(const orc_scene* s, const orc_ray* primary, const orc_hit* hits, int64_t n,
                   int32_t spp, uint32_t seed, float origin_offset, float ray_tmax,
                   int32_t normal_mode, int nthreads, orc_ray* out);

// Lambert + AO shading of secondary hits (DiffuseTrace.glsl:368-372, 486-494).
// Per secondary ray j: rgb radiance and AO term written to out4[j*4 .. j*4+3].  Shadow
// visibility (nullable) is 1 = lit.  albedo: 3 floats per mesh id.
// Surface data of the shading: ModelColor per mesh id and optional albedo textures (per mesh a
// texture index or -1; per texture first texel, width, height, flags 1 = sRGB, 2 = clamp; RGBA8
// texels as little-endian words).
typedef struct {
    const float* albedo;
    int32_t n_albedo;
    int32_t n_mesh_tex;
    const int32_t* mesh_tex;
    const int32_t* tex;
    const uint32_t* texels;
} orc_materials;

void orc_hit_albedo(const orc_scene* s, const orc_hit* hits, int64_t n, const orc_materials* mat,
                    int nthreads, float* out3);
// GetData's interpolated normal (normal_mode 0) or the geometric normal, and the hit's UV.
void orc_hit_normal(const orc_scene* s, const orc_hit* hits, int64_t n, int32_t normal_mode, float* out3);
void orc_hit_uv(const orc_scene* s, const orc_hit* hits, int64_t n, float* out2);
void orc_spec_raygen(const orc_scene* s, const orc_ray* primary, const orc_hit* hits, int64_t n, uint32_t seed,
                     float roughness, float ray_tmax, int32_t normal_mode, int nthreads, orc_ray* out);
// The reflection direction of the specular pass for given incident directions and normals.
void orc_spec_direction(const float* incident, const float* normals, int64_t n, float roughness, uint32_t seed,
                        const uint32_t* rid, float* out);
void orc_spec_shade(const orc_scene* s, const orc_ray* rays, const orc_hit* hits, int64_t n, const uint8_t* lit,
                    const orc_materials* mat, float roughness, const float sun_color[3], const float sky[3],
                    const float ambient[3], int nthreads, float* out4);
void orc_shade(const orc_scene* s, const orc_ray* rays, const orc_hit* hits, int64_t n,
               const uint8_t* shadow_lit, const orc_materials* mat,
               const float sun_dir[3], const float sun_color[3], const float sky_color[3],
               int32_t normal_mode, int nthreads, float* out4);

// Shadow rays toward -sun_dir from secondary hits (origin = hit + N*offset); misses get tmax=-1.
void orc_shadow_raygen(const orc_scene* s, const orc_ray* rays, const orc_hit* hits, int64_t n,
                       const float sun_dir[3], float origin_offset, int32_t normal_mode,
                       int nthreads, orc_ray* out);
void orc_bounce_raygen(const orc_scene* s, const orc_ray* rays, const orc_hit* hits, const uint8_t* alive,
                       const uint32_t* sample_id, int64_t n, uint32_t seed, int32_t bounce, float offset,
                       float ray_tmax, int32_t normal_mode, int nthreads, orc_ray* out);

// Counter-based hash (Jarzynski & Olano 2020, "pcg_hash") and the turn-based sine/cosine used
// by the GI ray generator, exposed for tests.
// AABB collision queries (Collide.comp): boxes = n x {min[4], max[4]} (w unused), out = n x
// {collided, entity, mesh, tri} (-1 fields when nothing collides).  ORC_FLAG_REF_COMPAT keeps the
// reference's repeated separating axis and, for the stack layout, the within-leaf triangle index.
void orc_collide(const orc_scene* s, const float* boxes, int64_t n, int32_t* out, int flags, int nthreads);

// One frame of the radiance-probe update (UpdateRadianceProbes.glsl); the parameters have the
// layout of rq_probe_params.  orc_probe_raygen writes one ray per probe (probe-major, x fastest);
// after the caller traces them (closest hit) and the shadow rays (orc_shadow_raygen, any hit),
// orc_probe_shade shades, encodes, blends and packs: prev_sh / out_sh 8 words per probe, prev_raw
// / out_raw 4 floats, probe_map 128 floats (updated in place); lit (nullable) 1 = lit.
typedef struct {
    int32_t grid[3];
    float origin[3];
    float prev_origin[3];
    float size[3];
    uint32_t seed;
    int32_t temporal;
    int32_t normal_mode;
    int32_t shadow_rays;
    float shadow_offset;
    float ray_tmax;
    float sun_dir[3];
    float sun_color[3];
    float sky_color[3];
} orc_probe_params;
void orc_probe_raygen(const orc_probe_params* p, int nthreads, orc_ray* out);
void orc_probe_direction(uint32_t seed, const uint32_t* ids, int64_t n, float* out3);
void orc_probe_shade(const orc_scene* s, const orc_probe_params* p, const orc_ray* rays, const orc_hit* hits,
                     const uint8_t* lit, const orc_materials* mat, const uint32_t* prev_sh, const float* prev_raw,
                     float* probe_map, uint32_t* out_sh, float* out_raw, int raw_r11, int nthreads);
// The value a GL_R11F_G11F_B10F channel with `mbits` mantissa bits (6: R, G; 5: B) holds for x.
float orc_small_ufloat(float x, int mbits);

// The RT second-bounce loop's accumulation for n GI slots (DiffuseTrace.glsl:499-535): fr and thr0
// 3 floats per slot, in 12 floats per slot and bounce {t, albedo rgb, emissive, normal xyz,
// direction xyz, sun visibility}; out3 = FinalRadiance + Bounced.
void orc_bounce_accumulate(const float* fr, const float* thr0, const float* in, int64_t n, int32_t n_bounces,
                           const float sun_dir[3], const float sun_color[3], const float sky[3], int ref_miss,
                           float* out3);

uint32_t orc_pcg_hash(uint32_t x);
void orc_sincos_turns(float x, float* s, float* c);
// CosWeightedHemisphere (Sampling.glsl:1-12) with the turn-based sine / cosine, n normals.
void orc_cos_hemisphere(const float* normals, const float* r, int64_t n, float* out);

// Brute force over every triangle of every entity, no box tests: the lexicographic minimum of
// (t, triangle, entity) with tmin < t < tmax (strict triangle test); occluded (nullable) = any such
// triangle.  Used to decide hits where two walks disagree.  flags: ORC_FLAG_IGNORE_TRANSPARENT.
void orc_brute_closest(const orc_scene* s, const orc_ray* rays, int64_t n, orc_hit* hits, uint8_t* occluded,
                       int flags, int nthreads);

#ifdef __cplusplus
}
#endif
