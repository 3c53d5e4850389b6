/*
 * wf_oracle.h — CPU oracle for the wavefront path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a scalar C restatement of the reference
 * renderer's software acceleration-structure builders, traversal and shading
 * (Contingencyy/WavefrontPathtracing, source/renderer/bvh/ builders and
 * source/renderer/shaders/ HLSL), plus the same restatement of the scattering
 * models this project adds (metal, dielectric, next-event estimation, Russian
 * roulette).  It is the checker the GPU library is compared against and the
 * timed CPU baseline; the product never links, loads or calls it.
 *
 * Build: oracle/Makefile, gcc -O2 -ffp-contract=off (no fused multiply-add, so
 * every float operation rounds exactly as written — on aarch64 gcc would
 * otherwise contract a*b+c into fma).
 *
 * Pinning: the builders are pinned byte-for-byte against the reference's own
 * bvh_builder.cpp / tlas_builder.cpp compiled from the reference sources
 * (oracle/build_ref.sh -> oracle/_ref/libref_bvh.so) and against golden blobs
 * in tests/golden/.  Traversal, intersection, the RNG, primary rays, Lambert
 * sampling, materials, the environment, the debug views and the shade stage
 * are pinned bit for bit against the reference's own HLSL text compiled as
 * C++ (oracle/ref_hlsl/ -> oracle/_ref/libref_hlsl.so, tests/test_ref_hlsl.py);
 * what that comparison shares with this oracle (intrinsic implementations,
 * the keyed seeds) is listed in oracle/ref_hlsl/hlsl_shim.h.  The scattering
 * models the reference does not have (metal, dielectric, next-event
 * estimation, Russian roulette) are checked against the physics instead:
 * energy, normalisation, reciprocity and an independently written FP64
 * estimator (tests/test_physics.py).
 */
#ifndef WF_ORACLE_H
#define WF_ORACLE_H

#include <stdint.h>
#include "../include/wf_shared.h"

#ifdef __cplusplus
extern "C" {
#endif

/* --- builders (bvh_builder.cpp:6-264, tlas_builder.cpp:6-110) ----------- */
/* Writes a malloc'ed blob [bvh_header_t | nodes | bvh_triangle_t | uint32]. */
int orc_bvh_build(const triangle_t* tris, uint32_t n, uint32_t interval_count,
                  uint32_t subdivide_single_prim, uint32_t max_leaf_prims,
                  uint8_t** out_blob, uint64_t* out_size);
/* Writes a malloc'ed blob [tlas_header_t | nodes | bvh_instance_t]. */
int orc_tlas_build(const bvh_instance_t* inst, uint32_t n, uint8_t** out_blob, uint64_t* out_size);
/* metric 0: the reference's; 1: half area of the merged box (an added option); 2: parallel
 * locally-ordered clustering (the GPU library's fast build, an added option). */
int orc_tlas_build_metric(const bvh_instance_t* inst, uint32_t n, uint32_t metric, uint8_t** out_blob,
                          uint64_t* out_size);
void orc_free(void* p);

/* --- scene ----------------------------------------------------------------- */
typedef struct orc_mesh {
    const triangle_t* tris;   /* original triangle order (primitive ids) */
    uint32_t tri_count;
    const uint8_t* blas;      /* [bvh_header_t | nodes | bvh_triangle_t | uint32] */
} orc_mesh;

typedef struct orc_instance {
    float local_to_world[16];
    float world_to_local[16];
    material_t material;
    uint32_t mesh;            /* index into orc_scene.meshes */
    uint32_t bsdf;            /* 0 lambert, 1 metal, 2 dielectric */
    float ior;
} orc_instance;

/* RGBA float texels, row-major, row 0 at v = 0. */
typedef struct orc_texture {
    const float* texels;
    uint32_t w, h;
} orc_texture;

typedef struct orc_scene {
    const orc_mesh* meshes;
    uint32_t mesh_count;
    const uint8_t* tlas;      /* [tlas_header_t | nodes | bvh_instance_t]; bvh_index = mesh */
    const orc_instance* inst;
    uint32_t inst_count;
    /* optional per-triangle albedo (3 per scene triangle; NULL = material base
     * colour); scene triangle of (instance i, primitive p) = inst_tri_offset[i] + p */
    const double* tri_albedo;
    const uint32_t* inst_tri_offset;
    /* textures by id (textures[id - 1]; id 0 = the slot's default texture),
     * named by material_t's four texture indices; env_texture 0 = constant
     * env_color, else an equirect texture id */
    const orc_texture* textures;
    uint32_t texture_count;
    uint32_t env_texture;
} orc_scene;

typedef struct orc_counters {
    uint64_t tlas_node_loads, instance_loads, blas_node_loads, triangle_tests;
} orc_counters;

/* ORC_TIE_RULE: closest hit = smallest (t, instance, primitive), whatever
 * the visiting order (the reference keeps the first of equal-t hits it
 * visits); the GPU library's quantized 4-wide BLAS layout uses it. */
enum { ORC_ANY_HIT = 1, ORC_NO_CULL = 2, ORC_TIE_RULE = 4 };

/* Software closest-hit / any-hit query (accelstruct.hlsl:58-218,
 * intersect.hlsl:7-76).  Returns the number of rays whose 64-entry stack
 * overflowed (those report a miss).  threads <= 1 runs single-threaded. */
uint32_t orc_trace(const orc_scene* s, const RayDesc2* rays, uint32_t n, hit_result_t* hits,
                   uint32_t flags, orc_counters* counters, int threads);
/* The same query evaluated in double precision (intersection and slab math). */
uint32_t orc_trace_f64(const orc_scene* s, const RayDesc2* rays, uint32_t n, hit_result_t* hits,
                       uint32_t flags, int threads);

/* --- rendering -------------------------------------------------------------- */
typedef struct orc_render_params {
    uint32_t max_bounces;
    uint32_t cosine_weighted_diffuse;
    float hdr_env_strength;
    float env_color[3];
    uint32_t spp;
    uint32_t sample_offset;   /* first sample index (accumulated renders) */
    uint32_t nee;
    uint32_t rr_start_depth;
    uint32_t frame_seed;
    uint32_t pixel_begin, pixel_end;   /* render only this pixel range (end 0 = all) */
    uint32_t view_mode;       /* RENDER_VIEW_MODE_* (shade.hlsl:140-153); 0 = path tracing */
    uint32_t tie_rule;        /* 1: closest-hit rays use ORC_TIE_RULE */
} orc_render_params;

typedef struct orc_render_stats {
    uint64_t extend_rays[16];   /* rays traced at each depth */
    uint64_t shadow_rays[16];   /* shadow rays traced at each depth */
    uint64_t stack_overflows;
    orc_counters extend_traffic, shadow_traffic;
} orc_render_stats;

/* FP32 restatement of generate/extend/shade/connect: adds each path's
 * contributions to accum (RGBA float, width*height*4; alpha counts samples) in
 * the same per-pixel order as the GPU kernels. */
int orc_render(const orc_scene* s, const view_t* view, const orc_render_params* p,
               float* accum, orc_render_stats* stats, int threads);
/* Same paths in double precision (libm sin/cos, double geometry math, the same
 * uniform random numbers); accum is double RGBA. */
int orc_render_f64(const orc_scene* s, const view_t* view, const orc_render_params* p,
                   double* accum, int threads);

/* Path-replay adjoint reference (double precision, single thread): for the
 * paths orc_render_f64 would trace, accumulates d(loss)/d(albedo) per scene
 * triangle (3 per triangle) and d(loss)/d(emissive_strength) per instance,
 * given dloss_dimage = d(loss)/d(average radiance), 3 per pixel.  Everything a
 * path gathers after a Lambert vertex (its next-event contribution and the
 * rest of the path) is linear in that vertex's albedo, so the vertex adds
 * (L - L_before) / albedo; every emitted contribution (an emission hit or an
 * unoccluded shadow ray) is linear in its emitter's strength and adds
 * contribution / strength.  Russian roulette's survival probabilities are
 * held constant (the replay takes the same decisions), which keeps the
 * gradient of the expected image unbiased.  Only Lambert albedos are
 * differentiated (a metal's base colour enters through Fresnel). */
int orc_adjoint_f64(const orc_scene* s, const view_t* view, const orc_render_params* p, const double* dloss_dimage,
                    double* d_albedo, double* d_emission);
/* The same with every path traced in single precision, as orc_render traces
 * it (the GPU's paths; gradients still summed in double). */
int orc_adjoint_f32(const orc_scene* s, const view_t* view, const orc_render_params* p, const double* dloss_dimage,
                    double* d_albedo, double* d_emission);

/* --- the scattering models on their own (physics tests) -------------------- */
/* One scattering direction at a surface (bsdf 0 Lambert, 1 GGX metal, 2
 * smooth dielectric, 3 mirror) for a ray arriving along rd, normal n; f64
 * selects the double instance.  Returns flags: bit 0 delta lobe, bit 1 valid,
 * bit 2 the ray crosses into / out of the dielectric. */
int orc_sample_bsdf(int f64, uint32_t bsdf, const double base[3], double alpha, double ior, const double n[3],
                    const double rd[3], double r1, double r2, int cosine, double L[3], double wgt[3], double* pdf);
/* The BSDF value toward wl and the pdf with which orc_sample_bsdf draws wl
 * (v: direction back to the viewer), double instance.  Returns 1 if valid. */
int orc_eval_bsdf(uint32_t bsdf, const double base[3], double alpha, const double n[3], const double v[3],
                  const double wl[3], int cosine, double f[3], double* pdf);
/* The same for m random pairs r[2m] / m directions wl[3m]. */
void orc_sample_bsdf_batch(int f64, uint32_t bsdf, const double base[3], double alpha, double ior, const double n[3],
                           const double rd[3], const double* r, uint32_t m, int cosine, double* L, double* wgt,
                           double* pdf, int* flags);
void orc_eval_bsdf_batch(uint32_t bsdf, const double base[3], double alpha, const double n[3], const double v[3],
                         const double* wl, uint32_t m, int cosine, double* f, double* pdf, int* ok);

/* --- block-compressed textures (orc_bc.c) ----------------------------------- */
/* BC1-BC5 blocks (format = the library's WF_TEXTURE_BC* value) -> RGBA8;
 * returns 0, or -1 for another format. */
int orc_decode_bc(uint32_t format, const uint8_t* blocks, uint32_t w, uint32_t h, uint8_t* rgba);

/* --- small helpers exported for known-answer tests --------------------------- */
uint32_t orc_wang_hash(uint32_t seed);
float orc_rand_float(uint32_t* seed);
uint32_t orc_path_seed(uint32_t frame_seed, uint32_t pixel, uint32_t sample, uint32_t depth);
void orc_sincos_2pi(float r, float* s, float* c);
/* sin / cos of an angle in radians (the definition of the HLSL intrinsics). */
void orc_sincos(float phi, float* s, float* c);
int orc_intersect_triangle(const float v0[3], const float v1[3], const float v2[3],
                           const float org[3], const float dir[3], float* t_inout,
                           float bary[2], int no_cull);
float orc_intersect_aabb(const float bmin[3], const float bmax[3], const float org[3],
                         const float inv_dir[3], float t);
void orc_primary_ray(const view_t* view, uint32_t px, uint32_t py, RayDesc2* out);
float orc_atan2(float y, float x);
float orc_asin(float y);
void orc_int_to_color(uint32_t v, float out[3]);
void orc_tex_sample(const orc_texture* t, float u, float v, float out[4]);
void orc_env_texel(const orc_texture* t, const float dir[3], float out[3]);
/* Lambert direction about the normal n (cosine-weighted or uniform), as the
 * path loop draws it from r1, r2. */
void orc_hemisphere_sample(const float n[3], float r1, float r2, int cosine, float out[3]);

#ifdef __cplusplus
}
#endif

#endif
