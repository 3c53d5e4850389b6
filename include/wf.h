/*
 * wf.h — C ABI of the GB300 wavefront path tracer.
 *
 * The entry points replace the reference renderer's front end for its hot
 * path (source/renderer/renderer.h:13-55, renderer.cpp:632-1049) and its two
 * acceleration-structure builders (source/renderer/bvh/bvh_builder.h:32-33,
 * tlas_builder.h:17-18).  Data crosses the boundary in the reference's own
 * layouts (wf_shared.h).  Conventions:
 *   - every call returns an int status: WF_OK (0) or a negative WF_ERR_*;
 *     nothing aborts the process (the reference aborts through ASSERT_MSG /
 *     FATAL_ERROR, source/core/assertion.h:51-67);
 *   - a wf_ctx owns one CUDA device, one stream and all device memory; one
 *     context must not be used from two threads at once, separate contexts may;
 *   - host pointers are plain host memory unless the name says "device";
 *   - wf_last_error() returns a message for the calling thread's last failure.
 */
#ifndef WF_H
#define WF_H

#include <stddef.h>
#include <stdint.h>
#include "wf_shared.h"

#ifdef __cplusplus
extern "C" {
#endif

#define WF_ABI_VERSION 1

enum wf_status {
    WF_OK = 0,
    WF_ERR_INVALID = -1,   /* bad argument: null pointer, size, unknown handle */
    WF_ERR_OOM = -2,       /* a device or pinned-host allocation failed */
    WF_ERR_CAPACITY = -3,  /* a fixed capacity was exceeded (instances, output size) */
    WF_ERR_TIMEOUT = -4,   /* a bounded device wait gave up */
    WF_ERR_STACK = -5,     /* a traversal stack overflowed (the ray was abandoned) */
    WF_ERR_CUDA = -6,      /* a CUDA runtime call failed */
    WF_ERR_STATE = -7,     /* call out of order (e.g. render before scene_end) */
    WF_ERR_BOUNDS = -8     /* checked builds (libwf_checked.so): a device index was out of
                              bounds; the access was skipped */
};

typedef struct wf_ctx wf_ctx;

/* renderer::init_params_t (renderer.h:15-21) plus device-side options. */
typedef struct wf_init_params {
    uint32_t render_width;
    uint32_t render_height;
    uint32_t backbuffer_count;  /* accepted for source compatibility; unused (headless) */
    uint32_t vsync;             /* accepted for source compatibility; unused */
    int32_t  device;            /* CUDA device ordinal */
    uint32_t wave_capacity;     /* max paths in flight per wave; 0 = min(16 * width * height, 2^25) */
    uint32_t tlas_metric;       /* TLAS build: 0 = the reference's agglomerative walk and pairing metric
                                   (tlas_builder.cpp:96-97, bit-exact), 1 = the same walk pairing by the
                                   half area of the merged box (better trees), 2 = parallel
                                   locally-ordered clustering on the merged-box area (fast rebuilds),
                                   3 = top-down surface-area-heuristic sweep over every boundary of
                                   the box centres' x / y / z orders (the cheapest trees to traverse) */
    /* BLAS layout the traversal reads: 0 = the reference's binary tree, child
     * pairs of 32-byte nodes (bvh_node_t) walked in the reference's order;
     * 1 = the same tree collapsed to 4-wide 64-byte nodes with child boxes
     * quantized to 8 bits per plane (conservatively: each contains its exact
     * box), half the dependent steps per ray; 2 = the same 4-wide nodes with
     * exact float boxes, 128 bytes each (no decoding, two 64-byte lines per
     * step).  With 1 and 2, closest hits follow an order-independent tie rule
     * (smallest t, then smallest (instance, primitive)) instead of "the first
     * of equal-t hits visited": hits differ from layout 0 only on exact-t
     * ties.  The megakernel and the batched pipeline read the binary nodes
     * (kept in every layout). */
    uint32_t blas_layout;
    /* world box of each instance, the TLAS's leaf box: 0 = the world box of
     * the 8 transformed corners of the BLAS root box (renderer.cpp:1324-1336);
     * 1 = the union of the world boxes of up to 4096 BLAS frontier boxes (the
     * interior nodes of largest area opened first), computed on the GPU at
     * wf_scene_end: nearly the transformed geometry's own box (about half the
     * area of 0's for rotated rounded meshes), so rays enter fewer TLAS
     * subtrees and instances that they miss.  The TLAS differs, so hits can
     * differ only in which of exactly equal-t hits is found first.  The
     * batched pipeline keeps 0's boxes. */
    uint32_t instance_bounds;
} wf_init_params;

/* bvh_builder_t::build_options_t (bvh_builder.h:13-17) plus max_leaf_prims:
 * 0 keeps the reference's rule (stop when the best split is not cheaper);
 * k > 0 also forces a split of any node holding more than k triangles. */
typedef struct wf_bvh_options {
    uint32_t interval_count;        /* SAH bins per axis (reference renderer: 8) */
    uint32_t subdivide_single_prim; /* split down to one triangle per leaf */
    uint32_t max_leaf_prims;
} wf_bvh_options;

/* Scattering models.  The reference shades Lambert only (shade.hlsl:107-137);
 * metal and dielectric are additions. */
enum wf_bsdf_type {
    WF_BSDF_LAMBERT = 0,
    WF_BSDF_METAL = 1,       /* GGX conductor, alpha = roughness^2, F0 = base colour */
    WF_BSDF_DIELECTRIC = 2   /* smooth glass, exact Fresnel, index of refraction ior */
};

typedef struct wf_material_ext {
    material_t base;
    uint32_t   bsdf;   /* enum wf_bsdf_type */
    float      ior;    /* dielectric only */
} wf_material_ext;

/* Environment seen by rays that miss: an equirectangular HDR texture
 * (begin_scene's env texture handle, renderer.cpp:599-611; sampled as
 * shade.hlsl:36-40) or, with texture 0, a constant colour (the reference's
 * default environment is a 1x1 white texture). */
typedef struct wf_env {
    float    color[3];
    uint32_t texture;   /* 0 = constant colour; else a wf_texture_create id */
} wf_env;

/* Texel formats of wf_texture_create (renderer::create_render_texture,
 * render_texture_params_t.format).  Texels are converted once to RGBA float:
 * 8-bit UNORM c -> c / 255, sRGB -> linear, RG8 -> (r, g, 0, 1). */
enum wf_texture_format {
    WF_TEXTURE_RGBA8 = 0,
    WF_TEXTURE_RGBA8_SRGB = 1,
    WF_TEXTURE_RG8 = 2,
    WF_TEXTURE_RGBA32F = 3,
    /* block-compressed (the reference's TEXTURE_FORMAT_BC*, dds.h:125-147):
     * data = the 4x4 blocks as a DDS file stores them, decoded on the GPU
     * (BC7 texel for texel as the GPU's texture sampler decodes it; BC1-BC5
     * with the palette interpolations rounded to nearest 8-bit integers) */
    WF_TEXTURE_BC1 = 4,
    WF_TEXTURE_BC1_SRGB = 5,
    WF_TEXTURE_BC2 = 6,
    WF_TEXTURE_BC2_SRGB = 7,
    WF_TEXTURE_BC3 = 8,
    WF_TEXTURE_BC3_SRGB = 9,
    WF_TEXTURE_BC4 = 10,
    WF_TEXTURE_BC5 = 11,
    WF_TEXTURE_BC7 = 12,
    WF_TEXTURE_BC7_SRGB = 13
};

/* Options of one wf_render call beyond render_settings_t. */
typedef struct wf_render_options {
    uint32_t spp;            /* samples per pixel rendered by this call (>= 1) */
    uint32_t nee;            /* 1 = next-event estimation with shadow rays (connect stage) */
    uint32_t rr_start_depth; /* Russian roulette from this depth; 0xFFFFFFFF = off */
    uint32_t wave_paths;     /* paths per wave, <= context capacity; 0 = capacity */
    uint32_t profile;        /* 1 = time every stage with CUDA events (wf_get_stats) */
    uint32_t count_traffic;  /* 1 = count node/instance/triangle fetches (slower) */
    /* how the shadow rays of depth d are traced (next-event estimation on):
     * WF_SCHEDULE_SEPARATE (0) = their own launch on a second stream beside
     * the extension rays of depth d + 1; WF_SCHEDULE_FUSED (1) = in one
     * persistent launch with the extension rays of depth d + 1 (ms_extend then
     * includes them, ms_connect is 0, and the launch counts in both
     * launches_extend and launches_connect); WF_SCHEDULE_SERIAL (2) = their
     * own launch on the main stream after shade (nothing overlaps: each
     * launch's profile time is its own, for per-kernel measurements).
     * Images are identical.  count_traffic uses the separate schedule. */
    uint32_t trace_schedule;
    /* the tail: once a wave's extension queue is expected to hold fewer than
     * tail_paths paths (from the previous wave's queue sizes, scaled to this
     * wave), its remaining bounces run one path per thread in a single launch
     * (the megakernel's loop, resumed from the wavefront's path state) instead
     * of one launch per stage and depth.  0 = never (the default: on the
     * 1080p instanced frame the tail from depth 4 took 2.0 ms against 1.5 ms
     * for the staged depths).  Images are identical either way. */
    uint32_t tail_paths;
    /* WF_SCHEDULE_SEPARATE only: from this depth (>= 1) on, the extension
     * launch of depth d also traces the shadow rays of depth d - 1, as the
     * fused schedule does, while the earlier, larger queues keep their
     * overlapped launches (one launch fewer per fused depth; the bench frame
     * uses 2).  0 = never.  Images are identical. */
    uint32_t fused_from_depth;
} wf_render_options;

enum wf_trace_schedule {
    WF_SCHEDULE_SEPARATE = 0,
    WF_SCHEDULE_FUSED = 1,
    WF_SCHEDULE_SERIAL = 2
};

enum wf_trace_flags {
    WF_TRACE_ANY_HIT = 1u,       /* stop at the first accepted hit (shadow-ray query) */
    WF_TRACE_NO_CULL = 2u,       /* accept back-facing triangles (|det| test) */
    WF_TRACE_COUNT_TRAFFIC = 4u, /* count node/instance/triangle fetches into wf_stats (slower) */
    WF_TRACE_REORDER = 8u        /* trace the rays in the order of their origins' Morton codes in the
                                    scene box (a stable radix sort inside the call, timed with it):
                                    rays that start close together run together and share nodes in
                                    L2; the hits, still at each ray's own index, do not change.  The
                                    sort is skipped when the input is already coherent (three in four
                                    neighbouring rays start in one cell of a 16^3 grid) */
};

/* Counters and timings of the most recent wf_render / wf_trace call. */
typedef struct wf_stats {
    double   ms_total;       /* GPU time of the whole call (CUDA events) */
    /* per stage; the wavefront path makes its camera rays inside the depth-0
     * extend launch, so ms_generate is 0 there */
    double   ms_generate, ms_extend, ms_shade, ms_connect, ms_post, ms_tlas_build;
    uint64_t launches;       /* kernels this library launched */
    uint64_t launches_extend, launches_connect;
    uint64_t rays_extend;    /* closest-hit rays traced */
    uint64_t rays_connect;   /* shadow rays traced */
    uint64_t paths;          /* camera paths started */
    /* count_traffic = 1 only: fetches made by the traversal kernels */
    uint64_t tlas_node_loads, instance_loads, blas_node_loads, triangle_tests;
    uint64_t shadow_tlas_node_loads, shadow_instance_loads, shadow_blas_node_loads, shadow_triangle_tests;
    /* host<->device bytes copied by this context since wf_create (cumulative) */
    uint64_t h2d_bytes, d2h_bytes;
    /* queue sizes of the call (wavefront path): extension and shadow rays per depth */
    uint64_t extend_rays_depth[16], shadow_rays_depth[16];
    /* the tail (wf_render_options.tail_paths): GPU time of its launches
     * (profile = 1; not in ms_extend) and the depth at which the last wave
     * handed its remaining bounces to it (0 = the wave ran every depth in
     * stages; a tail launch counts in launches, not in launches_extend) */
    double   ms_tail;
    uint64_t tail_depth;
    /* profile = 1: GPU time of the extension (incl. the depth-0 camera rays)
     * and shadow-ray launches, per depth */
    double   ms_extend_depth[16], ms_connect_depth[16];
    /* count_traffic = 1: the fetches per depth, {TLAS nodes, instances, BLAS
     * nodes, triangle tests}, of the extension and the shadow rays */
    uint64_t extend_fetch_depth[16][4], shadow_fetch_depth[16][4];
} wf_stats;

/* ---- lifetime (renderer::init / exit, renderer.h:23-24) ------------------ */
int wf_create(const wf_init_params* params, wf_ctx** out_ctx);
int wf_destroy(wf_ctx* ctx);
const char* wf_status_string(int status);
const char* wf_last_error(void);
int wf_abi_version(void);
/* 1 for the bounds-checked build (libwf_checked.so, compiled with WF_CHECKED:
 * every index a kernel reads is checked before use, a bad one raises
 * WF_ERR_BOUNDS), 0 for the normal build. */
int wf_checked_build(void);
/* Process-wide cap on the device memory the library allocates (all contexts
 * and batches); an allocation past it fails with WF_ERR_OOM and leaves the
 * caller's objects usable.  0 = no cap (the default). */
int wf_set_device_memory_limit(uint64_t bytes);
int wf_get_device_memory_usage(uint64_t* out_bytes);
/* The context's cudaStream_t, for callers that time or order work around it. */
int wf_get_stream(wf_ctx* ctx, void** out_stream);
/* Waits for the context's stream; reports a device-side error flag if set. */
int wf_synchronize(wf_ctx* ctx);

/* ---- meshes (renderer::create_render_mesh, renderer.cpp:1246-1281) ------- */
/* De-indexes (vertices, indices) into triangle_t, uploads it and builds the
 * mesh's BLAS on the GPU with `opts` (NULL = reference defaults: 8 bins). */
int wf_mesh_create(wf_ctx* ctx, const vertex_t* vertices, uint32_t vertex_count,
                   const uint32_t* indices, uint32_t index_count,
                   const wf_bvh_options* opts, uint32_t* out_mesh);
/* Same, but uploads a BLAS blob built elsewhere ([bvh_header_t | extract()],
 * the buffer renderer.cpp:113-155 uploads) instead of building one. */
int wf_mesh_create_prebuilt(wf_ctx* ctx, const triangle_t* triangles, uint32_t triangle_count,
                            const void* blas_blob, uint64_t blob_size, uint32_t* out_mesh);
/* Copies the mesh's BLAS blob ([bvh_header_t | nodes | bvh_triangle_t | uint32 index]). */
int wf_mesh_get_blas(wf_ctx* ctx, uint32_t mesh, void* out_blob, uint64_t* inout_size);

/* ---- textures (renderer::create_render_texture) ------------------------- */
/* Uploads a width x height texture (row 0 first); *out_texture is its id
 * (>= 1).  material_t's base_color_index / normal_index /
 * metallic_roughness_index / emissive_index and wf_env.texture take these
 * ids; 0 selects the reference's default texture for the slot (white base
 * colour and emission, normal (127, 127, 255)/255, metallic-roughness
 * (1, 1, 0)).  Materials sample with bilinear filtering and wrap addressing;
 * the metal BSDF's roughness is roughness_factor x the texture's green. */
int wf_texture_create(wf_ctx* ctx, uint32_t width, uint32_t height, uint32_t format, const void* texels,
                      uint32_t* out_texture);

/* ---- scene (renderer::begin_scene / submit_render_mesh / end_scene) ------ */
/* begin_scene (renderer.cpp:599-630): sets the view, clears the instance list,
 * and resets accumulation when the view changed. env may be NULL (white). */
int wf_scene_begin(wf_ctx* ctx, const view_t* view, const wf_env* env);
/* submit_render_mesh (renderer.cpp:1283-1350): local_to_world is a glm
 * column-major mat4; world_to_local is its inverse. Lambert BSDF. */
int wf_instance_submit(wf_ctx* ctx, uint32_t mesh, const float local_to_world[16],
                       const material_t* material);
/* Same with a chosen scattering model (metal, dielectric). */
int wf_instance_submit_ex(wf_ctx* ctx, uint32_t mesh, const float local_to_world[16],
                          const wf_material_ext* material);
/* count wf_instance_submit_ex calls in one: meshes[i], local_to_world[16 i ..
 * 16 i + 15], materials[i]; all are submitted or none (on an error). */
int wf_instance_submit_many(wf_ctx* ctx, uint32_t count, const uint32_t* meshes, const float* local_to_world,
                            const wf_material_ext* materials);
/* Uploads instances, builds the TLAS on the GPU (renderer.cpp:637-669 builds
 * it on the CPU every frame) and the emitter table used by next-event
 * estimation.  Returns once the work is queued on the context's stream (the
 * host arrays are consumed by then); wf_render and the readbacks run after it. */
int wf_scene_end(wf_ctx* ctx);
/* The scene's bvh_instance_t array (world_to_local, world AABB, mesh id). */
int wf_scene_get_instances(wf_ctx* ctx, bvh_instance_t* out, uint32_t capacity, uint32_t* out_count);
/* The scene's TLAS blob ([tlas_header_t | nodes | bvh_instance_t]). */
int wf_scene_get_tlas(wf_ctx* ctx, void* out_blob, uint64_t* inout_size);

/* ---- rendering (renderer::render, renderer.cpp:742-939 + post_process) ---
 * settings->render_view_mode selects the reference's debug views
 * (shade.hlsl:140-153): the primary hit's instance / primitive colour,
 * barycentrics, vertex normal, uv, material base colour / normal map /
 * metallic-roughness / emission, world normal or depth / far_plane; as in the
 * reference a view mode never accumulates over calls. */
/* Renders opts->spp samples per pixel through generate -> extend -> shade ->
 * connect for depth 0..settings->max_bounces, adding them to the accumulator
 * (or replacing it when settings->accumulate == 0).  Asynchronous: errors
 * detected on the device are reported by the next synchronizing call. */
int wf_render(wf_ctx* ctx, const render_settings_t* settings,
              const wf_render_options* opts, uint32_t frame_seed);
/* Average radiance per pixel, RGBA float32 (alpha = samples), row-major, row 0 = top. */
int wf_read_image(wf_ctx* ctx, float* out_rgba, uint64_t float_count);
/* The same image, copied on a stream of its own while the caller goes on
 * (the next wf_scene_begin .. wf_render overlap the copy): out_rgba is
 * complete once wf_synchronize returns (immediately for pageable memory,
 * which the copy finishes before returning; page-locked memory is copied
 * asynchronously).  A later resolve waits for the copy on the device. */
int wf_read_image_async(wf_ctx* ctx, float* out_rgba, uint64_t float_count);
/* post_process.hlsl:25-72: NaN/Inf flag, Reinhard, linear->sRGB, RGBA8. */
int wf_read_image_ldr(wf_ctx* ctx, uint8_t* out_rgba8, uint64_t byte_count);
int wf_get_stats(wf_ctx* ctx, wf_stats* out);

/* ---- checkpoint / resume of a progressive render (no counterpart in the reference,
 * whose only accumulation state is accum_count, renderer.cpp:47-51, 593-596) --
 * The state is the accumulator (per pixel radiance sum and sample count), the
 * number of samples accumulated, the view and the last frame seed.  Resume:
 * wf_create, the same meshes and scene (wf_scene_begin with the saved view),
 * wf_load_accumulator, then wf_render with accumulate = 1 and the same
 * frame_seed: the result equals one uninterrupted render bit for bit. */
int wf_save_accumulator(wf_ctx* ctx, const char* path);
int wf_load_accumulator(wf_ctx* ctx, const char* path, uint32_t* out_samples, uint32_t* out_frame_seed);

/* ---- differentiable rendering (no counterpart in the reference) ---------- */
/* Number of scene triangles: the instances' triangles in submission order,
 * each instance's in primitive order.  Valid after wf_scene_end. */
int wf_scene_triangle_count(wf_ctx* ctx, uint64_t* out_count);
/* Per scene triangle RGB albedo (3 floats each), replacing the instances'
 * base colours until the next wf_scene_begin; NULL restores them. */
int wf_scene_set_albedo(wf_ctx* ctx, const float* rgb, uint64_t triangle_count);
/* Sets an instance's emissive_strength and rebuilds the scene tables. */
int wf_scene_set_emission(wf_ctx* ctx, uint32_t instance, float strength);
/* Path-replay adjoint of the image that wf_render(settings, opts, frame_seed)
 * produces with accumulate = 0: dloss_dimage = d(loss)/d(average radiance),
 * 3 floats per pixel (row-major); writes d(loss)/d(albedo) (3 floats per scene
 * triangle) and d(loss)/d(emissive_strength) (1 per instance).  Each wave is
 * traced once forward (path radiance L) and replayed from the same per-path
 * seeds (w = dloss_dimage / spp, atomics, memory O(paths), no tape): a Lambert
 * vertex adds w*(L - L_before)/albedo, L_before being what the path gathered
 * before it (everything after it, its next-event shadow ray included, is
 * linear in its albedo); each emitted contribution c (an emission hit, or an
 * unoccluded shadow ray with next-event estimation) adds w.c/strength to its
 * emitter.  Russian roulette's survival probabilities are held constant (the
 * replay takes the forward pass's decisions): the gradient of the expected
 * image stays unbiased.  Metal and dielectric base colours are not
 * differentiated, nor an albedo of exactly 0 (its path carries nothing
 * further).  Requires wf_scene_set_albedo; the shadow rays are traced in
 * their own launches whatever trace_schedule says. */
int wf_adjoint(wf_ctx* ctx, const render_settings_t* settings, const wf_render_options* opts, uint32_t frame_seed,
               const float* dloss_dimage, float* d_albedo, float* d_emission);

/* ---- batched rendering (no counterpart in the reference) ----------------
 * Many independent scenes, each with its own camera, resolution, spp and
 * instances of the context's meshes, rendered together.  All scenes share one
 * pool of paths in flight that is refilled with the scenes' camera paths
 * whenever the live count falls below a threshold (path regeneration); every
 * stage reads its sizes from the device, so the whole render is one CUDA-graph
 * launch whose device-side loop runs until every path has finished.  A scene's
 * image equals the image wf_render produces for the same scene, settings and
 * frame_seed with accumulate = 0, bit for bit. */
typedef struct wf_batch wf_batch;

typedef struct wf_batch_config {
    uint32_t capacity;        /* paths in flight (pool entries), 1024 .. 2^27; 0 = 2^21 */
    float    regen_threshold; /* admit new camera paths when fewer than threshold * capacity
                                 are live, (0, 1]; 0 = 1 (refill every iteration) */
    uint32_t block;           /* threads per block of regeneration and shading: 128, 256 or 512; 0 = 256 */
    uint32_t use_graph;       /* 1 = one CUDA-graph launch with a device-side loop (default);
                                 0 = host-driven loop that polls for completion */
    uint32_t max_iterations;  /* iteration budget of the device loop: 0 = a bound derived from the
                                 batch (never reached by a correct run); a render that needs more
                                 stops and returns WF_ERR_TIMEOUT, leaving the batch usable */
    uint32_t reserved[3];
} wf_batch_config;

typedef struct wf_batch_stats {
    double   ms_total;        /* GPU time of the last wf_batch_render (CUDA events) */
    uint64_t paths;           /* camera paths: sum over scenes of width * height * spp */
    uint64_t rays_extend;     /* closest-hit rays traced */
    uint64_t rays_connect;    /* shadow rays traced */
    uint64_t kernel_launches; /* kernels the device executed for the last render */
    uint32_t iterations;      /* pipeline iterations (regenerate, extend, shade, connect) */
    uint32_t graph_launches;  /* CUDA-graph launches of the last render (0 with the host loop) */
    uint32_t scenes;
    uint32_t reserved[3];
} wf_batch_stats;

/* A batch renders instances of ctx's meshes on ctx's device and stream; it
 * must be destroyed before ctx. */
int wf_batch_create(wf_ctx* ctx, wf_batch** out_batch);
int wf_batch_destroy(wf_batch* batch);
/* Opens scene *out_scene (numbered from 0): image width x height, spp camera
 * paths per pixel, view as wf_scene_begin, env NULL = white. */
int wf_batch_scene_begin(wf_batch* batch, uint32_t width, uint32_t height, uint32_t spp,
                         const view_t* view, const wf_env* env, uint32_t* out_scene);
/* wf_instance_submit_ex into the open scene. */
int wf_batch_instance_submit(wf_batch* batch, uint32_t mesh, const float local_to_world[16],
                             const wf_material_ext* material);
int wf_batch_scene_end(wf_batch* batch);
int wf_batch_set_config(wf_batch* batch, const wf_batch_config* config);
int wf_batch_get_config(wf_batch* batch, wf_batch_config* out_config);
/* Renders every scene (opts->spp is ignored: each scene has its own), then
 * synchronizes.  The first render after a scene change builds the scene tables
 * (one GPU TLAS per scene) and the CUDA graph. */
int wf_batch_render(wf_batch* batch, const render_settings_t* settings,
                    const wf_render_options* opts, uint32_t frame_seed);
/* Picks capacity, regeneration threshold and block size by timing renders of
 * this batch (coordinate descent); leaves the best configuration set. */
int wf_batch_autotune(wf_batch* batch, const render_settings_t* settings,
                      const wf_render_options* opts, uint32_t frame_seed, wf_batch_config* out_config);
/* Average radiance of one scene, RGBA float32 (alpha = samples), as wf_read_image. */
int wf_batch_read_image(wf_batch* batch, uint32_t scene, float* out_rgba, uint64_t float_count);
int wf_batch_get_stats(wf_batch* batch, wf_batch_stats* out);

/* ---- ray queries (extend.hlsl / accelstruct.hlsl:151-218) ---------------- */
/* Traces host rays against the current scene; copies in, traces, copies out. */
int wf_trace(wf_ctx* ctx, const RayDesc2* rays, uint32_t count, hit_result_t* hits, uint32_t flags);
/* Same on device buffers already resident on the context's device; enqueued
 * on the context stream (no synchronization). */
int wf_trace_device(wf_ctx* ctx, const RayDesc2* device_rays, uint32_t count,
                    hit_result_t* device_hits, uint32_t flags);

/* ---- stand-alone builders (bvh_builder_t / tlas_builder_t) --------------- */
/* Builds a BLAS on the GPU; writes [bvh_header_t | extract()] byte-identical to
 * the reference builder's output at equal options.  *inout_size: capacity in,
 * bytes written out (WF_ERR_CAPACITY with the needed size if too small, after
 * a whole build).  The blob never exceeds WF_BVH_BLOB_MAX(triangle_count)
 * bytes (at most 2n nodes of 32 bytes, 36 + 4 bytes per triangle), so a
 * buffer of that size needs a single call. */
#define WF_BVH_BLOB_MAX(n) (12ull + 104ull * (unsigned long long)(n))
int wf_bvh_build(wf_ctx* ctx, const triangle_t* triangles, uint32_t triangle_count,
                 const wf_bvh_options* opts, void* out_blob, uint64_t* inout_size);
/* Builds a TLAS on the GPU with the context's tlas_metric; with metric 0 it
 * writes [tlas_header_t | extract()] byte-identical to tlas_builder_t.  Up to
 * 32768 instances (16-bit child indices). */
int wf_tlas_build(wf_ctx* ctx, const bvh_instance_t* instances, uint32_t instance_count,
                  void* out_blob, uint64_t* inout_size);
/* The quantized 4-wide nodes (blas_layout 1) of a BLAS blob, built on the
 * host: 64 bytes per node (4 x float4: {origin xyz, biased exponents and child
 * count}, {lo planes x/y/z, leaf counts low bytes}, {hi planes, leaf counts
 * high bytes}, {child: node index, or first triangle of a leaf}) into
 * out_nodes (NULL = size query through *inout_size); *out_root_count = the
 * triangles of a BLAS that is a single leaf (then no nodes), else 0.  No
 * counterpart in the reference (its BLAS is binary). */
int wf_bvh_quantize(const void* blob, uint64_t blob_size, void* out_nodes, uint64_t* inout_size,
                    uint32_t* out_root_count);
/* The exact 4-wide nodes (wf_init_params.blas_layout = 2) of a BLAS blob, on
 * the host: 128 bytes per node (8 x float4: the four children's lo x / hi x /
 * lo y / hi y / lo z / hi z planes as float4 lanes, child[4] = node index or
 * a leaf's first triangle in leaf order, count[4] = leaf triangle counts with
 * the child count in count[0]'s top byte) into out_nodes (NULL = size query
 * through *inout_size); *out_root_count as wf_bvh_quantize.  No counterpart
 * in the reference (its BLAS is binary). */
int wf_bvh_widen(const void* blob, uint64_t blob_size, void* out_nodes, uint64_t* inout_size,
                 uint32_t* out_root_count);

/* ---- image files (asset_loader.cpp:56-206) -----------------------------
 * Decodes a .jpg / .jpeg (baseline or progressive) or a .png (every colour
 * type and bit depth, interlaced or not; 16-bit samples keep their high
 * byte) — the reference calls stbi_load with 4 channels for both,
 * asset_loader.cpp:109 — a Radiance .hdr (stbi_loadf with 4 channels, :150)
 * or a .dds (its top mip level, :179-206) held in memory: *out_format =
 * WF_TEXTURE_RGBA8 (JPEG, PNG), WF_TEXTURE_RGBA32F (HDR) or
 * the DDS file's format (RGBA8 / RGBA8_SRGB / RG8 / RGBA32F texels, BC1-BC5 /
 * BC7 blocks as stored); out receives what wf_texture_create takes with that
 * format (NULL = size query through *inout_size).  Host only. */
int wf_image_decode(const void* file, uint64_t file_size, uint32_t* out_width, uint32_t* out_height,
                    uint32_t* out_format, void* out, uint64_t* inout_size);
/* Reads a texture's RGBA float texels back (width * height * 4 floats). */
int wf_texture_read(wf_ctx* ctx, uint32_t texture, float* out, uint64_t float_count);

/* ---- allocation-free TLAS build (no counterpart in the reference) --------
 * For callers that cannot allocate device memory: per-frame render threads
 * that must not pay an allocation's implicit device synchronisation, and
 * engines that hand out all of their device memory from a budget fixed up
 * front (their own pool, a hard memory cap).  The caller owns both device
 * buffers: device_aabbs = instance_count x {min xyz, max xyz} floats,
 * device_nodes = 2 * instance_count tlas_node_t (one when instance_count is 0);
 * the result equals the nodes wf_tlas_build writes with the same tlas_metric (0 or 1;
 * metric 2 needs a larger working set and is not offered here).
 * The build's working list lives in a static 224 KiB device array, so:
 *   - at most 8192 instances (larger counts return WF_ERR_CAPACITY);
 *   - every call on a device shares that array: calls that overlap on the GPU
 *     (other streams, other threads) race and must be serialised by the caller;
 *   - the first call in a CUDA context (the device's primary context, or one the
 *     caller created and made current) loads the module and looks up the
 *     array's device address in that context; make it before any stream
 *     capture.  Up to 64 contexts are remembered; in others the address is
 *     looked up on every call.
 * Enqueued on `stream` (a cudaStream_t; NULL = default stream), not synchronised;
 * allocates nothing. */
int wf_tlas_build_noalloc(const float* device_aabbs, uint32_t instance_count, void* device_nodes,
                          uint32_t tlas_metric, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WF_H */
