// wf_kernels.h — launch wrappers shared by the host orchestration (wf_api.cu)
// and the kernel translation units.  Every wrapper enqueues on `stream` and
// returns the launch error (cudaGetLastError) without synchronizing.
#pragma once
#include <vector>
#include <cstdint>
#include <cuda_runtime.h>
#include "wf_device.cuh"
#include "../../include/wf_shared.h"

namespace wf {

// Shading-side scene (see the layout comment in wf_device.cuh).
struct ShadeRefs {
    const float4* sinst;          // kInstRows x float4 per instance
    const float4* const* stri;    // per mesh: 6 x float4 per triangle, original order (uv in .w)
    const LightTri* lights;
    uint32_t light_count;
    float light_total;
    const float4* tri_albedo;     // optional per scene triangle albedo (replaces the base colour)
    const uint32_t* inst_tri_offset;  // scene triangle of (instance i, primitive p) = offset[i] + p
    const TexRef* textures;       // indexed by texture id (entry 0 unused: id 0 = default texture)
    // checked builds: bounds of the indices a hit record and the tables carry
    const BlasRef* blas;          // per mesh (triangle counts)
    uint32_t inst_count, mesh_count, texture_count, albedo_count;
    uint32_t* status;
};

// Path-replay adjoint (null pointers in a forward pass).  The replay traces
// the same paths as the forward pass; every path contribution is the product
// of the Lambert albedos along the path and the emitter strength, so a vertex
// on scene triangle t adds w * L / albedo(t) and the emitter adds w . L / strength,
// with L the path's radiance from the forward pass and w = dloss/dimage / spp.
struct AdjointRefs {
    const float4* L_final;        // per path: radiance of the forward pass
    const float4* dimage;         // per pixel: dloss/d(average radiance)
    float4* g_albedo;             // replicas x scene triangles (atomic adds to x, y, z)
    float* g_emission;            // per instance
    float inv_spp;
    uint32_t replicas;            // power of two; a warp adds into replica (block ^ warp) % replicas
    uint32_t triangles;
    const float4* L_final_lo;     // per path: the forward pass's ps_Lc (L_final + L_final_lo = the exact sum)
    float* g_em_rep;              // shadow rays' emitter gradients: 32 replicas x instances
    uint32_t instances;
};

// Sums the gradient replicas into replica 0.
cudaError_t launch_reduce_replicas(float4* g, uint32_t triangles, uint32_t replicas, cudaStream_t stream);

// Wavefront buffers: double-buffered ray queues (the reference reads and
// appends to one ray buffer inside a single shade dispatch, shade.hlsl:52,167),
// hits, per-path state, the shadow-ray queue and the per-pixel accumulator.
struct RenderBuffers {
    float4* q_o[2];       // {origin, ray flags}
    float4* q_d[2];       // {direction, tmax}
    uint32_t* q_path[2];  // path id within the wave
    float4* h_tuvp;       // {t, bary u, bary v, primitive}
    uint32_t* h_inst;     // instance id
    float4* ps_T;         // {throughput rgb, pdf of the last BSDF sample}
    uint32_t* ps_flags;   // path flags
    float4* ps_L;         // path radiance (rgb), summed from zero
    float4* ps_Lc;        // wf_adjoint's passes only (else null): the rounding errors of ps_L's additions
    float4* s_o[2];       // shadow {origin, tmax}, by depth parity (connect at depth d
    float4* s_d[2];       // shadow {direction, path id}   runs while shade at d + 1
    float4* s_c[2];       // shadow {contribution rgb, -}  fills the other buffer)
    uint32_t* counts;     // [d] extension rays at depth d, [kMaxDepth + d] shadow rays,
                          // [2 kMaxDepth + d], [3 kMaxDepth + d] the traversal kernels' fetch counters
    float4* accum;        // per pixel {radiance sum rgb, samples}
    uint32_t* status;     // device error flags (ERRF_*)
    Counters* counters;   // fetch counts per depth: [d] extension rays, [kMaxDepth + d] shadow rays
    uint32_t capacity;    // paths per wave (queue and path-state entries)
};

constexpr uint32_t kMaxDepth = 16;
constexpr uint32_t kFlagInside = 1u;    // ray travels inside a dielectric: no back-face culling
constexpr uint32_t kFlagSpecular = 2u;  // last scattering event was a delta lobe

struct WaveParams {
    float4 clip_to_view[4];   // matrix columns (x,y,z of m[4c..4c+2]), see xform()
    float4 view_to_world[4];
    uint32_t width, height;     // image size (pixel index -> x, y)
    float dim_x, dim_y;         // view_t.render_dim (uv of the primary ray)
    // A wave holds samples [s0, s0 + nsamples) of pixels [pix0, pix0 + np),
    // pixel-major: path p is sample s0 + p % nsamples of pixel pix0 + p / nsamples
    // (npaths = nsamples * np), so the identical camera rays of a pixel's
    // samples share a warp and traverse in lockstep.
    uint32_t pix0, np, s0, nsamples, npaths;
    uint32_t frame_seed;
    uint32_t max_bounces, nee, rr_start, cosine;
    float env_strength;
    float env[3];
    TexRef env_tex;             // texels null: constant env
    uint32_t view_mode;
    float far_plane;
};

// fetch: a zeroed device counter the persistent kernel hands rays out from;
// perm (optional): trace ray perm[k] as the k-th ray (hits at the rays' own
// indices) when the device word *varied is non-zero, ray k otherwise.
cudaError_t launch_trace_aos(const SceneRefs& S, const void* rays, uint32_t n, void* hits, uint32_t flags,
                             bool count, uint32_t* fetch, uint32_t* status, Counters* counters, cudaStream_t stream,
                             const uint32_t* perm = nullptr, const uint32_t* varied = nullptr);
// Ray order for WF_TRACE_REORDER (wf_sort.cu): a stable radix sort of the rays
// by the Morton code of their origin in the scene box (root = the TLAS root
// node, unused when has_scene is false); scratch holds
// reorder_scratch_words(n) words; *perm points into it on return and *varied
// to a device word that stays 0 when every origin fell in one cell (the sort
// then did nothing and perm must not be used).
size_t reorder_scratch_words(uint32_t n);
cudaError_t launch_reorder_rays(const float4* rays, uint32_t n, const float4* root, bool has_scene,
                                uint32_t* scratch, const uint32_t** perm, const uint32_t** varied,
                                cudaStream_t stream);
// total (device) accumulates the number of rays each launch traced.
cudaError_t launch_extend(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, uint32_t max_rays,
                          bool count, unsigned long long* total, cudaStream_t stream);
// The camera rays of a wave (depth 0), made inside the traversal launch.
cudaError_t launch_extend_camera(const SceneRefs& S, const RenderBuffers& B, const WaveParams& W, bool count,
                                 unsigned long long* total, cudaStream_t stream);
cudaError_t launch_shade(const ShadeRefs& SH, const RenderBuffers& B, const WaveParams& W, uint32_t depth,
                         uint32_t max_rays, const AdjointRefs& A, cudaStream_t stream);
// The adjoint replay's shadow rays (wf_adjoint with next-event estimation):
// each unoccluded ray's contribution is linear in its emitter's strength.
struct AdjConnect {
    const float4* dimage;   // per pixel: dloss/d(average radiance)
    const float4* sinst;    // shading rows (row 5 .w = emissive strength)
    float* g_rep;           // 32 replicas x ninst emitter gradients (replica = queue slot % 32)
    uint32_t ninst, pix0, nsamples;
    float inv_spp;
};
cudaError_t launch_connect(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, uint32_t max_rays,
                           bool count, unsigned long long* total, cudaStream_t stream,
                           const AdjConnect* adj = nullptr);
// The shadow rays of depth - 1 and the extension rays of depth in one launch
// (depth >= 1); totals[0] / totals[1] count the extension / shadow rays.
cudaError_t launch_trace_pair(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, unsigned long long* totals,
                              cudaStream_t stream);
// The megakernel (use_wavefront_pathtracing = 0): whole paths per thread, each
// path's radiance left in ps_L like the wavefront stages; fetch = a device
// counter (zeroed here), totals[0..1] += extension / shadow rays.
cudaError_t launch_megakernel(const SceneRefs& S, const ShadeRefs& SH, const RenderBuffers& B, const WaveParams& W,
                              uint32_t* fetch, unsigned long long* totals, cudaStream_t stream);
// The wave's remaining bounces from `depth` on, one path per thread: the paths
// of queue `depth` resume from the state shade(depth - 1) left (the shadow
// rays of depth - 1 must have been traced); fetch = a zeroed device counter;
// the rays traced after the queue are added to the wave's per-depth counts.
cudaError_t launch_megakernel_tail(const SceneRefs& S, const ShadeRefs& SH, const RenderBuffers& B,
                                   const WaveParams& W, uint32_t depth, uint32_t* fetch,
                                   unsigned long long* totals, cudaStream_t stream);
// per_depth[d] += counts[d] for the wave's extension (d < kMaxDepth) and shadow
// (kMaxDepth + d) ray counts.
cudaError_t launch_depth_counts(const uint32_t* counts, unsigned long long* per_depth, cudaStream_t stream);
// Adds each pixel's paths of the wave to the accumulator in sample order.
cudaError_t launch_wave_resolve(const RenderBuffers& B, const WaveParams& W, cudaStream_t stream);
// post_process.hlsl:25-72 for a render view mode (tonemap only for mode 0,
// sRGB for modes 0, base colour and emissive).
cudaError_t launch_post(const float4* accum, uint32_t npix, uint32_t view_mode, uchar4* out, cudaStream_t stream);
cudaError_t launch_resolve(const float4* accum, uint32_t npix, float4* out, cudaStream_t stream);

// TLAS: builds nodes [0, 2n) from per-instance world AABBs (tlas_builder.cpp).
// metric 0 = the reference's pairing metric, 1 = merged-box half area (both the
// reference's agglomerative walk), 2 = parallel locally-ordered clustering.
// scratch: tlas_scratch_words(n, metric) words.
size_t tlas_scratch_words(uint32_t n, uint32_t metric);
// instance_bounds 1: a mesh's BLAS frontier boxes ({min, max} float4 pairs).
struct HullRef {
    const float4* boxes;
    uint32_t count;
    uint32_t pad;
};
// World AABBs (6 floats per instance) of n instances from their shading rows
// (rows float4 per instance; rows 0-3 = the local-to-world columns, the mesh
// index in row 0's w) and their meshes' frontier boxes.
cudaError_t launch_instance_bounds(const float4* sinst, uint32_t rows, uint32_t n, const HullRef* hulls,
                                   uint32_t mesh_count, float* aabbs, cudaStream_t stream);
cudaError_t launch_tlas_build(const float* aabbs /* 6 floats per instance */, uint32_t n, float4* nodes,
                              uint32_t* scratch, uint32_t metric, cudaStream_t stream);

int sm_count();
// Device allocations of the library go through these: they enforce the
// process-wide limit set by wf_set_device_memory_limit (an allocation past it
// fails with cudaErrorMemoryAllocation without reaching the driver).
cudaError_t dmalloc(void** p, size_t bytes);
void dfree(void* p);
// Sets the calling thread's wf_last_error() message; returns code.
int report_error(int code, const char* msg);
// Block-compressed textures (csrc/wf_texture.cu): bytes of a w x h BC image,
// and the GPU decode of its blocks into RGBA float texels (lut: the 8-bit to
// float table of the colour channels).
uint64_t bc_bytes(uint32_t format, uint32_t w, uint32_t h);
cudaError_t launch_decode_bc(const uint8_t* d_blocks, uint32_t format, uint32_t w, uint32_t h, const float* d_lut,
                             float4* d_out, cudaStream_t stream);
// The quantized 4-wide nodes of a BLAS blob (csrc/wf_qbvh.cu): 16 words per
// node; *root_count = the triangles of a single-leaf BLAS (no nodes), else 0.
int qbvh_convert(const uint8_t* blob, uint64_t size, std::vector<uint32_t>& out, uint32_t* root_count,
                 const char** error, bool exact = false);

}  // namespace wf
