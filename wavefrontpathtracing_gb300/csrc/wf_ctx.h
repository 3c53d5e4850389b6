// wf_ctx.h — host-side pieces of a context that the batched pipeline
// (wf_batch.cu) shares with the single-scene path (wf_api.cu): mesh access,
// the instance record built by submit_render_mesh, its device table rows and
// its emitter triangles.  Both paths build scenes with these functions, so a
// scene rendered in a batch sees the same bytes as the same scene rendered
// alone.
#pragma once
#include <string>
#include <vector>

#include "../../include/wf.h"
#include "wf_kernels.h"

namespace wf {

// One submitted instance (renderer::submit_render_mesh, renderer.cpp:1283-1350).
struct Instance {
    uint32_t mesh;
    float l2w[16], w2l[16];
    material_t mat;
    uint32_t bsdf;
    float ior;
    bvh_instance_t bi;
};

struct MeshView {
    uint32_t tri_count, node_count;
    const triangle_t* tris;       // host copy, original order
    const float* root_min;
    const float* root_max;
    const float4* d_nodes;
    const float4* d_tris;
    const float4* d_stri;
};

int ctx_use_device(wf_ctx* c);
cudaStream_t ctx_stream(wf_ctx* c);
uint32_t* ctx_status(wf_ctx* c);
uint32_t ctx_mesh_count(wf_ctx* c);
uint32_t ctx_tlas_metric(wf_ctx* c);
// Device table of the context's textures (indexed by id) and one texture by id.
const TexRef* ctx_texture_table(wf_ctx* c);
uint32_t ctx_texture_count(wf_ctx* c);
TexRef ctx_texture(wf_ctx* c, uint32_t id);
bool ctx_mesh(wf_ctx* c, uint32_t mesh, MeshView* out);
// Reads and clears the device status word; maps its flags to a WF_ERR_* code.
int ctx_take_status(wf_ctx* c);
// Host <-> device copies on the context stream, counted in the context's byte totals.
cudaError_t ctx_h2d(wf_ctx* c, void* dst, const void* src, size_t bytes);
cudaError_t ctx_d2h(wf_ctx* c, void* dst, const void* src, size_t bytes);

// Validates and fills an instance record; who names the caller in errors.
int make_instance(wf_ctx* c, uint32_t mesh, const float* l2w, const material_t* mat, uint32_t bsdf, float ior,
                  const char* who, Instance* out);
// The instance's rows of the traversal table (4 float4), the shading table
// (kInstRows float4) and its world AABB (min xyz, max xyz).
void instance_rows(const Instance& in, float4 ti[4], float4 si[kInstRows], float aabb[6]);
// Appends the world-space emitter triangles of an emissive instance, with the
// running area sum the light sampler searches.
// inst: the instance's index, kept in each triangle's n.w (the adjoint's emitter key).
void append_emitters(const Instance& in, uint32_t inst, const MeshView& m, std::vector<LightTri>& out,
                     float& running_area);

int fail_code(int code, const std::string& msg);

}  // namespace wf
