// wf_bvh.cu — GPU binned-SAH BLAS builder.
#include "wf_bvh.h"

namespace wf {

static thread_local const char* g_bvh_error = "";

const char* bvh_last_error() { return g_bvh_error; }

int gpu_bvh_build(const triangle_t*, uint32_t, const wf_bvh_options&, cudaStream_t, BvhBuildOut*) {
    g_bvh_error = "GPU BLAS builder not built yet";
    return WF_ERR_STATE;
}

}  // namespace wf
