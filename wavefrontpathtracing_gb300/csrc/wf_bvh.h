// wf_bvh.h — GPU binned-SAH BLAS builder (bvh_builder.cpp:6-264 semantics).
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/wf.h"

namespace wf {

struct BvhBuildOut {
    // in
    bool keep_device = true;       // keep d_nodes / d_tris (a mesh's device BLAS)
    uint8_t* dst = nullptr;        // optional caller buffer for the blob
    uint64_t dst_capacity = 0;
    // out
    uint32_t node_count = 0;
    float4* d_nodes = nullptr;     // 2 x float4 per node (reference bvh_node_t layout)
    float4* d_tris = nullptr;      // 3 x float4 per triangle in leaf order {v0, idx} {e1} {e2}
    std::vector<uint8_t> blob;     // [bvh_header_t | nodes | bvh_triangle_t | uint32 index] unless in_dst
    uint64_t blob_size = 0;
    bool in_dst = false;           // the blob went to dst (capacity sufficed)
    float root_min[3], root_max[3];
};

// Builds on `stream` and synchronizes it.  Returns a WF_* status.
int gpu_bvh_build(const triangle_t* tris, uint32_t n, const wf_bvh_options& opts, cudaStream_t stream,
                  BvhBuildOut* out);
const char* bvh_last_error();

// The library's accounted device allocator (wf_api.cu).
cudaError_t dmalloc(void** p, size_t bytes);
void dfree(void* p);

}  // namespace wf
