// wf_bvh.h — GPU binned-SAH BLAS builder (bvh_builder.cpp:6-264 semantics).
#pragma once
#include <algorithm>
#include <cstdint>
#include <thread>
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

// f(lo, hi) over [0, n) in parts of at least `grain`, on up to 16 host threads
// (a part whose thread cannot start runs on the caller's thread).
template <typename F>
void host_parallel(uint64_t n, uint64_t grain, F f) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const uint64_t parts = std::min<uint64_t>(std::min(hw, 16u), (n + grain - 1) / grain);
    if (parts <= 1) { f(0, n); return; }
    const uint64_t step = (n + parts - 1) / parts;
    std::vector<std::thread> th;
    for (uint64_t q = 1; q < parts; ++q) {
        const uint64_t lo = q * step, hi = std::min(n, lo + step);
        if (lo >= hi) continue;
        try {
            th.emplace_back(f, lo, hi);
        } catch (...) {
            f(lo, hi);
        }
    }
    f(0, std::min(n, step));
    for (auto& t : th) t.join();
}

// The library's accounted device allocator (wf_api.cu).
cudaError_t dmalloc(void** p, size_t bytes);
void dfree(void* p);

}  // namespace wf
