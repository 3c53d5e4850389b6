// wf_tlas.cu — agglomerative TLAS builder on the GPU, node-for-node identical
// to tlas_builder_t::build (tlas_builder.cpp:6-68).
//
// The reference's A/B/C walk is inherently sequential: each step asks
// find_best_match (:86-110) for the partner of one node among the remaining
// ones.  One warp runs the walk; every find_best_match is a warp-parallel scan
// of the remaining list (each lane scans a strided slice in increasing order,
// keeping its first strict minimum, then a shuffle reduction takes the
// smallest value and, on equal values, the smallest list position — exactly
// the element the reference's sequential "area < smallest" loop keeps).  The
// remaining list and its boxes live in shared memory when they fit.
#include "wf_kernels.h"

namespace wf {

namespace {

constexpr uint32_t kSmemInstances = 7168;   // 7 words per list entry -> 200,704 bytes

__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }   // glm::min
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }   // glm::max

struct List {
    uint32_t* idx;   // node index per list position
    float* bmn;      // 3 floats per position
    float* bmx;
};

// find_best_match: partner of list position X among positions [0, count).
__device__ uint32_t best_match(const List& L, uint32_t X, uint32_t count, uint32_t metric) {
    const uint32_t lane = threadIdx.x;
    const float ax0 = L.bmn[3 * X], ax1 = L.bmn[3 * X + 1], ax2 = L.bmn[3 * X + 2];
    const float bx0 = L.bmx[3 * X], bx1 = L.bmx[3 * X + 1], bx2 = L.bmx[3 * X + 2];
    float best = FLT_MAX;
    uint32_t bi = 0xFFFFFFFFu;
    for (uint32_t j = lane; j < count; j += 32u) {
        if (j == X) continue;
        float hx, hy, hz, lx, ly, lz;
        if (metric == 0) {
            // the reference's corners: "max" = max(A.min, B.min), "min" = max(A.max, B.max)
            hx = gmax(ax0, L.bmn[3 * j]); hy = gmax(ax1, L.bmn[3 * j + 1]); hz = gmax(ax2, L.bmn[3 * j + 2]);
            lx = gmax(bx0, L.bmx[3 * j]); ly = gmax(bx1, L.bmx[3 * j + 1]); lz = gmax(bx2, L.bmx[3 * j + 2]);
        } else {
            // the merged box
            lx = gmin(ax0, L.bmn[3 * j]); ly = gmin(ax1, L.bmn[3 * j + 1]); lz = gmin(ax2, L.bmn[3 * j + 2]);
            hx = gmax(bx0, L.bmx[3 * j]); hy = gmax(bx1, L.bmx[3 * j + 1]); hz = gmax(bx2, L.bmx[3 * j + 2]);
        }
        float ex = hx - lx, ey = hy - ly, ez = hz - lz;
        float area = ex * ey + ey * ez + ez * ex;
        if (area < best) { best = area; bi = j; }
    }
    for (int off = 16; off > 0; off >>= 1) {
        float ob = __shfl_down_sync(0xffffffffu, best, off);
        uint32_t oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    return __shfl_sync(0xffffffffu, bi, 0);
}

__device__ __forceinline__ void store_node(float4* nodes, uint32_t k, const float* mn, uint32_t lr, const float* mx,
                                           uint32_t inst) {
    nodes[2 * k] = make_float4(mn[0], mn[1], mn[2], __uint_as_float(lr));
    nodes[2 * k + 1] = make_float4(mx[0], mx[1], mx[2], __uint_as_float(inst));
}

// One warp.  aabbs: 6 floats per instance (min xyz, max xyz); nodes: 2n nodes.
__global__ void __launch_bounds__(32) k_tlas_build(const float* __restrict__ aabbs, uint32_t n, float4* nodes,
                                                   uint32_t* gscratch, uint32_t metric) {
    extern __shared__ uint32_t smem[];
    uint32_t* base = (n <= kSmemInstances) ? smem : gscratch;
    List L;
    L.idx = base;
    L.bmn = reinterpret_cast<float*>(base + n);
    L.bmx = reinterpret_cast<float*>(base + 4 * n);
    const uint32_t lane = threadIdx.x;
    for (uint32_t i = lane; i < n; i += 32u) {
        float mn[3] = {aabbs[6 * i], aabbs[6 * i + 1], aabbs[6 * i + 2]};
        float mx[3] = {aabbs[6 * i + 3], aabbs[6 * i + 4], aabbs[6 * i + 5]};
        store_node(nodes, 1 + i, mn, 0u, mx, i);
        L.idx[i] = 1 + i;
        for (int a = 0; a < 3; ++a) { L.bmn[3 * i + a] = mn[a]; L.bmx[3 * i + a] = mx[a]; }
    }
    __syncwarp();
    uint32_t remaining = n, at = n + 1;
    uint32_t A = 0;
    uint32_t B = best_match(L, A, remaining, metric);
    while (remaining > 1) {
        const uint32_t C = best_match(L, B, remaining, metric);
        if (A == C) {
            if (lane == 0) {
                const uint32_t ia = L.idx[A], ib = L.idx[B];
                float mn[3], mx[3];
                for (int a = 0; a < 3; ++a) {
                    mn[a] = gmin(L.bmn[3 * A + a], L.bmn[3 * B + a]);
                    mx[a] = gmax(L.bmx[3 * A + a], L.bmx[3 * B + a]);
                }
                store_node(nodes, at, mn, ia + (ib << 16), mx, 0u);
                L.idx[A] = at;
                for (int a = 0; a < 3; ++a) { L.bmn[3 * A + a] = mn[a]; L.bmx[3 * A + a] = mx[a]; }
                const uint32_t last = remaining - 1;
                L.idx[B] = L.idx[last];
                for (int a = 0; a < 3; ++a) { L.bmn[3 * B + a] = L.bmn[3 * last + a]; L.bmx[3 * B + a] = L.bmx[3 * last + a]; }
            }
            __syncwarp();
            at++;
            remaining--;
            B = best_match(L, A, remaining, metric);
        } else {
            A = B;
            B = C;
        }
    }
    __syncwarp();
    if (lane == 0) {
        const uint32_t r = L.idx[A];
        const float4 a = nodes[2 * r], b = nodes[2 * r + 1];
        nodes[0] = a;
        nodes[1] = b;
    }
}

}  // namespace

cudaError_t launch_tlas_build(const float* aabbs, uint32_t n, float4* nodes, uint32_t* scratch, uint32_t metric,
                              cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    size_t smem = (n <= kSmemInstances) ? (size_t)n * 7u * 4u : 0u;
    if (smem > 48u * 1024u) {
        cudaError_t e = cudaFuncSetAttribute(k_tlas_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_tlas_build<<<1, 32, smem, stream>>>(aabbs, n, nodes, scratch, metric);
    return cudaGetLastError();
}

}  // namespace wf
