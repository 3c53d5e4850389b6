// wf_trace.cu — ray-query kernels: extend (closest hit, extend.hlsl:25-40),
// connect (any-hit shadow rays; the reference's connect.hlsl is empty) and the
// stand-alone query behind wf_trace.
#include "wf_kernels.h"
#include "wf_traverse.cuh"

namespace wf {

namespace {

constexpr int kBlock = 128;

int g_sms = 0;

unsigned grid_for(uint32_t n) {
    unsigned blocks = (n + kBlock - 1) / kBlock;
    unsigned cap = (unsigned)sm_count() * 16u;
    if (blocks > cap) blocks = cap;
    return blocks ? blocks : 1u;
}

// RayDesc2 in, hit_result_t out (wf_trace / wf_trace_device).
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kBlock) k_trace_aos(SceneRefs S, const float4* __restrict__ rays, uint32_t n,
                                                      uint32_t* __restrict__ hits, bool no_cull,
                                                      uint32_t* status, Counters* counters) {
    LocalCounters c = {0, 0, 0, 0};
    bool overflow = false;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 a = ldg4(rays + 2ull * i), b = ldg4(rays + 2ull * i + 1);
        Hit h;
        if (!trace_ray<ANY, COUNT>(S, xyz(a), xyz(b), b.w, no_cull, h, c)) overflow = true;
        uint32_t* o = hits + 5ull * i;
        o[0] = h.inst;
        o[1] = h.prim;
        o[2] = __float_as_uint(h.t);
        o[3] = __float_as_uint(h.u);
        o[4] = __float_as_uint(h.v);
    }
    if (overflow) atomicOr(status, ERRF_STACK);
    if (COUNT) flush_counters(c, counters);
}

// Extend: queue[depth & 1] -> hits.  Ray flags in origin.w select culling.
template <bool COUNT>
__global__ void __launch_bounds__(kBlock) k_extend(SceneRefs S, RenderBuffers B, uint32_t depth,
                                                   unsigned long long* total) {
    const uint32_t n = B.counts[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(total, (unsigned long long)n);
    const int cur = depth & 1;
    const float4* __restrict__ qo = B.q_o[cur];
    const float4* __restrict__ qd = B.q_d[cur];
    LocalCounters c = {0, 0, 0, 0};
    bool overflow = false;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 a = qo[i], b = qd[i];
        Hit h;
        bool no_cull = (__float_as_uint(a.w) & kFlagInside) != 0u;
        if (!trace_ray<false, COUNT>(S, xyz(a), xyz(b), b.w, no_cull, h, c)) overflow = true;
        B.h_tuvp[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        B.h_inst[i] = h.inst;
    }
    if (overflow) atomicOr(B.status, ERRF_STACK);
    if (COUNT) flush_counters(c, B.counters);
}

// Connect: any-hit query per shadow ray; unoccluded rays add their
// contribution to their path's radiance (a path has at most one shadow ray
// per depth, so the read-modify-write needs no atomic).
template <bool COUNT>
__global__ void __launch_bounds__(kBlock) k_connect(SceneRefs S, RenderBuffers B, uint32_t depth,
                                                    unsigned long long* total) {
    const uint32_t n = B.counts[kMaxDepth + depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(total, (unsigned long long)n);
    LocalCounters c = {0, 0, 0, 0};
    bool overflow = false;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 a = B.s_o[i], b = B.s_d[i];
        Hit h;
        bool ok = trace_ray<true, COUNT>(S, xyz(a), xyz(b), a.w, false, h, c);
        if (!ok) overflow = true;
        if (ok && h.inst == kInvalid) {
            float4 k = B.s_c[i];
            uint32_t path = __float_as_uint(b.w);
            float4 acc = B.ps_L[path];
            acc.x = acc.x + k.x;
            acc.y = acc.y + k.y;
            acc.z = acc.z + k.z;
            B.ps_L[path] = acc;
        }
    }
    if (overflow) atomicOr(B.status, ERRF_STACK);
    if (COUNT) flush_counters(c, B.counters + 1);
}

}  // namespace

int sm_count() {
    if (g_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}

cudaError_t launch_trace_aos(const SceneRefs& S, const void* rays, uint32_t n, void* hits, uint32_t flags,
                             bool count, uint32_t* status, Counters* counters, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const bool any = (flags & 1u) != 0, no_cull = (flags & 2u) != 0;
    const float4* r = static_cast<const float4*>(rays);
    uint32_t* h = static_cast<uint32_t*>(hits);
    unsigned g = grid_for(n);
    if (any) {
        if (count) k_trace_aos<true, true><<<g, kBlock, 0, stream>>>(S, r, n, h, no_cull, status, counters);
        else k_trace_aos<true, false><<<g, kBlock, 0, stream>>>(S, r, n, h, no_cull, status, counters);
    } else {
        if (count) k_trace_aos<false, true><<<g, kBlock, 0, stream>>>(S, r, n, h, no_cull, status, counters);
        else k_trace_aos<false, false><<<g, kBlock, 0, stream>>>(S, r, n, h, no_cull, status, counters);
    }
    return cudaGetLastError();
}

cudaError_t launch_extend(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, uint32_t max_rays, bool count,
                          unsigned long long* total, cudaStream_t stream) {
    unsigned g = grid_for(max_rays);
    if (count) k_extend<true><<<g, kBlock, 0, stream>>>(S, B, depth, total);
    else k_extend<false><<<g, kBlock, 0, stream>>>(S, B, depth, total);
    return cudaGetLastError();
}

cudaError_t launch_connect(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, uint32_t max_rays, bool count,
                           unsigned long long* total, cudaStream_t stream) {
    unsigned g = grid_for(max_rays);
    if (count) k_connect<true><<<g, kBlock, 0, stream>>>(S, B, depth, total);
    else k_connect<false><<<g, kBlock, 0, stream>>>(S, B, depth, total);
    return cudaGetLastError();
}

}  // namespace wf
