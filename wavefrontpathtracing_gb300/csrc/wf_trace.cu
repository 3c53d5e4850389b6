// wf_trace.cu — ray-query kernels: extend (closest hit, extend.hlsl:25-40),
// connect (any-hit shadow rays; the reference's connect.hlsl is empty) and the
// stand-alone query behind wf_trace.
#include "wf_kernels.h"
#include "wf_traverse.cuh"

namespace wf {

namespace {

int g_sms = 0;

// Extension rays: queue[depth & 1] -> hits.  Ray flags in origin.w select culling.
struct ExtendIO {
    const float4* qo;
    const float4* qd;
    float4* tuvp;
    uint32_t* inst;
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        const float4 a = qo[i], b = qd[i];
        o = xyz(a); d = xyz(b); tmax = b.w;
        nc = (__float_as_uint(a.w) & kFlagInside) != 0u;
    }
    __device__ __forceinline__ uint32_t root(uint32_t, const SceneRefs& S) const { return S.inst_count ? 0u : kInvalid; }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool) const {
        tuvp[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        inst[i] = h.inst;
    }
};

// Shadow rays: an unoccluded ray adds its contribution to its path's radiance
// (a path has at most one shadow ray per depth, so the read-modify-write
// needs no atomic).
struct ConnectIO {
    const float4* so;
    const float4* sd;
    const float4* sc;
    float4* L;
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        const float4 a = so[i], b = sd[i];
        o = xyz(a); d = xyz(b); tmax = a.w; nc = false;
    }
    __device__ __forceinline__ uint32_t root(uint32_t, const SceneRefs& S) const { return S.inst_count ? 0u : kInvalid; }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool ok) const {
        if (!ok || h.inst != kInvalid) return;
        const float4 k = sc[i];
        const uint32_t path = __float_as_uint(sd[i].w);
        float4 acc = L[path];
        acc.x = acc.x + k.x;
        acc.y = acc.y + k.y;
        acc.z = acc.z + k.z;
        L[path] = acc;
    }
};

template <bool ANY, bool COUNT, class IO>
cudaError_t launch(const SceneRefs& S, const IO& io, const uint32_t* count_ptr, uint32_t count, uint32_t* fetch,
                   uint32_t* status, Counters* counters, unsigned long long* total, cudaStream_t stream) {
    auto k = k_trace<ANY, COUNT, IO>;
    k<<<persistent_grid(k), kTraceBlock, 0, stream>>>(S, io, count_ptr, count, fetch, status, counters, total);
    return cudaGetLastError();
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
                             bool count, uint32_t* fetch, uint32_t* status, Counters* counters, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    AosIO io;
    io.rays = static_cast<const float4*>(rays);
    io.hits = static_cast<uint32_t*>(hits);
    io.no_cull = (flags & 2u) != 0;
    const bool any = (flags & 1u) != 0;
    if (any) return count ? launch<true, true>(S, io, nullptr, n, fetch, status, counters, nullptr, stream)
                          : launch<true, false>(S, io, nullptr, n, fetch, status, counters, nullptr, stream);
    return count ? launch<false, true>(S, io, nullptr, n, fetch, status, counters, nullptr, stream)
                 : launch<false, false>(S, io, nullptr, n, fetch, status, counters, nullptr, stream);
}

cudaError_t launch_extend(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, uint32_t, bool count,
                          unsigned long long* total, cudaStream_t stream) {
    ExtendIO io;
    const int cur = depth & 1;
    io.qo = B.q_o[cur]; io.qd = B.q_d[cur]; io.tuvp = B.h_tuvp; io.inst = B.h_inst;
    uint32_t* fetch = B.counts + 2 * kMaxDepth + depth;
    return count ? launch<false, true>(S, io, B.counts + depth, 0, fetch, B.status, B.counters, total, stream)
                 : launch<false, false>(S, io, B.counts + depth, 0, fetch, B.status, B.counters, total, stream);
}

cudaError_t launch_connect(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, uint32_t, bool count,
                           unsigned long long* total, cudaStream_t stream) {
    ConnectIO io;
    const int par = depth & 1;
    io.so = B.s_o[par]; io.sd = B.s_d[par]; io.sc = B.s_c[par]; io.L = B.ps_L;
    uint32_t* fetch = B.counts + 3 * kMaxDepth + depth;
    return count ? launch<true, true>(S, io, B.counts + kMaxDepth + depth, 0, fetch, B.status, B.counters + 1, total,
                                      stream)
                 : launch<true, false>(S, io, B.counts + kMaxDepth + depth, 0, fetch, B.status, B.counters + 1, total,
                                       stream);
}

}  // namespace wf
