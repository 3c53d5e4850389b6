// wf_trace.cu — ray-query kernels: extend (closest hit, extend.hlsl:25-40),
// connect (any-hit shadow rays; the reference's connect.hlsl is empty) and the
// stand-alone query behind wf_trace.
#include "wf_shade.cuh"
#include "wf_traverse.cuh"

namespace wf {

namespace {

// Extension rays: queue[depth & 1] -> hits.  Ray flags in origin.w select culling.
struct ExtendIO {
    const float4* qo;
    const float4* qd;
    float4* tuvp;
    uint32_t* inst;
    uint32_t cap;        // checked builds: queue entries
    uint32_t* status;
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        if (!in_bounds(i, cap, status)) i = 0u;   // checked builds: flagged, entry 0 stands in
        const float4 a = qo[i], b = qd[i];
        o = xyz(a); d = xyz(b); tmax = b.w;
        nc = (__float_as_uint(a.w) & kFlagInside) != 0u;
    }
    __device__ __forceinline__ uint32_t root(uint32_t, const SceneRefs& S) const { return S.inst_count ? 0u : kInvalid; }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool) const {
        if (!in_bounds(i, cap, status)) return;
        tuvp[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        inst[i] = h.inst;
    }
};

// Camera rays (depth 0), made where they are traced instead of read from a
// queue that a separate generate pass wrote (generate.hlsl): path i is sample
// s0 + i % nsamples of pixel pix0 + i / nsamples, its ray make_primary_ray's
// (common.hlsl:182-195) with tmax = FLT_MAX and no ray flags.
struct CameraIO {
    WaveParams W;
    float4* tuvp;
    uint32_t* inst;
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        const uint32_t pixel = W.pix0 + i / W.nsamples;
        primary_ray(W, pixel % W.width, pixel / W.width, o, d);
        tmax = FLT_MAX;
        nc = false;
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
    float4* Lc;          // wf_adjoint's passes: the additions' rounding errors (else null)
    uint32_t cap;        // checked builds: queue and path entries
    uint32_t* status;
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        if (!in_bounds(i, cap, status)) i = 0u;   // checked builds: flagged, entry 0 stands in
        const float4 a = so[i], b = sd[i];
        o = xyz(a); d = xyz(b); tmax = a.w; nc = false;
    }
    __device__ __forceinline__ uint32_t root(uint32_t, const SceneRefs& S) const { return S.inst_count ? 0u : kInvalid; }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool ok) const {
        if (!ok || h.inst != kInvalid || !in_bounds(i, cap, status)) return;
        const float4 k = sc[i];
        const uint32_t path = __float_as_uint(sd[i].w);
        if (!in_bounds(path, cap, status)) return;
        float4 acc = L[path];
        if (Lc) {
            float4 lc = Lc[path];
            float e;
            acc.x = two_sum(acc.x, k.x, e); lc.x = lc.x + e;
            acc.y = two_sum(acc.y, k.y, e); lc.y = lc.y + e;
            acc.z = two_sum(acc.z, k.z, e); lc.z = lc.z + e;
            Lc[path] = lc;
        } else {
            acc.x = acc.x + k.x;
            acc.y = acc.y + k.y;
            acc.z = acc.z + k.z;
        }
        L[path] = acc;
    }
};

// The adjoint replay's shadow rays: ConnectIO's store, and an unoccluded
// ray's contribution (linear in its emitter's strength) adds
// dloss/dimage . contribution / strength to that emitter's gradient.
struct AdjConnectIO : ConnectIO {
    AdjConnect A;
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool ok) const {
        if (!ok || h.inst != kInvalid || !in_bounds(i, cap, status)) return;
        ConnectIO::store(i, h, ok);
        const float4 k = sc[i];
        const uint32_t path = __float_as_uint(sd[i].w), inst = __float_as_uint(k.w);
        if (!in_bounds(path, cap, status) || !in_bounds(inst, A.ninst, status)) return;
        const float strength = A.sinst[(size_t)kInstRows * inst + 5].w;
        if (strength == 0.0f) return;
        const float4 g = A.dimage[A.pix0 + path / A.nsamples];
        const float v = (g.x * A.inv_spp) * k.x + (g.y * A.inv_spp) * k.y + (g.z * A.inv_spp) * k.z;
        atomicAdd(&A.g_rep[(size_t)(i & 31u) * A.ninst + inst], v / strength);
    }
};

// The shadow rays of depth d and the extension rays of depth d + 1 in one
// persistent launch: both queues are complete once shade(d) has run, and one
// shared pool of rays keeps every warp busy until the last ray of either kind
// instead of leaving two half-empty tails.  Rays [0, n_first) are shadow rays
// (any hit), the rest extension rays (closest hit); each is loaded, traced
// and stored exactly as in its own launch.
struct PairIO {
    ConnectIO c;
    ExtendIO e;
    uint32_t n_first;
    __device__ __forceinline__ bool any(uint32_t i) const { return i < n_first; }
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        if (i < n_first) c.load(i, o, d, tmax, nc);
        else e.load(i - n_first, o, d, tmax, nc);
    }
    __device__ __forceinline__ uint32_t root(uint32_t, const SceneRefs& S) const { return S.inst_count ? 0u : kInvalid; }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool ok) const {
        if (i < n_first) c.store(i, h, ok);
        else e.store(i - n_first, h, ok);
    }
};

template <int LAY>
__global__ void __launch_bounds__(kTraceBlock, LAY ? WF_TRACE_QB_MIN_BLOCKS : WF_TRACE_MIN_BLOCKS)
    k_trace_pair(SceneRefs S, PairIO io, const uint32_t* n_shadow, const uint32_t* n_extend, uint32_t* fetch,
                 uint32_t* status, unsigned long long* totals) {
    io.n_first = *n_shadow;
    const uint32_t ne = *n_extend;
    if (totals && blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&totals[0], (unsigned long long)ne);
        atomicAdd(&totals[1], (unsigned long long)io.n_first);
    }
    LocalCounters c = {0, 0, 0, 0};
    bool overflow = false;
    trace_persistent<false, false, LAY>(S, io, io.n_first + ne, fetch, c, overflow);
    if (overflow) atomicOr(status, ERRF_STACK);
}

// The traversal kernel for the scene's BLAS layout (binary child pairs, or
// the quantized / exact 4-wide nodes with the tie rule).
template <bool ANY, bool COUNT, int LAY, class IO>
void launch_layout(const SceneRefs& S, const IO& io, const uint32_t* count_ptr, uint32_t count, uint32_t* fetch,
                   uint32_t* status, Counters* counters, unsigned long long* total, cudaStream_t stream) {
    auto k = k_trace<ANY, COUNT, LAY, IO>;
    k<<<persistent_grid(k), kTraceBlock, 0, stream>>>(S, io, count_ptr, count, fetch, status, counters, total);
}
template <bool ANY, bool COUNT, class IO>
cudaError_t launch(const SceneRefs& S, const IO& io, const uint32_t* count_ptr, uint32_t count, uint32_t* fetch,
                   uint32_t* status, Counters* counters, unsigned long long* total, cudaStream_t stream) {
    if (S.qbvh == 2u)
        launch_layout<ANY, COUNT, 2>(S, io, count_ptr, count, fetch, status, counters, total, stream);
    else if (S.qbvh == 1u)
        launch_layout<ANY, COUNT, 1>(S, io, count_ptr, count, fetch, status, counters, total, stream);
    else
        launch_layout<ANY, COUNT, 0>(S, io, count_ptr, count, fetch, status, counters, total, stream);
    return cudaGetLastError();
}

}  // namespace

int sm_count() {
    // per device (a process may drive different GPUs), queried once each
    static int s_sms[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int* slot = (dev >= 0 && dev < 64) ? &s_sms[dev] : nullptr;
    if (slot && *slot > 0) return *slot;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    if (slot) *slot = sms;
    return sms;
}

cudaError_t launch_trace_aos(const SceneRefs& S, const void* rays, uint32_t n, void* hits, uint32_t flags,
                             bool count, uint32_t* fetch, uint32_t* status, Counters* counters, cudaStream_t stream,
                             const uint32_t* perm, const uint32_t* varied) {
    if (n == 0) return cudaSuccess;
    AosIO io;
    io.rays = static_cast<const float4*>(rays);
    io.hits = static_cast<uint32_t*>(hits);
    io.no_cull = (flags & 2u) != 0;
    const bool any = (flags & 1u) != 0;
    if (perm) {
        PermutedAosIO pio;
        pio.io = io;
        pio.perm = perm;
        pio.varied = varied;
        if (any) return count ? launch<true, true>(S, pio, nullptr, n, fetch, status, counters, nullptr, stream)
                              : launch<true, false>(S, pio, nullptr, n, fetch, status, counters, nullptr, stream);
        return count ? launch<false, true>(S, pio, nullptr, n, fetch, status, counters, nullptr, stream)
                     : launch<false, false>(S, pio, nullptr, n, fetch, status, counters, nullptr, stream);
    }
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
    io.cap = B.capacity; io.status = B.status;
    uint32_t* fetch = B.counts + 2 * kMaxDepth + depth;
    Counters* ctr = B.counters + depth;
    return count ? launch<false, true>(S, io, B.counts + depth, 0, fetch, B.status, ctr, total, stream)
                 : launch<false, false>(S, io, B.counts + depth, 0, fetch, B.status, ctr, total, stream);
}

cudaError_t launch_extend_camera(const SceneRefs& S, const RenderBuffers& B, const WaveParams& W, bool count,
                                 unsigned long long* total, cudaStream_t stream) {
    if (W.npaths == 0) return cudaSuccess;
    CameraIO io;
    io.W = W; io.tuvp = B.h_tuvp; io.inst = B.h_inst;
    uint32_t* fetch = B.counts + 2 * kMaxDepth;
    return count ? launch<false, true>(S, io, nullptr, W.npaths, fetch, B.status, B.counters, total, stream)
                 : launch<false, false>(S, io, nullptr, W.npaths, fetch, B.status, B.counters, total, stream);
}

cudaError_t launch_connect(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, uint32_t, bool count,
                           unsigned long long* total, cudaStream_t stream, const AdjConnect* adj) {
    ConnectIO io;
    const int par = depth & 1;
    io.so = B.s_o[par]; io.sd = B.s_d[par]; io.sc = B.s_c[par]; io.L = B.ps_L; io.Lc = B.ps_Lc;
    io.cap = B.capacity; io.status = B.status;
    uint32_t* fetch = B.counts + 3 * kMaxDepth + depth;
    Counters* ctr = B.counters + kMaxDepth + depth;
    if (adj) {
        AdjConnectIO aio;
        static_cast<ConnectIO&>(aio) = io;
        aio.A = *adj;
        return launch<true, false>(S, aio, B.counts + kMaxDepth + depth, 0, fetch, B.status, ctr, total, stream);
    }
    return count ? launch<true, true>(S, io, B.counts + kMaxDepth + depth, 0, fetch, B.status, ctr, total, stream)
                 : launch<true, false>(S, io, B.counts + kMaxDepth + depth, 0, fetch, B.status, ctr, total, stream);
}

cudaError_t launch_trace_pair(const SceneRefs& S, const RenderBuffers& B, uint32_t depth, unsigned long long* totals,
                              cudaStream_t stream) {
    PairIO io;
    const int par = (depth - 1) & 1, cur = depth & 1;
    io.c.so = B.s_o[par]; io.c.sd = B.s_d[par]; io.c.sc = B.s_c[par]; io.c.L = B.ps_L; io.c.Lc = B.ps_Lc;
    io.e.qo = B.q_o[cur]; io.e.qd = B.q_d[cur]; io.e.tuvp = B.h_tuvp; io.e.inst = B.h_inst;
    io.c.cap = io.e.cap = B.capacity; io.c.status = io.e.status = B.status;
    io.n_first = 0;
    uint32_t* fetch = B.counts + 2 * kMaxDepth + depth;
    const uint32_t* ns = B.counts + kMaxDepth + depth - 1;
    const uint32_t* ne = B.counts + depth;
    if (S.qbvh == 2u)
        k_trace_pair<2><<<persistent_grid(k_trace_pair<2>), kTraceBlock, 0, stream>>>(S, io, ns, ne, fetch, B.status,
                                                                                       totals);
    else if (S.qbvh == 1u)
        k_trace_pair<1><<<persistent_grid(k_trace_pair<1>), kTraceBlock, 0, stream>>>(S, io, ns, ne, fetch, B.status,
                                                                                       totals);
    else
        k_trace_pair<0><<<persistent_grid(k_trace_pair<0>), kTraceBlock, 0, stream>>>(S, io, ns, ne, fetch, B.status,
                                                                                       totals);
    return cudaGetLastError();
}

}  // namespace wf
