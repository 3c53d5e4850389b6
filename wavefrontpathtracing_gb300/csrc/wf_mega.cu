// wf_mega.cu — the megakernel path (render_settings_t.use_wavefront_pathtracing
// = 0; the reference's pathtracer.hlsl:37-169, renderer.cpp:940-1015): one
// thread carries one camera path through every bounce — closest hit, shading,
// its shadow ray — with no queues between the stages.
//
// It is the A/B comparator of the wavefront stages: the per-path arithmetic
// is shade_one() and the traversal visits the same nodes in the same order
// (trace_single), and each path leaves its radiance in the same per-path slot
// the wavefront uses, so the images of the two paths are equal bit for bit.
// Each warp takes 32 paths at a time from a counter.
//
// The same loop also finishes a wavefront wave's last bounces (the tail):
// once a wave's queue is smaller than the GPU has traversal threads, each of
// the remaining paths runs its remaining bounces in one thread, resuming from
// the queue and the path state the previous depth's shade left, so the wave
// pays for its longest remaining path once instead of for its longest ray at
// every remaining depth.
#include "wf_shade.cuh"
#include "wf_traverse.cuh"

namespace wf {

namespace {

constexpr int kMegaBlock = 128;

__device__ __forceinline__ ShadeCtl make_ctl(const ShadeRefs& SH, const WaveParams& W) {
    ShadeCtl K;
    K.frame_seed = W.frame_seed; K.max_bounces = W.max_bounces; K.nee = W.nee; K.rr_start = W.rr_start;
    K.cosine = W.cosine; K.env_strength = W.env_strength; K.env0 = W.env[0]; K.env1 = W.env[1]; K.env2 = W.env[2];
    K.lights = SH.lights; K.light_count = SH.light_count; K.light_total = SH.light_total;
    K.env_tex = W.env_tex; K.view_mode = W.view_mode; K.far_plane = W.far_plane;
    return K;
}

// Per-block counts of the rays the tail traces at each depth (extension rays
// at depths after the first, shadow rays at every depth), added to the wave's
// queue counters once per block so the per-depth statistics stay whole.
struct DepthTally {
    uint32_t* ext;   // shared, kMaxDepth
    uint32_t* sh;    // shared, kMaxDepth
};

// One path from `depth0` (its ray ro/rd, throughput T, last pdf, flags and
// radiance L so far) through its remaining bounces; returns L.
template <bool TALLY>
__device__ __forceinline__ float4 run_path(const SceneRefs& S, const ShadeRefs& SH, const ShadeCtl& K, uint32_t root,
                                           uint32_t pixel, uint32_t sample, uint32_t depth0, uint32_t max_bounces,
                                           V3 ro, V3 rd, V3 T, float last_pdf, uint32_t flags, float4 L,
                                           unsigned long long& n_ext, unsigned long long& n_con, bool& overflow,
                                           const DepthTally& tally) {
    const AdjointRefs none = {nullptr, nullptr, nullptr, nullptr, 0.0f, 1u, 0u};
    for (uint32_t depth = depth0; depth <= max_bounces; ++depth) {
        Hit h;
        n_ext++;
        if (TALLY && depth > depth0) atomicAdd(&tally.ext[depth], 1u);
        if (!trace_single<false>(S, root, ro, rd, FLT_MAX, (flags & kFlagInside) != 0u, h)) overflow = true;
        ShadeIn in;
        in.rd = rd;
        in.tuvp = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        in.inst = h.inst;
        in.T = T;
        in.last_pdf = last_pdf;
        in.flags = flags;
        in.pixel = pixel;
        in.sample = sample;
        in.depth = depth;
        ShadeOut o;
        shade_one(SH, K, in, none, 0u, 0u, o);
        if (o.has_add) {
            L.x = L.x + o.add.x;
            L.y = L.y + o.add.y;
            L.z = L.z + o.add.z;
        }
        if (o.shadow) {
            Hit sh;
            n_con++;
            if (TALLY) atomicAdd(&tally.sh[depth], 1u);
            const bool ok = trace_single<true>(S, root, o.spos, o.sdir, o.stmax, false, sh);
            if (!ok) overflow = true;
            if (ok && sh.inst == kInvalid) {
                L.x = L.x + o.contrib.x;
                L.y = L.y + o.contrib.y;
                L.z = L.z + o.contrib.z;
            }
        }
        if (!o.enqueue) break;
        ro = o.org;
        rd = o.dir;
        T = o.T;
        last_pdf = o.pdf;
        flags = o.flags;
    }
    return L;
}

__device__ __forceinline__ void finish(bool overflow, uint32_t* status, unsigned long long n_ext,
                                       unsigned long long n_con, unsigned long long* totals) {
    if (overflow) atomicOr(status, ERRF_STACK);
    for (int off = 16; off > 0; off >>= 1) {
        n_ext += __shfl_down_sync(0xffffffffu, n_ext, off);
        n_con += __shfl_down_sync(0xffffffffu, n_con, off);
    }
    if ((threadIdx.x & 31u) == 0 && totals) {
        atomicAdd(&totals[0], n_ext);
        atomicAdd(&totals[1], n_con);
    }
}

__global__ void __launch_bounds__(kMegaBlock) k_mega(SceneRefs S, ShadeRefs SH, RenderBuffers B, WaveParams W,
                                                     uint32_t* fetch, unsigned long long* totals) {
    const ShadeCtl K = make_ctl(SH, W);
    const uint32_t root = S.inst_count ? 0u : kInvalid;
    const uint32_t lane = threadIdx.x & 31u;
    const DepthTally none = {nullptr, nullptr};
    unsigned long long n_ext = 0, n_con = 0;
    bool overflow = false;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= W.npaths) break;
        const uint32_t path = base + lane;
        if (path < W.npaths) {
            const uint32_t pixel = W.pix0 + path / W.nsamples;
            const uint32_t sample = W.s0 + path % W.nsamples;
            V3 ro, rd;
            primary_ray(W, pixel % W.width, pixel / W.width, ro, rd);
            B.ps_L[path] = run_path<false>(S, SH, K, root, pixel, sample, 0u, W.max_bounces, ro, rd,
                                           mk(1.0f, 1.0f, 1.0f), 0.0f, kFlagSpecular,
                                           make_float4(0.0f, 0.0f, 0.0f, 0.0f), n_ext, n_con, overflow, none);
        }
    }
    finish(overflow, B.status, n_ext, n_con, totals);
}

// The tail: the paths queued for `depth` resume where shade(depth - 1) left
// them (ray queue depth & 1, ps_T / ps_flags / ps_L by path) after the shadow
// rays of depth - 1 have added their contributions.
__global__ void __launch_bounds__(kMegaBlock) k_mega_tail(SceneRefs S, ShadeRefs SH, RenderBuffers B, WaveParams W,
                                                          uint32_t depth, uint32_t* fetch,
                                                          unsigned long long* totals) {
    __shared__ uint32_t s_ext[kMaxDepth], s_sh[kMaxDepth];
    if (threadIdx.x < kMaxDepth) { s_ext[threadIdx.x] = 0u; s_sh[threadIdx.x] = 0u; }
    __syncthreads();
    const ShadeCtl K = make_ctl(SH, W);
    const uint32_t root = S.inst_count ? 0u : kInvalid;
    const uint32_t lane = threadIdx.x & 31u;
    const DepthTally tally = {s_ext, s_sh};
    const uint32_t n = B.counts[depth];
    const int cur = depth & 1;
    const float4* const qo = cur ? B.q_o[1] : B.q_o[0];
    const float4* const qd = cur ? B.q_d[1] : B.q_d[0];
    const uint32_t* const qp = cur ? B.q_path[1] : B.q_path[0];
    unsigned long long n_ext = 0, n_con = 0;
    bool overflow = false;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const uint32_t i = base + lane;
        if (i < n) {
            const uint32_t path = qp[i];
            const float4 T4 = B.ps_T[path];
            B.ps_L[path] = run_path<true>(S, SH, K, root, W.pix0 + path / W.nsamples, W.s0 + path % W.nsamples, depth,
                                          W.max_bounces, xyz(qo[i]), xyz(qd[i]), xyz(T4), T4.w, B.ps_flags[path],
                                          B.ps_L[path], n_ext, n_con, overflow, tally);
        }
    }
    finish(overflow, B.status, n_ext, n_con, totals);
    __syncthreads();
    if (threadIdx.x < kMaxDepth) {
        if (s_ext[threadIdx.x]) atomicAdd(&B.counts[threadIdx.x], s_ext[threadIdx.x]);
        if (s_sh[threadIdx.x]) atomicAdd(&B.counts[kMaxDepth + threadIdx.x], s_sh[threadIdx.x]);
    }
}

template <class K>
unsigned mega_grid(K kernel) {
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kMegaBlock, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    return (unsigned)(sm_count() * per_sm);
}

}  // namespace

cudaError_t launch_megakernel(const SceneRefs& S, const ShadeRefs& SH, const RenderBuffers& B, const WaveParams& W,
                              uint32_t* fetch, unsigned long long* totals, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    k_mega<<<mega_grid(k_mega), kMegaBlock, 0, stream>>>(S, SH, B, W, fetch, totals);
    return cudaGetLastError();
}

cudaError_t launch_megakernel_tail(const SceneRefs& S, const ShadeRefs& SH, const RenderBuffers& B,
                                   const WaveParams& W, uint32_t depth, uint32_t* fetch,
                                   unsigned long long* totals, cudaStream_t stream) {
    k_mega_tail<<<mega_grid(k_mega_tail), kMegaBlock, 0, stream>>>(S, SH, B, W, depth, fetch, totals);
    return cudaGetLastError();
}

}  // namespace wf
