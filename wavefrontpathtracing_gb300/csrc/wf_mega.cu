// wf_mega.cu — the megakernel path (render_settings_t.use_wavefront_pathtracing
// = 0; the reference's pathtracer.hlsl:37-169, renderer.cpp:940-1015): one
// thread carries one camera path through every bounce — closest hit, shading,
// its shadow ray — with no queues between the stages.
//
// It exists as the A/B comparator of the wavefront stages: the per-path
// arithmetic is shade_one() and the traversal visits the same nodes in the
// same order (trace_single), and each path leaves its radiance in the same
// per-path slot the wavefront uses, so the images of the two paths are equal
// bit for bit.  Each warp takes 32 camera paths at a time from a counter.
#include "wf_shade.cuh"
#include "wf_traverse.cuh"

namespace wf {

namespace {

constexpr int kMegaBlock = 128;

__global__ void __launch_bounds__(kMegaBlock) k_mega(SceneRefs S, ShadeRefs SH, RenderBuffers B, WaveParams W,
                                                     uint32_t* fetch, unsigned long long* totals) {
    ShadeCtl K;
    K.frame_seed = W.frame_seed; K.max_bounces = W.max_bounces; K.nee = W.nee; K.rr_start = W.rr_start;
    K.cosine = W.cosine; K.env_strength = W.env_strength; K.env0 = W.env[0]; K.env1 = W.env[1]; K.env2 = W.env[2];
    K.lights = SH.lights; K.light_count = SH.light_count; K.light_total = SH.light_total;
    K.env_tex = W.env_tex; K.view_mode = W.view_mode; K.far_plane = W.far_plane;
    const AdjointRefs none = {nullptr, nullptr, nullptr, nullptr, 0.0f, 1u, 0u};
    const uint32_t root = S.inst_count ? 0u : kInvalid;
    const uint32_t lane = threadIdx.x & 31u;
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
            V3 T = mk(1.0f, 1.0f, 1.0f);
            uint32_t flags = kFlagSpecular;
            float last_pdf = 0.0f;
            float4 L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            for (uint32_t depth = 0; depth <= W.max_bounces; ++depth) {
                Hit h;
                n_ext++;
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
            B.ps_L[path] = L;
        }
    }
    if (overflow) atomicOr(B.status, ERRF_STACK);
    for (int off = 16; off > 0; off >>= 1) {
        n_ext += __shfl_down_sync(0xffffffffu, n_ext, off);
        n_con += __shfl_down_sync(0xffffffffu, n_con, off);
    }
    if (lane == 0 && totals) {
        atomicAdd(&totals[0], n_ext);
        atomicAdd(&totals[1], n_con);
    }
}

}  // namespace

cudaError_t launch_megakernel(const SceneRefs& S, const ShadeRefs& SH, const RenderBuffers& B, const WaveParams& W,
                              uint32_t* fetch, unsigned long long* totals, cudaStream_t stream) {
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mega, kMegaBlock, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    k_mega<<<sm_count() * per_sm, kMegaBlock, 0, stream>>>(S, SH, B, W, fetch, totals);
    return cudaGetLastError();
}

}  // namespace wf
