// wf_shade.cu — shade (shade.hlsl:42-174 plus the added metal / dielectric /
// next-event / Russian-roulette steps; at depth 0 it also stands in for
// clear_buffers.hlsl + generate.hlsl: the camera rays themselves are made in
// the depth-0 traversal launch) and post-process (post_process.hlsl:25-72).
//
// The per-path arithmetic is the CPU oracle's (oracle/orc_impl.h) operation
// for operation; both are compiled without fused multiply-add.
#include "wf_shade.cuh"

namespace wf {

namespace {

constexpr int kBlock = 256;

unsigned grid_for(uint32_t n) {
    unsigned blocks = (n + kBlock - 1) / kBlock;
    unsigned cap = (unsigned)sm_count() * 8u;
    if (blocks > cap) blocks = cap;
    return blocks ? blocks : 1u;
}

// Shade's block size and, for the plain variant, the resident blocks per SM
// asked of the compiler (which caps its registers accordingly): 3 blocks of
// 256 (80 registers, 120 bytes of spills) measured 7 % faster per frame's
// shade than 2 (126 registers) and 20 % faster than the one kernel for every
// case (121 registers); 5 blocks of 128 (96 registers) in between.
#ifndef WF_SHADE_BLOCK
#define WF_SHADE_BLOCK 256
#endif
#ifndef WF_SHADE_MIN_BLOCKS
#define WF_SHADE_MIN_BLOCKS 3
#endif
constexpr int kShadeBlock = WF_SHADE_BLOCK;

// PLAIN: path tracing without the adjoint's buffers or a debug view, the
// render loop's usual case; the other variant serves every case, at 2
// resident blocks (128 registers at most; left free it took 137, one block).
template <bool PLAIN>
__global__ void __launch_bounds__(kShadeBlock, PLAIN ? WF_SHADE_MIN_BLOCKS : 2)
    k_shade(ShadeRefs SH, RenderBuffers B, WaveParams W, uint32_t depth, AdjointRefs A_in) {
    const AdjointRefs A = PLAIN ? AdjointRefs{} : A_in;
    if (PLAIN) B.ps_Lc = nullptr;
    // depth 0 shades the camera paths of the wave in path order, their state
    // the one a path starts with (throughput 1, specular flag, no radiance),
    // so nothing is read but the hit; it also records the depth-0 count
    const uint32_t n = depth ? B.counts[depth] : W.npaths;
    if (depth == 0 && blockIdx.x == 0 && threadIdx.x == 0) B.counts[0] = W.npaths;
    const int cur = depth & 1, nxt = cur ^ 1;
    ShadeCtl K;
    K.frame_seed = W.frame_seed; K.max_bounces = W.max_bounces; K.nee = W.nee; K.rr_start = W.rr_start;
    K.cosine = W.cosine; K.env_strength = W.env_strength; K.env0 = W.env[0]; K.env1 = W.env[1]; K.env2 = W.env[2];
    K.lights = SH.lights; K.light_count = SH.light_count; K.light_total = SH.light_total;
    K.env_tex = W.env_tex; K.view_mode = PLAIN ? 0u : W.view_mode; K.far_plane = W.far_plane;
    // shadow queue of this depth's parity (selects, not a dynamic index into the parameter)
    float4* const s_o = cur ? B.s_o[1] : B.s_o[0];
    float4* const s_d = cur ? B.s_d[1] : B.s_d[0];
    float4* const s_c = cur ? B.s_c[1] : B.s_c[0];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        ShadeOut o;
        o.enqueue = false; o.shadow = false; o.em_key = kInvalid; o.em_val = 0.0f;
        uint32_t path = 0;
        if (i < n) {
            ShadeIn in;
            if (depth == 0) {
                path = i;
                in.pixel = W.pix0 + path / W.nsamples;
                V3 ro;
                primary_ray(W, in.pixel % W.width, in.pixel / W.width, ro, in.rd);
                in.T = mk(1.0f, 1.0f, 1.0f);
                in.last_pdf = 0.0f;
                in.flags = kFlagSpecular;
            } else {
                path = B.q_path[cur][i];
                if (!in_bounds(path, W.npaths, B.status)) path = 0u;   // checked builds: flagged, path 0 stands in
                in.pixel = W.pix0 + path / W.nsamples;
                in.rd = xyz(B.q_d[cur][i]);
                const float4 T4 = B.ps_T[path];
                in.T = xyz(T4);
                in.last_pdf = T4.w;
                in.flags = B.ps_flags[path];
            }
            in.tuvp = B.h_tuvp[i];
            in.inst = B.h_inst[i];
            in.sample = W.s0 + path % W.nsamples;
            in.depth = depth;
            in.Lb = mk(0.0f, 0.0f, 0.0f);
            in.Lb_lo = in.Lb;
            if (A.g_albedo && depth) {
                in.Lb = xyz(B.ps_L[path]);
                in.Lb_lo = xyz(B.ps_Lc[path]);
            }
            shade_one(SH, K, in, A, path, in.pixel, o);
            if (o.has_add || depth == 0) {
                // the path's radiance starts at zero here
                float4 acc = depth ? B.ps_L[path] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (B.ps_Lc) {
                    // the adjoint's passes also keep the additions' rounding errors
                    float4 lc = depth ? B.ps_Lc[path] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (o.has_add) {
                        float e;
                        acc.x = two_sum(acc.x, o.add.x, e); lc.x = lc.x + e;
                        acc.y = two_sum(acc.y, o.add.y, e); lc.y = lc.y + e;
                        acc.z = two_sum(acc.z, o.add.z, e); lc.z = lc.z + e;
                    }
                    B.ps_Lc[path] = lc;
                } else if (o.has_add) {
                    acc.x = acc.x + o.add.x;
                    acc.y = acc.y + o.add.y;
                    acc.z = acc.z + o.add.z;
                }
                B.ps_L[path] = acc;
            }
        }
        if (A.g_emission) warp_add_by_key(A.g_emission, o.em_key, o.em_val);
        const uint32_t slot = warp_append(&B.counts[depth + 1], o.enqueue);
        if (o.enqueue && in_bounds(slot, B.capacity, B.status)) {
            B.q_o[nxt][slot] = make_float4(o.org.x, o.org.y, o.org.z, __uint_as_float(o.flags & kFlagInside));
            B.q_d[nxt][slot] = make_float4(o.dir.x, o.dir.y, o.dir.z, FLT_MAX);
            B.q_path[nxt][slot] = path;
            B.ps_T[path] = make_float4(o.T.x, o.T.y, o.T.z, o.pdf);
            B.ps_flags[path] = o.flags;
        }
        const uint32_t sslot = warp_append(&B.counts[kMaxDepth + depth], o.shadow);
        if (o.shadow && in_bounds(sslot, B.capacity, B.status)) {
            s_o[sslot] = make_float4(o.spos.x, o.spos.y, o.spos.z, o.stmax);
            s_d[sslot] = make_float4(o.sdir.x, o.sdir.y, o.sdir.z, __uint_as_float(path));
            s_c[sslot] = make_float4(o.contrib.x, o.contrib.y, o.contrib.z, __uint_as_float(o.light_inst));
        }
    }
}

// post_process.hlsl:25-72 with accumulate on: average, NaN/Inf -> magenta,
// Reinhard, linear -> sRGB, RGBA8.
__device__ __forceinline__ float srgb(float c) {
    float x = fminf(fmaxf(c, 0.0f), 1.0f);
    return (x <= 0.0031308f) ? x * 12.92f : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ unsigned char unorm8(float c) {
    return (unsigned char)(fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f + 0.5f);
}
__device__ __forceinline__ bool bad(float x) { return isnan(x) || isinf(x); }

__global__ void k_post(const float4* __restrict__ accum, uint32_t npix, uint32_t view_mode, uchar4* __restrict__ out) {
    const bool tonemap = view_mode == RENDER_VIEW_MODE_NONE;
    const bool to_srgb = tonemap || view_mode == RENDER_VIEW_MODE_MATERIAL_BASE_COLOR ||
                         view_mode == RENDER_VIEW_MODE_MATERIAL_EMISSIVE;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += stride) {
        float4 a = accum[i];
        float inv = a.w > 0.0f ? 1.0f / a.w : 0.0f;
        float r = a.x * inv, g = a.y * inv, b = a.z * inv;
        if (bad(r) || bad(g) || bad(b)) { r = 1.0f; g = 0.0f; b = 1.0f; }
        if (tonemap) { r = r / (1.0f + r); g = g / (1.0f + g); b = b / (1.0f + b); }
        if (to_srgb) { r = srgb(r); g = srgb(g); b = srgb(b); }
        out[i] = make_uchar4(unorm8(r), unorm8(g), unorm8(b), 255);
    }
}

__global__ void k_wave_resolve(RenderBuffers B, WaveParams W) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < W.np; p += stride) {
        float4 acc = B.accum[W.pix0 + p];
        for (uint32_t s = 0; s < W.nsamples; ++s) {
            const float4 L = B.ps_L[(size_t)p * W.nsamples + s];
            acc.x = acc.x + L.x;
            acc.y = acc.y + L.y;
            acc.z = acc.z + L.z;
            acc.w = acc.w + 1.0f;
        }
        B.accum[W.pix0 + p] = acc;
    }
}

__global__ void k_resolve(const float4* __restrict__ accum, uint32_t npix, float4* __restrict__ out) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += stride) {
        float4 a = accum[i];
        out[i] = a.w > 0.0f ? make_float4(a.x / a.w, a.y / a.w, a.z / a.w, a.w) : make_float4(0, 0, 0, 0);
    }
}

__global__ void k_reduce_replicas(float4* g, uint32_t triangles, uint32_t replicas) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < triangles; t += stride) {
        float4 a = g[t];
        for (uint32_t r = 1; r < replicas; ++r) {
            const float4 b = g[(size_t)r * triangles + t];
            a.x += b.x; a.y += b.y; a.z += b.z;
        }
        g[t] = a;
    }
}

}  // namespace

cudaError_t launch_shade(const ShadeRefs& SH, const RenderBuffers& B, const WaveParams& W, uint32_t depth,
                         uint32_t max_rays, const AdjointRefs& A, cudaStream_t stream) {
    unsigned blocks = (max_rays + kShadeBlock - 1) / kShadeBlock;
    const unsigned cap = (unsigned)sm_count() * 8u * (256u / kShadeBlock);
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    const bool plain = !A.g_albedo && !A.g_emission && !B.ps_Lc && W.view_mode == 0u;
    if (plain) k_shade<true><<<blocks, kShadeBlock, 0, stream>>>(SH, B, W, depth, A);
    else k_shade<false><<<blocks, kShadeBlock, 0, stream>>>(SH, B, W, depth, A);
    return cudaGetLastError();
}

cudaError_t launch_reduce_replicas(float4* g, uint32_t triangles, uint32_t replicas, cudaStream_t stream) {
    k_reduce_replicas<<<grid_for(triangles), kBlock, 0, stream>>>(g, triangles, replicas);
    return cudaGetLastError();
}

namespace {
__global__ void k_depth_counts(const uint32_t* counts, unsigned long long* per_depth) {
    const uint32_t d = threadIdx.x;
    if (d < 2 * kMaxDepth) per_depth[d] += counts[d];
}
}  // namespace

cudaError_t launch_depth_counts(const uint32_t* counts, unsigned long long* per_depth, cudaStream_t stream) {
    k_depth_counts<<<1, 2 * kMaxDepth, 0, stream>>>(counts, per_depth);
    return cudaGetLastError();
}

cudaError_t launch_wave_resolve(const RenderBuffers& B, const WaveParams& W, cudaStream_t stream) {
    k_wave_resolve<<<grid_for(W.np), kBlock, 0, stream>>>(B, W);
    return cudaGetLastError();
}

cudaError_t launch_post(const float4* accum, uint32_t npix, uint32_t view_mode, uchar4* out, cudaStream_t stream) {
    k_post<<<grid_for(npix), kBlock, 0, stream>>>(accum, npix, view_mode, out);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const float4* accum, uint32_t npix, float4* out, cudaStream_t stream) {
    k_resolve<<<grid_for(npix), kBlock, 0, stream>>>(accum, npix, out);
    return cudaGetLastError();
}

}  // namespace wf
