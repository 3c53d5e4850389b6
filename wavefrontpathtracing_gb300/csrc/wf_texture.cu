// wf_texture.cu — block-compressed textures decoded on the GPU.
//
// The reference uploads DDS files' BC blocks as they are and lets the
// hardware sampler decode them (core/assets/asset_loader.cpp:179-206,
// dds.h:125-147).  This library samples RGBA float texels in software, so
// wf_texture_create expands the blocks once, on the device: one thread per
// 4x4 block, its texels written straight to the texture in HBM.  Block
// formats (Microsoft's BC1-BC5, the S3TC / RGTC formats):
//   BC1  two RGB565 endpoints + 2-bit indices; c0 > c1: four colours
//        (c0, c1, (2 c0 + c1) / 3, (c0 + 2 c1) / 3), else three + transparent
//        black ((c0 + c1) / 2, black with alpha 0);
//   BC2  4-bit explicit alpha per texel + a BC1 colour block (four colours);
//   BC3  a BC4-style alpha block + a BC1 colour block (four colours);
//   BC4  one channel: two 8-bit endpoints + 3-bit indices; e0 > e1: eight
//        values ((8 - i) e0 + (i - 1) e1) / 7, else six ((6 - i) e0 +
//        (i - 1) e1) / 5 and 0, 255; read as (r, 0, 0, 1);
//   BC5  two BC4 blocks: (r, g, 0, 1).
// The interpolation's last-bit rounding is left to the hardware by the
// formats' definition; here endpoints expand by bit replication (5 -> 8 bits
// r << 3 | r >> 2, 6 -> 8 bits g << 2 | g >> 4) and every division rounds to
// nearest in integers, so the decode is exact and the CPU checker repeats it.
// The 8-bit results then convert to float as the uncompressed formats do.
#include "../../include/wf.h"
#include "wf_kernels.h"

namespace wf {
namespace {

__device__ __forceinline__ uint32_t rd32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// The four colours of a BC1 colour block (RGBA8 packed r | g << 8 | b << 16 | a << 24).
__device__ __forceinline__ void bc1_palette(const uint8_t* b, bool four, uint32_t pal[4]) {
    const uint32_t c0 = (uint32_t)b[0] | ((uint32_t)b[1] << 8), c1 = (uint32_t)b[2] | ((uint32_t)b[3] << 8);
    uint32_t e[2][3];
    const uint32_t cs[2] = {c0, c1};
    for (int k = 0; k < 2; ++k) {
        const uint32_t r = (cs[k] >> 11) & 31u, g = (cs[k] >> 5) & 63u, bl = cs[k] & 31u;
        e[k][0] = (r << 3) | (r >> 2);
        e[k][1] = (g << 2) | (g >> 4);
        e[k][2] = (bl << 3) | (bl >> 2);
    }
    uint32_t p[4][4];
    for (int ch = 0; ch < 3; ++ch) {
        p[0][ch] = e[0][ch];
        p[1][ch] = e[1][ch];
        if (four || c0 > c1) {
            p[2][ch] = (2u * e[0][ch] + e[1][ch] + 1u) / 3u;
            p[3][ch] = (e[0][ch] + 2u * e[1][ch] + 1u) / 3u;
        } else {
            p[2][ch] = (e[0][ch] + e[1][ch] + 1u) / 2u;
            p[3][ch] = 0u;
        }
    }
    const bool transparent = !(four || c0 > c1);
    for (int i = 0; i < 4; ++i)
        pal[i] = p[i][0] | (p[i][1] << 8) | (p[i][2] << 16) | ((transparent && i == 3) ? 0u : 255u << 24);
}

// The eight values of a BC4 block (BC3 alpha, BC5 channels).
__device__ __forceinline__ void bc4_palette(const uint8_t* b, uint32_t v[8]) {
    const uint32_t e0 = b[0], e1 = b[1];
    v[0] = e0;
    v[1] = e1;
    if (e0 > e1) {
        for (uint32_t i = 2; i < 8; ++i) v[i] = ((8u - i) * e0 + (i - 1u) * e1 + 3u) / 7u;
    } else {
        for (uint32_t i = 2; i < 6; ++i) v[i] = ((6u - i) * e0 + (i - 1u) * e1 + 2u) / 5u;
        v[6] = 0u;
        v[7] = 255u;
    }
}
// 3-bit index of texel t (0..15) in a BC4 block's 48 index bits.
__device__ __forceinline__ uint32_t bc4_index(const uint8_t* b, int t) {
    const uint64_t bits = (uint64_t)b[2] | ((uint64_t)b[3] << 8) | ((uint64_t)b[4] << 16) | ((uint64_t)b[5] << 24) |
                          ((uint64_t)b[6] << 32) | ((uint64_t)b[7] << 40);
    return (uint32_t)((bits >> (3 * t)) & 7u);
}

__global__ void k_decode_bc(const uint8_t* __restrict__ blocks, uint32_t format, uint32_t w, uint32_t h,
                            const float* __restrict__ lut, float4* __restrict__ out) {
    const uint32_t bw = (w + 3u) / 4u, bh = (h + 3u) / 4u;
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (uint64_t)bw * bh) return;
    const uint32_t bx = (uint32_t)(k % bw), by = (uint32_t)(k / bw);
    const bool small = format == WF_TEXTURE_BC1 || format == WF_TEXTURE_BC1_SRGB || format == WF_TEXTURE_BC4;
    const uint8_t* b = blocks + k * (small ? 8u : 16u);
    uint32_t rgba[16];
    if (format == WF_TEXTURE_BC4 || format == WF_TEXTURE_BC5) {
        uint32_t r[8], g[8];
        bc4_palette(b, r);
        if (format == WF_TEXTURE_BC5) bc4_palette(b + 8, g);
        for (int t = 0; t < 16; ++t) {
            const uint32_t gv = format == WF_TEXTURE_BC5 ? g[bc4_index(b + 8, t)] : 0u;
            rgba[t] = r[bc4_index(b, t)] | (gv << 8) | (255u << 24);
        }
    } else {
        const uint8_t* cb = small ? b : b + 8;
        uint32_t pal[4];
        bc1_palette(cb, !small, pal);
        const uint32_t idx = rd32(cb + 4);
        for (int t = 0; t < 16; ++t) rgba[t] = pal[(idx >> (2 * t)) & 3u];
        if (format == WF_TEXTURE_BC2 || format == WF_TEXTURE_BC2_SRGB) {
            for (int t = 0; t < 16; ++t) {
                const uint32_t a4 = (b[t >> 1] >> (4 * (t & 1))) & 15u;
                rgba[t] = (rgba[t] & 0x00FFFFFFu) | ((a4 * 17u) << 24);
            }
        } else if (format == WF_TEXTURE_BC3 || format == WF_TEXTURE_BC3_SRGB) {
            uint32_t a[8];
            bc4_palette(b, a);
            for (int t = 0; t < 16; ++t) rgba[t] = (rgba[t] & 0x00FFFFFFu) | (a[bc4_index(b, t)] << 24);
        }
    }
    for (int t = 0; t < 16; ++t) {
        const uint32_t x = bx * 4u + (uint32_t)(t & 3), y = by * 4u + (uint32_t)(t >> 2);
        if (x >= w || y >= h) continue;
        const uint32_t v = rgba[t];
        out[(size_t)y * w + x] = make_float4(lut[v & 255u], lut[(v >> 8) & 255u], lut[(v >> 16) & 255u],
                                             (float)(v >> 24) / 255.0f);
    }
}

}  // namespace

uint64_t bc_bytes(uint32_t format, uint32_t w, uint32_t h) {
    const uint64_t blocks = (uint64_t)((w + 3) / 4) * ((h + 3) / 4);
    const bool small = format == WF_TEXTURE_BC1 || format == WF_TEXTURE_BC1_SRGB || format == WF_TEXTURE_BC4;
    return blocks * (small ? 8u : 16u);
}

cudaError_t launch_decode_bc(const uint8_t* d_blocks, uint32_t format, uint32_t w, uint32_t h, const float* d_lut,
                             float4* d_out, cudaStream_t stream) {
    const uint64_t blocks = (uint64_t)((w + 3) / 4) * ((h + 3) / 4);
    const unsigned grid = (unsigned)((blocks + 255) / 256);
    k_decode_bc<<<grid, 256, 0, stream>>>(d_blocks, format, w, h, d_lut, d_out);
    return cudaGetLastError();
}

}  // namespace wf
