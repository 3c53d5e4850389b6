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
//   BC5  two BC4 blocks: (r, g, 0, 1);
//   BC7  eight modes (the lowest set bit of the first byte) of one to three
//        subsets chosen by a partition pattern, RGB or RGBA endpoints of 4-8
//        bits with optional p-bits, 2-4-bit indices with the subsets' anchor
//        texels one bit short, optional separate alpha indices and channel
//        rotation; every value is exact in 8-bit integers by the format's
//        definition, so the decode equals any conforming one (a first byte of
//        zero, the reserved mode, decodes to transparent black).
// The BC1-BC5 interpolation's last-bit rounding is left to the hardware by
// the formats' definition; here endpoints expand by bit replication (5 -> 8
// bits r << 3 | r >> 2, 6 -> 8 bits g << 2 | g >> 4) and every division
// rounds to nearest in integers, so the decode is exact and the CPU checker
// repeats it.  The 8-bit results then convert to float as the uncompressed
// formats do.
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

// BC7's partition patterns and anchor texels, as the format defines them.
// Two subsets: a 16-bit mask of the texels in subset 1 (bit t = texel t, row
// major).  Three subsets: texel t's subset in bits 2t..2t+1.
__device__ const uint16_t kBc7Part2[64] = {
    0xCCCC, 0x8888, 0xEEEE, 0xECC8, 0xC880, 0xFEEC, 0xFEC8, 0xEC80, 0xC800, 0xFFEC, 0xFE80, 0xE800, 0xFFE8,
    0xFF00, 0xFFF0, 0xF000, 0xF710, 0x008E, 0x7100, 0x08CE, 0x008C, 0x7310, 0x3100, 0x8CCE, 0x088C, 0x3110,
    0x6666, 0x366C, 0x17E8, 0x0FF0, 0x718E, 0x399C, 0xAAAA, 0xF0F0, 0x5A5A, 0x33CC, 0x3C3C, 0x55AA, 0x9696,
    0xA55A, 0x73CE, 0x13C8, 0x324C, 0x3BDC, 0x6996, 0xC33C, 0x9966, 0x0660, 0x0272, 0x04E4, 0x4E40, 0x2720,
    0xC936, 0x936C, 0x39C6, 0x639C, 0x9336, 0x9CC6, 0x817E, 0xE718, 0xCCF0, 0x0FCC, 0x7744, 0xEE22};
__device__ const uint32_t kBc7Part3[64] = {
    0xAA685050u, 0x6A5A5040u, 0x5A5A4200u, 0x5450A0A8u, 0xA5A50000u, 0xA0A05050u, 0x5555A0A0u, 0x5A5A5050u,
    0xAA550000u, 0xAA555500u, 0xAAAA5500u, 0x90909090u, 0x94949494u, 0xA4A4A4A4u, 0xA9A59450u, 0x2A0A4250u,
    0xA5945040u, 0x0A425054u, 0xA5A5A500u, 0x55A0A0A0u, 0xA8A85454u, 0x6A6A4040u, 0xA4A45000u, 0x1A1A0500u,
    0x0050A4A4u, 0xAAA59090u, 0x14696914u, 0x69691400u, 0xA08585A0u, 0xAA821414u, 0x50A4A450u, 0x6A5A0200u,
    0xA9A58000u, 0x5090A0A8u, 0xA8A09050u, 0x24242424u, 0x00AA5500u, 0x24924924u, 0x24499224u, 0x50A50A50u,
    0x500AA550u, 0xAAAA4444u, 0x66660000u, 0xA5A0A5A0u, 0x50A050A0u, 0x69286928u, 0x44AAAA44u, 0x66666600u,
    0xAA444444u, 0x54A854A8u, 0x95809580u, 0x96969600u, 0xA85454A8u, 0x80959580u, 0xAA141414u, 0x96960000u,
    0xAAAA1414u, 0xA05050A0u, 0xA0A5A5A0u, 0x96000000u, 0x40804080u, 0xA9A8A9A8u, 0xAAAAAA44u, 0x2A4A5254u};
// the anchor texel of subset 1 (two subsets), of subsets 1 and 2 (three)
__device__ const uint8_t kBc7Anchor2[64] = {
    15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2, 8, 2, 2, 8, 8, 15, 2, 8, 2, 2,
    8, 8, 2, 2, 15, 15, 6, 8, 2, 8, 15, 15, 2, 8, 2, 2, 2, 15, 15, 6, 6, 2, 6, 8, 15, 15, 2, 2, 15, 15,
    15, 15, 15, 2, 2, 15};
__device__ const uint8_t kBc7Anchor3a[64] = {
    3, 3, 15, 15, 8, 3, 15, 15, 8, 8, 6, 6, 6, 5, 3, 3, 3, 3, 8, 15, 3, 3, 6, 10, 5, 8, 8, 6, 8, 5, 15, 15,
    8, 15, 3, 5, 6, 10, 8, 15, 15, 3, 15, 5, 15, 15, 15, 15, 3, 15, 5, 5, 5, 8, 5, 10, 5, 10, 8, 13, 15, 12, 3, 3};
__device__ const uint8_t kBc7Anchor3b[64] = {
    15, 8, 8, 3, 15, 15, 3, 8, 15, 15, 15, 15, 15, 15, 15, 8, 15, 8, 15, 3, 15, 8, 15, 8, 3, 15, 6, 10, 15, 15, 10, 8,
    15, 3, 15, 10, 10, 8, 9, 10, 6, 15, 8, 15, 3, 6, 6, 8, 15, 3, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 3, 15, 15, 8};
// per mode: subsets, partition bits, rotation bits, index-selection bits,
// colour bits, alpha bits, p-bit per endpoint, p-bit per subset, index bits,
// second index bits
__device__ const uint8_t kBc7Mode[8][10] = {
    {3, 4, 0, 0, 4, 0, 1, 0, 3, 0}, {2, 6, 0, 0, 6, 0, 0, 1, 3, 0}, {3, 6, 0, 0, 5, 0, 0, 0, 2, 0},
    {2, 6, 0, 0, 7, 0, 1, 0, 2, 0}, {1, 0, 2, 1, 5, 6, 0, 0, 2, 3}, {1, 0, 2, 0, 7, 8, 0, 0, 2, 2},
    {1, 0, 0, 0, 7, 7, 1, 0, 4, 0}, {2, 6, 0, 0, 5, 5, 1, 0, 2, 0}};
__device__ const uint8_t kBc7W2[4] = {0, 21, 43, 64};
__device__ const uint8_t kBc7W3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
__device__ const uint8_t kBc7W4[16] = {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64};

// Little-endian bit reader over one 128-bit block.
struct Bits128 {
    uint64_t lo, hi;
    uint32_t pos;
    __device__ __forceinline__ uint32_t get(uint32_t n) {
        uint64_t v;
        if (pos >= 64) v = hi >> (pos - 64);
        else if (pos + n <= 64) v = lo >> pos;
        else v = (lo >> pos) | (hi << (64 - pos));
        pos += n;
        return (uint32_t)v & ((1u << n) - 1u);
    }
};

__device__ __forceinline__ uint32_t bc7_weight(uint32_t bits, uint32_t i) {
    return bits == 2 ? kBc7W2[i] : bits == 3 ? kBc7W3[i] : kBc7W4[i];
}

// The 16 texels of a BC7 block (b 16-byte aligned) as packed RGBA8.
__device__ void bc7_block(const uint8_t* b, uint32_t rgba[16]) {
    const ulonglong2 q = __ldg(reinterpret_cast<const ulonglong2*>(b));
    const uint32_t b0 = (uint32_t)(q.x & 0xFFu);
    if (b0 == 0) {
        for (int t = 0; t < 16; ++t) rgba[t] = 0u;
        return;
    }
    const uint32_t mode = (uint32_t)__ffs(b0) - 1u;
    const uint8_t* m = kBc7Mode[mode];
    const uint32_t ns = m[0], cb = m[4], ab = m[5], epb = m[6], spb = m[7], ib = m[8], ib2 = m[9];
    Bits128 r{q.x, q.y, mode + 1u};
    const uint32_t part = r.get(m[1]), rot = r.get(m[2]), isb = r.get(m[3]);
    uint32_t e[6][4];
    for (int ch = 0; ch < 3; ++ch)
        for (uint32_t i = 0; i < 2 * ns; ++i) e[i][ch] = r.get(cb);
    for (uint32_t i = 0; i < 2 * ns; ++i) e[i][3] = ab ? r.get(ab) : 255u;
    if (epb) {
        for (uint32_t i = 0; i < 2 * ns; ++i) {
            const uint32_t p = r.get(1);
            for (int ch = 0; ch < (ab ? 4 : 3); ++ch) e[i][ch] = (e[i][ch] << 1) | p;
        }
    }
    if (spb) {
        for (uint32_t s = 0; s < ns; ++s) {
            const uint32_t p = r.get(1);
            for (uint32_t i = 2 * s; i < 2 * s + 2; ++i)
                for (int ch = 0; ch < 3; ++ch) e[i][ch] = (e[i][ch] << 1) | p;
        }
    }
    const uint32_t nc = cb + epb + spb, na = ab + epb;
    for (uint32_t i = 0; i < 2 * ns; ++i) {
        for (int ch = 0; ch < 3; ++ch) e[i][ch] = ((e[i][ch] << (8 - nc)) | (e[i][ch] >> (2 * nc - 8))) & 255u;
        if (ab) e[i][3] = ((e[i][3] << (8 - na)) | (e[i][3] >> (2 * na - 8))) & 255u;
    }
    const uint32_t a1 = ns == 2 ? kBc7Anchor2[part] : ns == 3 ? kBc7Anchor3a[part] : 16u;
    const uint32_t a2 = ns == 3 ? kBc7Anchor3b[part] : 16u;
    uint32_t i1[16], i2[16];
    for (uint32_t t = 0; t < 16; ++t) i1[t] = r.get(ib - (t == 0 || t == a1 || t == a2));
    for (uint32_t t = 0; t < 16; ++t) i2[t] = ib2 ? r.get(ib2 - (t == 0)) : 0u;
    for (uint32_t t = 0; t < 16; ++t) {
        const uint32_t s = ns == 2 ? (kBc7Part2[part] >> t) & 1u : ns == 3 ? (kBc7Part3[part] >> (2 * t)) & 3u : 0u;
        // colour and alpha weights: one index set, or (modes 4, 5) two, swapped by the selection bit
        uint32_t wc, wa;
        if (!ib2) {
            wc = wa = bc7_weight(ib, i1[t]);
        } else if (isb) {
            wc = bc7_weight(ib2, i2[t]);
            wa = bc7_weight(ib, i1[t]);
        } else {
            wc = bc7_weight(ib, i1[t]);
            wa = bc7_weight(ib2, i2[t]);
        }
        uint32_t c[4];
        for (int ch = 0; ch < 4; ++ch) {
            const uint32_t w = ch < 3 ? wc : wa;
            c[ch] = ((64u - w) * e[2 * s][ch] + w * e[2 * s + 1][ch] + 32u) >> 6;
        }
        if (rot) {
            const uint32_t tmp = c[3];
            c[3] = c[rot - 1];
            c[rot - 1] = tmp;
        }
        rgba[t] = c[0] | (c[1] << 8) | (c[2] << 16) | (c[3] << 24);
    }
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
    if (format == WF_TEXTURE_BC7 || format == WF_TEXTURE_BC7_SRGB) {
        bc7_block(b, rgba);
    } else if (format == WF_TEXTURE_BC4 || format == WF_TEXTURE_BC5) {
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
