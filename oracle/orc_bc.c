/* orc_bc.c — oracle BC1-BC5 block decoder.  TEST INFRASTRUCTURE ONLY: the
 * checker for the GPU library's block decoder (wavefrontpathtracing_gb300/
 * csrc/wf_texture.cu), following the same definition of Microsoft's BC1-BC5
 * formats: RGB565 endpoints expanded by bit replication, BC1 four-colour mode
 * when c0 > c1 (or always inside BC2 / BC3) else three colours and
 * transparent black, BC4 eight-value mode when e0 > e1 else six values plus
 * 0 and 255, every interpolation rounded to nearest in integers.  The
 * reference decodes these blocks in the GPU's sampler hardware
 * (asset_loader.cpp:179-206), which no test here can run: the decoder is
 * pinned by the formats' known answers (tests/test_image_decode.py). */
#include <stdint.h>
#include <string.h>

enum { BC1 = 4, BC1S = 5, BC2 = 6, BC2S = 7, BC3 = 8, BC3S = 9, BC4 = 10, BC5 = 11 };

static void bc1_palette(const uint8_t* b, int four, uint8_t pal[4][4]) {
    const unsigned c0 = b[0] | (b[1] << 8), c1 = b[2] | (b[3] << 8);
    const unsigned cs[2] = {c0, c1};
    unsigned e[2][3];
    for (int k = 0; k < 2; ++k) {
        const unsigned r = (cs[k] >> 11) & 31u, g = (cs[k] >> 5) & 63u, bl = cs[k] & 31u;
        e[k][0] = (r << 3) | (r >> 2);
        e[k][1] = (g << 2) | (g >> 4);
        e[k][2] = (bl << 3) | (bl >> 2);
    }
    const int fourc = four || c0 > c1;
    for (int ch = 0; ch < 3; ++ch) {
        pal[0][ch] = (uint8_t)e[0][ch];
        pal[1][ch] = (uint8_t)e[1][ch];
        if (fourc) {
            pal[2][ch] = (uint8_t)((2u * e[0][ch] + e[1][ch] + 1u) / 3u);
            pal[3][ch] = (uint8_t)((e[0][ch] + 2u * e[1][ch] + 1u) / 3u);
        } else {
            pal[2][ch] = (uint8_t)((e[0][ch] + e[1][ch] + 1u) / 2u);
            pal[3][ch] = 0;
        }
    }
    for (int i = 0; i < 4; ++i) pal[i][3] = (!fourc && i == 3) ? 0 : 255;
}

static void bc4_palette(const uint8_t* b, uint8_t v[8]) {
    const unsigned e0 = b[0], e1 = b[1];
    v[0] = (uint8_t)e0;
    v[1] = (uint8_t)e1;
    if (e0 > e1) {
        for (unsigned i = 2; i < 8; ++i) v[i] = (uint8_t)(((8u - i) * e0 + (i - 1u) * e1 + 3u) / 7u);
    } else {
        for (unsigned i = 2; i < 6; ++i) v[i] = (uint8_t)(((6u - i) * e0 + (i - 1u) * e1 + 2u) / 5u);
        v[6] = 0;
        v[7] = 255;
    }
}

static unsigned bc4_index(const uint8_t* b, int t) {
    uint64_t bits = 0;
    for (int k = 0; k < 6; ++k) bits |= (uint64_t)b[2 + k] << (8 * k);
    return (unsigned)((bits >> (3 * t)) & 7u);
}

/* Decodes a w x h image of BC blocks (as a DDS file stores them) into RGBA8;
 * returns 0, or -1 for a format it does not know. */
int orc_decode_bc(uint32_t format, const uint8_t* blocks, uint32_t w, uint32_t h, uint8_t* rgba) {
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    const int small = format == BC1 || format == BC1S || format == BC4;
    if (format < BC1 || format > BC5) return -1;
    for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx) {
            const uint8_t* b = blocks + ((size_t)by * bw + bx) * (small ? 8u : 16u);
            uint8_t px[16][4];
            if (format == BC4 || format == BC5) {
                uint8_t r[8], g[8];
                bc4_palette(b, r);
                if (format == BC5) bc4_palette(b + 8, g);
                for (int t = 0; t < 16; ++t) {
                    px[t][0] = r[bc4_index(b, t)];
                    px[t][1] = format == BC5 ? g[bc4_index(b + 8, t)] : 0;
                    px[t][2] = 0;
                    px[t][3] = 255;
                }
            } else {
                const uint8_t* cb = small ? b : b + 8;
                uint8_t pal[4][4];
                bc1_palette(cb, !small, pal);
                const uint32_t idx = cb[4] | (cb[5] << 8) | (cb[6] << 16) | ((uint32_t)cb[7] << 24);
                for (int t = 0; t < 16; ++t) memcpy(px[t], pal[(idx >> (2 * t)) & 3u], 4);
                if (format == BC2 || format == BC2S) {
                    for (int t = 0; t < 16; ++t) px[t][3] = (uint8_t)(((b[t >> 1] >> (4 * (t & 1))) & 15u) * 17u);
                } else if (format == BC3 || format == BC3S) {
                    uint8_t a[8];
                    bc4_palette(b, a);
                    for (int t = 0; t < 16; ++t) px[t][3] = a[bc4_index(b, t)];
                }
            }
            for (int t = 0; t < 16; ++t) {
                const uint32_t x = bx * 4 + (t & 3), y = by * 4 + (t >> 2);
                if (x < w && y < h) memcpy(rgba + 4 * ((size_t)y * w + x), px[t], 4);
            }
        }
    return 0;
}
