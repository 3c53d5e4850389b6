/* orc_bc.c — oracle BC1-BC5 and BC7 block decoder.  TEST INFRASTRUCTURE ONLY: the
 * checker for the GPU library's block decoder (wavefrontpathtracing_gb300/
 * csrc/wf_texture.cu), following the same definition of Microsoft's BC1-BC5
 * formats: RGB565 endpoints expanded by bit replication, BC1 four-colour mode
 * when c0 > c1 (or always inside BC2 / BC3) else three colours and
 * transparent black, BC4 eight-value mode when e0 > e1 else six values plus
 * 0 and 255, every interpolation rounded to nearest in integers.  The
 * reference decodes these blocks in the GPU's sampler hardware
 * (asset_loader.cpp:179-206, d3d12_backend.cpp:725-740 maps them to DXGI's
 * BC formats); the GPU tests decode the same blocks in this GPU's texture
 * sampler as the checker of both decoders (BC7 exactly, its values being
 * exact 8-bit integers by definition), and the formats' known answers pin
 * them on the CPU (tests/test_image_decode.py).
 *
 * BC7 follows Microsoft's published BC7 format: mode = lowest set bit of the
 * first byte (none: reserved, transparent black); fields in bit order mode,
 * partition, rotation, index selection, R of every endpoint, G, B, A, p-bits,
 * primary indices (anchor texels one bit short), secondary indices; endpoints
 * expanded by bit replication after their p-bit; texels interpolated as
 * ((64 - w) e0 + w e1 + 32) >> 6 with the format's 2/3/4-bit weights. */
#include <stdint.h>
#include <string.h>

enum { BC1 = 4, BC1S = 5, BC2 = 6, BC2S = 7, BC3 = 8, BC3S = 9, BC4 = 10, BC5 = 11, BC7 = 12, BC7S = 13 };

/* BC7 partition patterns, texel by texel (row major): two subsets, three. */
static const uint8_t P2[64][16] = {
#define M(x) {(x)>>0&1,(x)>>1&1,(x)>>2&1,(x)>>3&1,(x)>>4&1,(x)>>5&1,(x)>>6&1,(x)>>7&1, \
              (x)>>8&1,(x)>>9&1,(x)>>10&1,(x)>>11&1,(x)>>12&1,(x)>>13&1,(x)>>14&1,(x)>>15&1}
    M(0xCCCC), M(0x8888), M(0xEEEE), M(0xECC8), M(0xC880), M(0xFEEC), M(0xFEC8), M(0xEC80),
    M(0xC800), M(0xFFEC), M(0xFE80), M(0xE800), M(0xFFE8), M(0xFF00), M(0xFFF0), M(0xF000),
    M(0xF710), M(0x008E), M(0x7100), M(0x08CE), M(0x008C), M(0x7310), M(0x3100), M(0x8CCE),
    M(0x088C), M(0x3110), M(0x6666), M(0x366C), M(0x17E8), M(0x0FF0), M(0x718E), M(0x399C),
    M(0xAAAA), M(0xF0F0), M(0x5A5A), M(0x33CC), M(0x3C3C), M(0x55AA), M(0x9696), M(0xA55A),
    M(0x73CE), M(0x13C8), M(0x324C), M(0x3BDC), M(0x6996), M(0xC33C), M(0x9966), M(0x0660),
    M(0x0272), M(0x04E4), M(0x4E40), M(0x2720), M(0xC936), M(0x936C), M(0x39C6), M(0x639C),
    M(0x9336), M(0x9CC6), M(0x817E), M(0xE718), M(0xCCF0), M(0x0FCC), M(0x7744), M(0xEE22)
#undef M
};
static const uint8_t P3[64][16] = {
    {0,0,1,1,0,0,1,1,0,2,2,1,2,2,2,2}, {0,0,0,1,0,0,1,1,2,2,1,1,2,2,2,1},
    {0,0,0,0,2,0,0,1,2,2,1,1,2,2,1,1}, {0,2,2,2,0,0,2,2,0,0,1,1,0,1,1,1},
    {0,0,0,0,0,0,0,0,1,1,2,2,1,1,2,2}, {0,0,1,1,0,0,1,1,0,0,2,2,0,0,2,2},
    {0,0,2,2,0,0,2,2,1,1,1,1,1,1,1,1}, {0,0,1,1,0,0,1,1,2,2,1,1,2,2,1,1},
    {0,0,0,0,0,0,0,0,1,1,1,1,2,2,2,2}, {0,0,0,0,1,1,1,1,1,1,1,1,2,2,2,2},
    {0,0,0,0,1,1,1,1,2,2,2,2,2,2,2,2}, {0,0,1,2,0,0,1,2,0,0,1,2,0,0,1,2},
    {0,1,1,2,0,1,1,2,0,1,1,2,0,1,1,2}, {0,1,2,2,0,1,2,2,0,1,2,2,0,1,2,2},
    {0,0,1,1,0,1,1,2,1,1,2,2,1,2,2,2}, {0,0,1,1,2,0,0,1,2,2,0,0,2,2,2,0},
    {0,0,0,1,0,0,1,1,0,1,1,2,1,1,2,2}, {0,1,1,1,0,0,1,1,2,0,0,1,2,2,0,0},
    {0,0,0,0,1,1,2,2,1,1,2,2,1,1,2,2}, {0,0,2,2,0,0,2,2,0,0,2,2,1,1,1,1},
    {0,1,1,1,0,1,1,1,0,2,2,2,0,2,2,2}, {0,0,0,1,0,0,0,1,2,2,2,1,2,2,2,1},
    {0,0,0,0,0,0,1,1,0,1,2,2,0,1,2,2}, {0,0,0,0,1,1,0,0,2,2,1,0,2,2,1,0},
    {0,1,2,2,0,1,2,2,0,0,1,1,0,0,0,0}, {0,0,1,2,0,0,1,2,1,1,2,2,2,2,2,2},
    {0,1,1,0,1,2,2,1,1,2,2,1,0,1,1,0}, {0,0,0,0,0,1,1,0,1,2,2,1,1,2,2,1},
    {0,0,2,2,1,1,0,2,1,1,0,2,0,0,2,2}, {0,1,1,0,0,1,1,0,2,0,0,2,2,2,2,2},
    {0,0,1,1,0,1,2,2,0,1,2,2,0,0,1,1}, {0,0,0,0,2,0,0,0,2,2,1,1,2,2,2,1},
    {0,0,0,0,0,0,0,2,1,1,2,2,1,2,2,2}, {0,2,2,2,0,0,2,2,0,0,1,2,0,0,1,1},
    {0,0,1,1,0,0,1,2,0,0,2,2,0,2,2,2}, {0,1,2,0,0,1,2,0,0,1,2,0,0,1,2,0},
    {0,0,0,0,1,1,1,1,2,2,2,2,0,0,0,0}, {0,1,2,0,1,2,0,1,2,0,1,2,0,1,2,0},
    {0,1,2,0,2,0,1,2,1,2,0,1,0,1,2,0}, {0,0,1,1,2,2,0,0,1,1,2,2,0,0,1,1},
    {0,0,1,1,1,1,2,2,2,2,0,0,0,0,1,1}, {0,1,0,1,0,1,0,1,2,2,2,2,2,2,2,2},
    {0,0,0,0,0,0,0,0,2,1,2,1,2,1,2,1}, {0,0,2,2,1,1,2,2,0,0,2,2,1,1,2,2},
    {0,0,2,2,0,0,1,1,0,0,2,2,0,0,1,1}, {0,2,2,0,1,2,2,1,0,2,2,0,1,2,2,1},
    {0,1,0,1,2,2,2,2,2,2,2,2,0,1,0,1}, {0,0,0,0,2,1,2,1,2,1,2,1,2,1,2,1},
    {0,1,0,1,0,1,0,1,0,1,0,1,2,2,2,2}, {0,2,2,2,0,1,1,1,0,2,2,2,0,1,1,1},
    {0,0,0,2,1,1,1,2,0,0,0,2,1,1,1,2}, {0,0,0,0,2,1,1,2,2,1,1,2,2,1,1,2},
    {0,2,2,2,0,1,1,1,0,1,1,1,0,2,2,2}, {0,0,0,2,1,1,1,2,1,1,1,2,0,0,0,2},
    {0,1,1,0,0,1,1,0,0,1,1,0,2,2,2,2}, {0,0,0,0,0,0,0,0,2,1,1,2,2,1,1,2},
    {0,1,1,0,0,1,1,0,2,2,2,2,2,2,2,2}, {0,0,2,2,0,0,1,1,0,0,1,1,0,0,2,2},
    {0,0,2,2,1,1,2,2,1,1,2,2,0,0,2,2}, {0,0,0,0,0,0,0,0,0,0,0,0,2,1,1,2},
    {0,0,0,2,0,0,0,1,0,0,0,2,0,0,0,1}, {0,2,2,2,1,2,2,2,0,2,2,2,1,2,2,2},
    {0,1,0,1,2,2,2,2,2,2,2,2,2,2,2,2}, {0,1,1,1,2,0,1,1,2,2,0,1,2,2,2,0}};
/* anchor texels: subset 1 of two; subsets 1 and 2 of three */
static const uint8_t A2[64] = {15,15,15,15,15,15,15,15, 15,15,15,15,15,15,15,15, 15,2,8,2,2,8,8,15, 2,8,2,2,8,8,2,2,
                               15,15,6,8,2,8,15,15, 2,8,2,2,2,15,15,6, 6,2,6,8,15,15,2,2, 15,15,15,15,15,2,2,15};
static const uint8_t A3a[64] = {3,3,15,15,8,3,15,15, 8,8,6,6,6,5,3,3, 3,3,8,15,3,3,6,10, 5,8,8,6,8,5,15,15,
                                8,15,3,5,6,10,8,15, 15,3,15,5,15,15,15,15, 3,15,5,5,5,8,5,10, 5,10,8,13,15,12,3,3};
static const uint8_t A3b[64] = {15,8,8,3,15,15,3,8, 15,15,15,15,15,15,15,8, 15,8,15,3,15,8,15,8, 3,15,6,10,15,15,10,8,
                                15,3,15,10,10,8,9,10, 6,15,8,15,3,6,6,8, 15,3,15,15,15,15,15,15, 15,15,15,15,3,15,15,8};
static const uint8_t W2[4] = {0, 21, 43, 64};
static const uint8_t W3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
static const uint8_t W4[16] = {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64};

typedef struct { int ns, pb, rb, isb, cb, ab, epb, spb, ib, ib2; } Bc7Mode;
static const Bc7Mode MODES[8] = {
    {3, 4, 0, 0, 4, 0, 1, 0, 3, 0}, {2, 6, 0, 0, 6, 0, 0, 1, 3, 0}, {3, 6, 0, 0, 5, 0, 0, 0, 2, 0},
    {2, 6, 0, 0, 7, 0, 1, 0, 2, 0}, {1, 0, 2, 1, 5, 6, 0, 0, 2, 3}, {1, 0, 2, 0, 7, 8, 0, 0, 2, 2},
    {1, 0, 0, 0, 7, 7, 1, 0, 4, 0}, {2, 6, 0, 0, 5, 5, 1, 0, 2, 0}};

/* n bits of the 128-bit block b starting at bit *pos (bit 0 = lowest bit of b[0]) */
static unsigned take(const uint8_t* b, int* pos, int n) {
    unsigned v = 0;
    for (int k = 0; k < n; ++k, ++*pos) v |= (unsigned)((b[*pos >> 3] >> (*pos & 7)) & 1) << k;
    return v;
}

static unsigned weight(int bits, unsigned i) { return bits == 2 ? W2[i] : bits == 3 ? W3[i] : W4[i]; }

static void bc7_block(const uint8_t* b, uint8_t px[16][4]) {
    int mode = 0;
    while (mode < 8 && !(b[0] >> mode & 1)) ++mode;
    if (mode == 8) {
        memset(px, 0, 64);
        return;
    }
    const Bc7Mode m = MODES[mode];
    int pos = mode + 1;
    const unsigned part = take(b, &pos, m.pb), rot = take(b, &pos, m.rb), isb = take(b, &pos, m.isb);
    unsigned e[6][4];
    for (int ch = 0; ch < 4; ++ch)
        for (int i = 0; i < 2 * m.ns; ++i) {
            if (ch < 3) e[i][ch] = take(b, &pos, m.cb);
            else e[i][ch] = m.ab ? take(b, &pos, m.ab) : 255u;
        }
    for (int i = 0; i < 2 * m.ns && m.epb; ++i) {
        const unsigned p = take(b, &pos, 1);
        for (int ch = 0; ch < (m.ab ? 4 : 3); ++ch) e[i][ch] = e[i][ch] << 1 | p;
    }
    for (int s = 0; s < m.ns && m.spb; ++s) {
        const unsigned p = take(b, &pos, 1);
        for (int ch = 0; ch < 3; ++ch) {
            e[2 * s][ch] = e[2 * s][ch] << 1 | p;
            e[2 * s + 1][ch] = e[2 * s + 1][ch] << 1 | p;
        }
    }
    const int nc = m.cb + m.epb + m.spb, na = m.ab + m.epb;
    for (int i = 0; i < 2 * m.ns; ++i)
        for (int ch = 0; ch < 4; ++ch) {
            const int n = ch < 3 ? nc : na;
            if (ch == 3 && !m.ab) continue;
            e[i][ch] = ((e[i][ch] << (8 - n)) | (e[i][ch] >> (2 * n - 8))) & 255u;
        }
    unsigned idx[16], idx2[16];
    for (int t = 0; t < 16; ++t) {
        int anchor = t == 0;
        if (m.ns == 2) anchor |= t == A2[part];
        if (m.ns == 3) anchor |= t == A3a[part] || t == A3b[part];
        idx[t] = take(b, &pos, m.ib - anchor);
    }
    for (int t = 0; t < 16; ++t) idx2[t] = m.ib2 ? take(b, &pos, m.ib2 - (t == 0)) : 0;
    for (int t = 0; t < 16; ++t) {
        const int s = m.ns == 1 ? 0 : m.ns == 2 ? P2[part][t] : P3[part][t];
        unsigned wc = weight(m.ib, idx[t]), wa = wc;
        if (m.ib2) {
            if (isb) {
                wc = weight(m.ib2, idx2[t]);
                wa = weight(m.ib, idx[t]);
            } else {
                wa = weight(m.ib2, idx2[t]);
            }
        }
        unsigned c[4];
        for (int ch = 0; ch < 4; ++ch) {
            const unsigned w = ch < 3 ? wc : wa;
            c[ch] = ((64u - w) * e[2 * s][ch] + w * e[2 * s + 1][ch] + 32u) >> 6;
        }
        if (rot) {
            const unsigned tmp = c[3];
            c[3] = c[rot - 1];
            c[rot - 1] = tmp;
        }
        for (int ch = 0; ch < 4; ++ch) px[t][ch] = (uint8_t)c[ch];
    }
}

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
    if (format < BC1 || format > BC7S) return -1;
    for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx) {
            const uint8_t* b = blocks + ((size_t)by * bw + bx) * (small ? 8u : 16u);
            uint8_t px[16][4];
            if (format == BC7 || format == BC7S) {
                bc7_block(b, px);
            } else if (format == BC4 || format == BC5) {
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
