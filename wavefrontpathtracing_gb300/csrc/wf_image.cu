// wf_image.cu — the image files the reference's asset loader reads
// (core/assets/asset_loader.cpp:56-206: .jpg / .jpeg through stbi_load, .hdr
// through stbi_loadf, .dds through its own header parser, dds.h), decoded on
// the host for wf_texture_create.  Host code only; written from the formats'
// specifications:
//   JPEG  ITU-T T.81 (1992): baseline and extended sequential (SOF0 / SOF1)
//         and progressive (SOF2) Huffman coding, 1 or 3 components, sampling
//         factors 1-2, restart intervals; inverse DCT in double precision;
//         chroma upsampled with the triangle filter of the JFIF convention
//         (weights 3/4, 1/4 per axis, libjpeg's "fancy" upsampling);
//         YCbCr -> RGB by JFIF's equations (ITU-T T.871).  Output RGBA8.
//   HDR   Greg Ward's Radiance RGBE: header, "-Y h +X w" resolution, scanlines
//         flat or with the 2-2-width run-length encoding; RGBE -> float as
//         mantissa * 2^(e - 136).  Output RGBA32F (alpha 1).
//   PNG   PNG (ISO/IEC 15948): zlib / DEFLATE (RFC 1950 / 1951: stored,
//         fixed and dynamic Huffman blocks), the five scanline filters,
//         Adam7 interlacing, colour types 0 / 2 / 3 / 4 / 6 at every bit
//         depth the format allows, tRNS transparency; 16-bit samples keep
//         their high byte (as the reference's stbi_load with 4 channels,
//         asset_loader.cpp:109).  Output RGBA8.
//   DDS   the DirectDraw Surface header (with or without the DX10 extension):
//         RGBA8, RG8, RGBA32F texels or BC1-BC5 / BC7 blocks of the top mip
//         level as stored (BC blocks are decoded on the GPU by
//         wf_texture_create).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wf.h"
#include "wf_kernels.h"

namespace wf {
namespace {

// ------------------------------------------------------------------ JPEG
struct Huff {
    // canonical code tables (T.81 Annex C / F.2.2.3)
    int maxcode[18], valptr[17], mincode[17];
    uint8_t vals[256];
    bool present = false;
};

struct Comp {
    int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
    int bw = 0, bh = 0;            // blocks per row / column (MCU-padded)
    int cw = 0, ch = 0;            // component size in samples
    std::vector<int16_t> coef;     // bw * bh * 64, zig-zag order
    int dcpred = 0;
};

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct Jpeg {
    const uint8_t* d;
    size_t n, pos = 0;
    uint16_t qt[4][64] = {};
    Huff dc[4], ac[4];
    std::vector<Comp> comp;
    int width = 0, height = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0, restart = 0;
    bool progressive = false;
    int eobrun = 0;
    // bit reader over entropy-coded data (0xFF00 stuffing, markers end the data)
    uint32_t bits = 0;
    int nbits = 0;
    bool hit_marker = false;
    std::string err;

    int u8() { return pos < n ? d[pos++] : (err = "truncated JPEG", 0); }
    int u16() { int a = u8(); return (a << 8) | u8(); }

    void reset_bits() { bits = 0; nbits = 0; hit_marker = false; }
    int bit() {
        if (nbits == 0) {
            int b = 0;
            if (!hit_marker && pos < n) {
                b = d[pos];
                if (b == 0xFF) {
                    const int m = pos + 1 < n ? d[pos + 1] : 0;
                    if (m == 0x00) { pos += 2; }
                    else { hit_marker = true; b = 0; }   // a marker: feed zeros
                } else {
                    pos++;
                }
            }
            bits = (uint32_t)b;
            nbits = 8;
        }
        nbits--;
        return (bits >> nbits) & 1;
    }
    int getbits(int k) { int v = 0; for (int i = 0; i < k; ++i) v = (v << 1) | bit(); return v; }
    // F.2.2.1 EXTEND: the value of an s-bit magnitude category
    int receive_extend(int s) {
        if (s == 0) return 0;
        int v = getbits(s);
        return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v;
    }
    int decode(const Huff& h) {
        int code = bit();
        for (int l = 1; l <= 16; ++l) {
            if (h.maxcode[l] >= 0 && code <= h.maxcode[l]) return h.vals[h.valptr[l] + code - h.mincode[l]];
            code = (code << 1) | bit();
        }
        err = "bad Huffman code";
        return 0;
    }

    bool read_dht(int len) {
        size_t end = pos + len - 2;
        while (pos < end && err.empty()) {
            const int tc = u8();
            const int cls = tc >> 4, id = tc & 15;
            if (id > 3 || cls > 1) { err = "bad DHT"; return false; }
            Huff& h = cls ? ac[id] : dc[id];
            int counts[17] = {0}, total = 0;
            for (int l = 1; l <= 16; ++l) { counts[l] = u8(); total += counts[l]; }
            if (total > 256) { err = "bad DHT"; return false; }
            for (int i = 0; i < total; ++i) h.vals[i] = (uint8_t)u8();
            int code = 0, k = 0;
            for (int l = 1; l <= 16; ++l) {
                h.valptr[l] = k;
                h.mincode[l] = code;
                code += counts[l];
                k += counts[l];
                h.maxcode[l] = counts[l] ? code - 1 : -1;
                code <<= 1;
            }
            h.maxcode[17] = 0x7FFFFFFF;
            h.present = true;
        }
        return err.empty();
    }

    bool read_dqt(int len) {
        size_t end = pos + len - 2;
        while (pos < end && err.empty()) {
            const int pq = u8();
            const int id = pq & 15, prec = pq >> 4;
            if (id > 3) { err = "bad DQT"; return false; }
            for (int i = 0; i < 64; ++i) qt[id][i] = (uint16_t)(prec ? u16() : u8());   // zig-zag order
        }
        return err.empty();
    }

    bool read_sof() {
        u16();
        if (u8() != 8) { err = "only 8-bit JPEG samples are supported"; return false; }
        height = u16();
        width = u16();
        const int nc = u8();
        if (nc != 1 && nc != 3) { err = "JPEG with 1 or 3 components expected"; return false; }
        if (width <= 0 || height <= 0 || width > 16384 || height > 16384) { err = "bad JPEG size"; return false; }
        comp.resize(nc);
        for (Comp& c : comp) {
            c.id = u8();
            const int hv = u8();
            c.h = hv >> 4;
            c.v = hv & 15;
            c.tq = u8();
            if (c.h < 1 || c.h > 2 || c.v < 1 || c.v > 2 || c.tq > 3) { err = "unsupported JPEG sampling"; return false; }
            hmax = std::max(hmax, c.h);
            vmax = std::max(vmax, c.v);
        }
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        for (Comp& c : comp) {
            c.bw = mcux * c.h;
            c.bh = mcuy * c.v;
            c.cw = (width * c.h + hmax - 1) / hmax;
            c.ch = (height * c.v + vmax - 1) / vmax;
            c.coef.assign((size_t)c.bw * c.bh * 64, 0);
        }
        return err.empty();
    }

    // one block of a sequential scan (F.2.2)
    void block_baseline(Comp& c, int16_t* z) {
        const int t = decode(dc[c.td]);
        c.dcpred += receive_extend(t);
        z[0] = (int16_t)c.dcpred;
        for (int k = 1; k < 64;) {
            const int rs = decode(ac[c.ta]);
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r != 15) break;
                k += 16;
                continue;
            }
            k += r;
            if (k > 63) { err = "bad JPEG AC run"; return; }
            z[k++] = (int16_t)receive_extend(s);
        }
    }
    // progressive scans (G.1.2): DC first / refine, AC first / refine
    void block_dc(Comp& c, int16_t* z, int ah, int al) {
        if (ah == 0) {
            const int t = decode(dc[c.td]);
            c.dcpred += receive_extend(t);
            z[0] = (int16_t)(c.dcpred * (1 << al));
        } else if (bit()) {
            z[0] = (int16_t)(z[0] | (1 << al));
        }
    }
    void block_ac_first(Comp& c, int16_t* z, int ss, int se, int al) {
        if (eobrun > 0) { eobrun--; return; }
        for (int k = ss; k <= se;) {
            const int rs = decode(ac[c.ta]);
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r < 15) {
                    eobrun = (1 << r) - 1;
                    if (r) eobrun += getbits(r);
                    break;
                }
                k += 16;
                continue;
            }
            k += r;
            if (k > 63) { err = "bad JPEG AC run"; return; }
            z[k++] = (int16_t)(receive_extend(s) * (1 << al));
        }
    }
    void block_ac_refine(Comp& c, int16_t* z, int ss, int se, int al) {
        const int p1 = 1 << al, m1 = -1 * (1 << al);
        int k = ss;
        if (eobrun == 0) {
            for (; k <= se;) {
                const int rs = decode(ac[c.ta]);
                int r = rs >> 4, s = rs & 15, val = 0;
                if (s == 0) {
                    if (r < 15) {
                        eobrun = (1 << r);
                        if (r) eobrun += getbits(r);
                        break;
                    }
                } else {
                    val = bit() ? p1 : m1;
                }
                // skip r zero-history coefficients, refining the non-zero ones passed
                while (k <= se) {
                    if (z[k] != 0) {
                        if (bit() && (z[k] & p1) == 0) z[k] = (int16_t)(z[k] >= 0 ? z[k] + p1 : z[k] + m1);
                    } else {
                        if (r == 0) {
                            if (val) z[k] = (int16_t)val;
                            k++;
                            break;
                        }
                        r--;
                    }
                    k++;
                }
                if (err.size()) return;
            }
        }
        if (eobrun > 0) {
            for (; k <= se; ++k)
                if (z[k] != 0 && bit() && (z[k] & p1) == 0) z[k] = (int16_t)(z[k] >= 0 ? z[k] + p1 : z[k] + m1);
            eobrun--;
        }
    }

    bool read_sos() {
        u16();
        const int ns = u8();
        std::vector<Comp*> sc;
        for (int i = 0; i < ns; ++i) {
            const int id = u8(), t = u8();
            Comp* c = nullptr;
            for (Comp& x : comp) if (x.id == id) c = &x;
            if (!c) { err = "bad SOS component"; return false; }
            c->td = t >> 4;
            c->ta = t & 15;
            if (c->td > 3 || c->ta > 3) { err = "bad SOS table"; return false; }
            sc.push_back(c);
        }
        const int ss = u8(), se = u8(), a = u8();
        const int ah = a >> 4, al = a & 15;
        if (!progressive && (ss != 0 || se != 63)) { err = "bad sequential scan"; return false; }
        for (Comp* c : sc) c->dcpred = 0;
        eobrun = 0;
        reset_bits();
        // interleaved: MCUs of h x v blocks per component; single: the component's own blocks
        const bool single = ns == 1;
        const int ux = single ? (sc[0]->cw + 7) / 8 : mcux;
        const int uy = single ? (sc[0]->ch + 7) / 8 : mcuy;
        int todo = restart;
        for (int my = 0; my < uy && err.empty(); ++my) {
            for (int mx = 0; mx < ux && err.empty(); ++mx) {
                if (restart && todo == 0) {
                    // expect RSTn: skip to the marker, reset predictions
                    while (pos + 1 < n && !(d[pos] == 0xFF && d[pos + 1] >= 0xD0 && d[pos + 1] <= 0xD7)) pos++;
                    pos += 2;
                    for (Comp* c : sc) c->dcpred = 0;
                    eobrun = 0;
                    reset_bits();
                    todo = restart;
                }
                for (Comp* c : sc) {
                    const int bx = single ? 1 : c->h, by = single ? 1 : c->v;
                    for (int j = 0; j < by; ++j)
                        for (int i = 0; i < bx; ++i) {
                            const int bxi = single ? mx : mx * c->h + i;
                            const int byi = single ? my : my * c->v + j;
                            int16_t* z = c->coef.data() + 64ull * ((size_t)byi * c->bw + bxi);
                            if (!progressive) block_baseline(*c, z);
                            else if (ss == 0) block_dc(*c, z, ah, al);
                            else if (ah == 0) block_ac_first(*c, z, ss, se, al);
                            else block_ac_refine(*c, z, ss, se, al);
                        }
                }
                if (restart) todo--;
            }
        }
        // resume at the next marker
        while (pos + 1 < n && !(d[pos] == 0xFF && d[pos + 1] != 0x00 && !(d[pos + 1] >= 0xD0 && d[pos + 1] <= 0xD7)))
            pos++;
        return err.empty();
    }

    // dequantize + inverse DCT (A.3.3) of every block, samples of each component
    void reconstruct(std::vector<std::vector<uint8_t>>& planes) {
        struct CosTable {
            double v[8][8];
            CosTable() {
                for (int x = 0; x < 8; ++x)
                    for (int u = 0; u < 8; ++u)
                        v[x][u] = (u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * M_PI / 16.0);
            }
        };
        static const CosTable table;   // initialised once, thread-safe
        const auto& cosv = table.v;
        planes.resize(comp.size());
        for (size_t ci = 0; ci < comp.size(); ++ci) {
            Comp& c = comp[ci];
            const int pw = c.bw * 8, ph = c.bh * 8;
            std::vector<uint8_t>& p = planes[ci];
            p.assign((size_t)pw * ph, 0);
            for (int by = 0; by < c.bh; ++by)
                for (int bx = 0; bx < c.bw; ++bx) {
                    const int16_t* z = c.coef.data() + 64ull * ((size_t)by * c.bw + bx);
                    double F[64], tmp[64];
                    for (int k = 0; k < 64; ++k) F[kZigzag[k]] = (double)z[k] * qt[c.tq][k];
                    for (int y = 0; y < 8; ++y)          // rows: over u
                        for (int x = 0; x < 8; ++x) {
                            double s = 0.0;
                            for (int u = 0; u < 8; ++u) s += cosv[x][u] * F[y * 8 + u];
                            tmp[y * 8 + x] = s;
                        }
                    for (int x = 0; x < 8; ++x)          // columns: over v
                        for (int y = 0; y < 8; ++y) {
                            double s = 0.0;
                            for (int v = 0; v < 8; ++v) s += cosv[y][v] * tmp[v * 8 + x];
                            const double val = std::floor(s / 4.0 + 128.0 + 0.5);
                            p[(size_t)(by * 8 + y) * pw + bx * 8 + x] =
                                (uint8_t)(val < 0.0 ? 0 : (val > 255.0 ? 255 : val));
                        }
                }
        }
    }
};

// Triangle-filter upsampling of one component plane by (fx, fy) in {1, 2}:
// each output sample weighs its nearer input sample 3/4 and the next 1/4 per
// axis (edges repeat), the rounding of libjpeg's "fancy" upsampling.
std::vector<uint8_t> upsample(const std::vector<uint8_t>& in, int pw, int cw, int ch, int fx, int fy, int W, int H) {
    std::vector<uint8_t> out((size_t)W * H);
    auto at = [&](int x, int y) -> int {
        x = x < 0 ? 0 : (x >= cw ? cw - 1 : x);
        y = y < 0 ? 0 : (y >= ch ? ch - 1 : y);
        return in[(size_t)y * pw + x];
    };
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            int v;
            if (fx == 1 && fy == 1) {
                v = at(x, y);
            } else if (fy == 1) {           // horizontal only: 3/4 near + 1/4 far, rounding +1 / +2
                const int i = x >> 1, far = (x & 1) ? i + 1 : i - 1;
                v = (3 * at(i, y) + at(far, y) + ((x & 1) ? 2 : 1)) >> 2;
            } else if (fx == 1) {           // vertical only
                const int j = y >> 1, far = (y & 1) ? j + 1 : j - 1;
                v = (3 * at(x, j) + at(x, far) + ((y & 1) ? 2 : 1)) >> 2;
            } else {                        // both: vertical 3:1 sums, then horizontal 3:1 with weight 16
                const int i = x >> 1, j = y >> 1;
                const int fi = (x & 1) ? i + 1 : i - 1, fj = (y & 1) ? j + 1 : j - 1;
                const int near_col = 3 * at(i, j) + at(i, fj);
                const int far_col = 3 * at(fi, j) + at(fi, fj);
                v = (3 * near_col + far_col + ((x & 1) ? 7 : 8)) >> 4;
            }
            out[(size_t)y * W + x] = (uint8_t)v;
        }
    }
    return out;
}

int decode_jpeg(const uint8_t* d, size_t n, uint32_t* w, uint32_t* h, std::vector<uint8_t>& rgba, std::string& err) {
    Jpeg j;
    j.d = d;
    j.n = n;
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) { err = "not a JPEG file"; return WF_ERR_INVALID; }
    j.pos = 2;
    bool frame = false, done = false;
    while (!done && j.err.empty() && j.pos + 1 < n) {
        if (d[j.pos] != 0xFF) { j.pos++; continue; }
        const int m = d[j.pos + 1];
        j.pos += 2;
        if (m == 0xFF || m == 0x00 || (m >= 0xD0 && m <= 0xD7) || m == 0x01) continue;
        if (m == 0xD9) { done = true; break; }
        if (m == 0xC4) { j.read_dht(j.u16()); continue; }
        if (m == 0xDB) { j.read_dqt(j.u16()); continue; }
        if (m == 0xDD) { j.u16(); j.restart = j.u16(); continue; }
        if (m == 0xC0 || m == 0xC1 || m == 0xC2) {
            j.progressive = m == 0xC2;
            if (!j.read_sof()) break;
            frame = true;
            continue;
        }
        if ((m >= 0xC3 && m <= 0xCF) && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            err = "unsupported JPEG coding (lossless, hierarchical or arithmetic)";
            return WF_ERR_INVALID;
        }
        if (m == 0xDA) {
            if (!frame) { err = "JPEG scan before its frame header"; return WF_ERR_INVALID; }
            j.read_sos();
            continue;
        }
        // APPn, COM, anything else with a length
        const int len = j.u16();
        j.pos += len >= 2 ? len - 2 : 0;
    }
    if (!j.err.empty()) { err = j.err; return WF_ERR_INVALID; }
    if (!frame) { err = "JPEG without a frame"; return WF_ERR_INVALID; }
    std::vector<std::vector<uint8_t>> planes;
    j.reconstruct(planes);
    const int W = j.width, H = j.height;
    std::vector<std::vector<uint8_t>> full(j.comp.size());
    for (size_t c = 0; c < j.comp.size(); ++c) {
        const Comp& cc = j.comp[c];
        full[c] = upsample(planes[c], cc.bw * 8, cc.cw, cc.ch, j.hmax / cc.h, j.vmax / cc.v, W, H);
    }
    rgba.resize((size_t)W * H * 4);
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        if (j.comp.size() == 1) {
            rgba[4 * i] = rgba[4 * i + 1] = rgba[4 * i + 2] = full[0][i];
        } else {
            // JFIF (T.871): R = Y + 1.402 (Cr - 128), G = Y - 0.344136 (Cb - 128) - 0.714136 (Cr - 128),
            // B = Y + 1.772 (Cb - 128)
            const double y = full[0][i], cb = full[1][i] - 128.0, cr = full[2][i] - 128.0;
            const double rgb[3] = {y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb};
            for (int k = 0; k < 3; ++k) {
                const double v = std::floor(rgb[k] + 0.5);
                rgba[4 * i + k] = (uint8_t)(v < 0.0 ? 0 : (v > 255.0 ? 255 : v));
            }
        }
        rgba[4 * i + 3] = 255;
    }
    *w = (uint32_t)W;
    *h = (uint32_t)H;
    return WF_OK;
}

// ------------------------------------------------------------------ Radiance HDR
int decode_hdr(const uint8_t* d, size_t n, uint32_t* w, uint32_t* h, std::vector<float>& rgba, std::string& err) {
    size_t pos = 0;
    auto line = [&]() {
        std::string s;
        while (pos < n && d[pos] != '\n') s.push_back((char)d[pos++]);
        if (pos < n) pos++;
        return s;
    };
    const std::string magic = line();
    if (magic != "#?RADIANCE" && magic != "#?RGBE") { err = "not a Radiance HDR file"; return WF_ERR_INVALID; }
    bool rgbe = false;
    for (;;) {
        if (pos >= n) { err = "truncated HDR header"; return WF_ERR_INVALID; }
        const std::string s = line();
        if (s.empty()) break;
        if (s == "FORMAT=32-bit_rle_rgbe") rgbe = true;
    }
    if (!rgbe) { err = "HDR format other than 32-bit_rle_rgbe"; return WF_ERR_INVALID; }
    int W = 0, H = 0;
    if (std::sscanf(line().c_str(), "-Y %d +X %d", &H, &W) != 2 || W <= 0 || H <= 0 || W > 16384 || H > 16384) {
        err = "unsupported HDR resolution line (only -Y h +X w)";
        return WF_ERR_INVALID;
    }
    std::vector<uint8_t> row((size_t)W * 4);
    rgba.resize((size_t)W * H * 4);
    for (int y = 0; y < H; ++y) {
        if (W >= 8 && W < 32768 && pos + 4 <= n && d[pos] == 2 && d[pos + 1] == 2 && !(d[pos + 2] & 0x80)) {
            if (((d[pos + 2] << 8) | d[pos + 3]) != W) { err = "HDR scanline width mismatch"; return WF_ERR_INVALID; }
            pos += 4;
            for (int c = 0; c < 4; ++c) {
                for (int x = 0; x < W;) {
                    if (pos >= n) { err = "truncated HDR data"; return WF_ERR_INVALID; }
                    int cnt = d[pos++];
                    if (cnt > 128) {
                        cnt -= 128;
                        if (pos >= n || x + cnt > W) { err = "bad HDR run"; return WF_ERR_INVALID; }
                        const uint8_t v = d[pos++];
                        for (int k = 0; k < cnt; ++k) row[4 * (x++) + c] = v;
                    } else {
                        if (cnt == 0 || pos + cnt > n || x + cnt > W) { err = "bad HDR run"; return WF_ERR_INVALID; }
                        for (int k = 0; k < cnt; ++k) row[4 * (x++) + c] = d[pos++];
                    }
                }
            }
        } else {
            if (pos + 4ull * W > n) { err = "truncated HDR data"; return WF_ERR_INVALID; }
            std::memcpy(row.data(), d + pos, 4ull * W);
            pos += 4ull * W;
        }
        for (int x = 0; x < W; ++x) {
            const uint8_t* p = &row[4 * x];
            float* o = &rgba[4 * ((size_t)y * W + x)];
            if (p[3] == 0) {
                o[0] = o[1] = o[2] = 0.0f;
            } else {
                const float f = std::ldexp(1.0f, (int)p[3] - 136);
                o[0] = (float)p[0] * f;
                o[1] = (float)p[1] * f;
                o[2] = (float)p[2] * f;
            }
            o[3] = 1.0f;
        }
    }
    *w = (uint32_t)W;
    *h = (uint32_t)H;
    return WF_OK;
}

// ------------------------------------------------------------------ DDS
uint32_t rd32(const uint8_t* p) { uint32_t v; std::memcpy(&v, p, 4); return v; }
constexpr uint32_t fourcc(char a, char b, char c, char d) {
    return (uint32_t)(uint8_t)a | ((uint32_t)(uint8_t)b << 8) | ((uint32_t)(uint8_t)c << 16) | ((uint32_t)(uint8_t)d << 24);
}

int decode_dds(const uint8_t* d, size_t n, uint32_t* w, uint32_t* h, uint32_t* fmt, const uint8_t** data,
               uint64_t* bytes, std::string& err) {
    if (n < 128 || rd32(d) != fourcc('D', 'D', 'S', ' ') || rd32(d + 4) != 124 || rd32(d + 76) != 32) {
        err = "not a DDS file";
        return WF_ERR_INVALID;
    }
    const uint32_t H = rd32(d + 12), W = rd32(d + 16);
    const uint32_t pf_flags = rd32(d + 80), four = rd32(d + 84), rgbbits = rd32(d + 88);
    const uint32_t rmask = rd32(d + 92), gmask = rd32(d + 96), bmask = rd32(d + 100), amask = rd32(d + 104);
    size_t off = 128;
    uint32_t f = ~0u;
    if ((pf_flags & 4u) && four == fourcc('D', 'X', '1', '0')) {
        if (n < 148) { err = "truncated DDS DX10 header"; return WF_ERR_INVALID; }
        off = 148;
        switch (rd32(d + 128)) {   // DXGI_FORMAT
            case 2: f = WF_TEXTURE_RGBA32F; break;        // R32G32B32A32_FLOAT
            case 28: f = WF_TEXTURE_RGBA8; break;         // R8G8B8A8_UNORM
            case 29: f = WF_TEXTURE_RGBA8_SRGB; break;    // R8G8B8A8_UNORM_SRGB
            case 49: f = WF_TEXTURE_RG8; break;           // R8G8_UNORM
            case 71: f = WF_TEXTURE_BC1; break;
            case 72: f = WF_TEXTURE_BC1_SRGB; break;
            case 74: f = WF_TEXTURE_BC2; break;
            case 75: f = WF_TEXTURE_BC2_SRGB; break;
            case 77: f = WF_TEXTURE_BC3; break;
            case 78: f = WF_TEXTURE_BC3_SRGB; break;
            case 80: f = WF_TEXTURE_BC4; break;
            case 83: f = WF_TEXTURE_BC5; break;
            case 98: f = WF_TEXTURE_BC7; break;
            case 99: f = WF_TEXTURE_BC7_SRGB; break;
            default: break;
        }
    } else if (pf_flags & 4u) {
        if (four == fourcc('D', 'X', 'T', '1')) f = WF_TEXTURE_BC1;
        else if (four == fourcc('D', 'X', 'T', '3')) f = WF_TEXTURE_BC2;
        else if (four == fourcc('D', 'X', 'T', '5')) f = WF_TEXTURE_BC3;
        else if (four == fourcc('A', 'T', 'I', '1') || four == fourcc('B', 'C', '4', 'U')) f = WF_TEXTURE_BC4;
        else if (four == fourcc('A', 'T', 'I', '2') || four == fourcc('B', 'C', '5', 'U')) f = WF_TEXTURE_BC5;
    } else if ((pf_flags & 0x40u) && rgbbits == 32 && rmask == 0xFFu && gmask == 0xFF00u && bmask == 0xFF0000u) {
        (void)amask;
        f = WF_TEXTURE_RGBA8;
    }
    if (f == ~0u) { err = "unsupported DDS pixel format"; return WF_ERR_INVALID; }
    if (W == 0 || H == 0 || W > 16384 || H > 16384) { err = "bad DDS size"; return WF_ERR_INVALID; }
    uint64_t sz = 0;
    const uint64_t bw = (W + 3) / 4, bh = (H + 3) / 4;
    switch (f) {
        case WF_TEXTURE_RGBA32F: sz = 16ull * W * H; break;
        case WF_TEXTURE_RGBA8: case WF_TEXTURE_RGBA8_SRGB: sz = 4ull * W * H; break;
        case WF_TEXTURE_RG8: sz = 2ull * W * H; break;
        case WF_TEXTURE_BC1: case WF_TEXTURE_BC1_SRGB: case WF_TEXTURE_BC4: sz = 8 * bw * bh; break;
        default: sz = 16 * bw * bh; break;
    }
    if (off + sz > n) { err = "truncated DDS data"; return WF_ERR_INVALID; }
    *w = W;
    *h = H;
    *fmt = f;
    *data = d + off;
    *bytes = sz;
    return WF_OK;
}

// ------------------------------------------------------------------ PNG
// DEFLATE decoder (RFC 1951), reading bits LSB first; Huffman codes decoded
// canonically one bit at a time.
struct Inflate {
    const uint8_t* d;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    bool bad = false;
    size_t limit = 0;   // the output the image needs: more is an error, not an allocation
    std::vector<uint8_t> out;

    uint32_t bits(int k) {
        while (cnt < k) {
            if (pos >= n) { bad = true; return 0; }
            buf |= (uint64_t)d[pos++] << cnt;
            cnt += 8;
        }
        const uint32_t v = (uint32_t)(buf & ((1ull << k) - 1));
        buf >>= k;
        cnt -= k;
        return v;
    }
    struct Huffman {
        uint16_t count[16] = {};
        uint16_t symbol[320] = {};
    };
    // counts per length and symbols in (length, value) order; false for an
    // over-subscribed set of lengths
    static bool build(Huffman& hf, const uint8_t* len, int nsym) {
        for (int i = 0; i < 16; ++i) hf.count[i] = 0;
        for (int i = 0; i < nsym; ++i) hf.count[len[i]]++;
        hf.count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left <<= 1;
            left -= hf.count[l];
            if (left < 0) return false;
        }
        uint16_t off[16];
        off[1] = 0;
        for (int l = 1; l < 15; ++l) off[l + 1] = off[l] + hf.count[l];
        for (int i = 0; i < nsym; ++i)
            if (len[i]) hf.symbol[off[len[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(const Huffman& hf) {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (int)bits(1);
            if (bad) return -1;
            const int c = hf.count[l];
            if (code - first < c) return hf.symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        bad = true;   // no code of 15 bits or fewer matched
        return -1;
    }
    bool codes(const Huffman& lit, const Huffman& dist) {
        static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                           31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
        static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                         2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
        static const uint16_t dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                           193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
        static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                         6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
        for (;;) {
            const int sym = decode(lit);
            if (sym < 0) return false;
            if (sym < 256) {
                if (out.size() >= limit) return false;
                out.push_back((uint8_t)sym);
            } else if (sym == 256) {
                return true;
            } else {
                const int li = sym - 257;
                if (li >= 29) return false;
                const size_t len = lbase[li] + bits(lext[li]);
                const int ds = decode(dist);
                if (ds < 0 || ds >= 30) return false;
                const size_t dd = dbase[ds] + bits(dext[ds]);
                if (bad || dd > out.size() || len > limit - out.size()) return false;
                const size_t from = out.size() - dd;
                for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
            }
        }
    }
    bool run() {
        int last;
        do {
            last = (int)bits(1);
            const uint32_t type = bits(2);
            if (bad) return false;
            if (type == 0) {
                buf = 0;   // stored block: the rest of the current byte is dropped
                cnt = 0;
                if (pos + 4 > n) return false;
                const uint32_t len = d[pos] | (d[pos + 1] << 8), nlen = d[pos + 2] | (d[pos + 3] << 8);
                pos += 4;
                if ((len ^ 0xFFFFu) != nlen || pos + len > n || len > limit - out.size()) return false;
                out.insert(out.end(), d + pos, d + pos + len);
                pos += len;
            } else if (type == 1) {
                static const struct Fixed {
                    Huffman lit, dist;
                    Fixed() {
                        uint8_t l[288];
                        for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
                        build(lit, l, 288);
                        uint8_t dl[30];
                        for (int i = 0; i < 30; ++i) dl[i] = 5;
                        build(dist, dl, 30);
                    }
                } fixed;
                if (!codes(fixed.lit, fixed.dist)) return false;
            } else if (type == 2) {
                const int hlit = (int)bits(5) + 257, hdist = (int)bits(5) + 1, hclen = (int)bits(4) + 4;
                static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
                uint8_t cl[19] = {};
                for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)bits(3);
                Huffman clh;
                if (bad || hlit > 286 || hdist > 30 || !build(clh, cl, 19)) return false;
                uint8_t lens[320] = {};
                int i = 0;
                while (i < hlit + hdist) {
                    const int sym = decode(clh);
                    if (sym < 0) return false;
                    if (sym < 16) {
                        lens[i++] = (uint8_t)sym;
                    } else {
                        int rep, val = 0;
                        if (sym == 16) {
                            if (i == 0) return false;
                            val = lens[i - 1];
                            rep = 3 + (int)bits(2);
                        } else if (sym == 17) {
                            rep = 3 + (int)bits(3);
                        } else {
                            rep = 11 + (int)bits(7);
                        }
                        if (i + rep > hlit + hdist) return false;
                        while (rep--) lens[i++] = (uint8_t)val;
                    }
                }
                Huffman lit, dist;
                if (bad || lens[256] == 0 || !build(lit, lens, hlit) || !build(dist, lens + hlit, hdist)) return false;
                if (!codes(lit, dist)) return false;
            } else {
                return false;
            }
        } while (!last);
        return !bad;
    }
};

uint32_t be32(const uint8_t* p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

int decode_png(const uint8_t* d, size_t n, uint32_t* w, uint32_t* h, std::vector<uint8_t>& rgba, std::string& err) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (n < 8 || std::memcmp(d, sig, 8) != 0) { err = "not a PNG file"; return WF_ERR_INVALID; }
    size_t pos = 8;
    uint32_t width = 0, height = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    bool ihdr = false, iend = false;
    while (pos + 12 <= n && !iend) {
        const uint32_t len = be32(d + pos);
        const uint8_t* type = d + pos + 4;
        if (len > n - pos - 12) { err = "truncated chunk"; return WF_ERR_INVALID; }
        const uint8_t* data = d + pos + 8;
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len != 13) { err = "bad IHDR"; return WF_ERR_INVALID; }
            width = be32(data);
            height = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
            if (data[10] != 0 || data[11] != 0 || interlace > 1) { err = "unknown compression, filter or interlace method"; return WF_ERR_INVALID; }
            ihdr = true;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            plte.assign(data, data + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(data, data + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            iend = true;
        } else if (!(type[0] & 0x20)) {
            err = "unknown critical chunk";
            return WF_ERR_INVALID;
        }
        pos += 12ull + len;
    }
    if (!ihdr || idat.size() < 2) { err = "missing IHDR or IDAT"; return WF_ERR_INVALID; }
    if (width == 0 || height == 0 || width > 16384 || height > 16384) { err = "unsupported image size"; return WF_ERR_INVALID; }
    int channels;
    switch (ctype) {
        case 0: channels = 1; break;
        case 2: channels = 3; break;
        case 3: channels = 1; break;
        case 4: channels = 2; break;
        case 6: channels = 4; break;
        default: err = "unknown colour type"; return WF_ERR_INVALID;
    }
    const bool depth_ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                          (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                          ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
    if (!depth_ok) { err = "invalid bit depth for the colour type"; return WF_ERR_INVALID; }
    if (ctype == 3 && (plte.empty() || plte.size() % 3 != 0)) { err = "missing or bad PLTE"; return WF_ERR_INVALID; }
    // zlib header (RFC 1950): deflate, no preset dictionary
    if ((idat[0] & 15) != 8 || ((idat[0] << 8) | idat[1]) % 31 != 0 || (idat[1] & 0x20)) {
        err = "bad zlib header";
        return WF_ERR_INVALID;
    }
    Inflate inf;
    inf.d = idat.data() + 2;
    inf.n = idat.size() - 2;
    // filtered scanlines of every pass: a filter byte and the packed samples per row
    for (int pass = 0; pass < (interlace ? 7 : 1); ++pass) {
        static const int px0[7] = {0, 4, 0, 2, 0, 1, 0}, py0[7] = {0, 0, 4, 0, 2, 0, 1};
        static const int pdx[7] = {8, 8, 4, 4, 2, 2, 1}, pdy[7] = {8, 8, 8, 4, 4, 2, 2};
        const uint32_t x0 = interlace ? px0[pass] : 0, y0 = interlace ? py0[pass] : 0;
        const uint32_t dx = interlace ? pdx[pass] : 1, dy = interlace ? pdy[pass] : 1;
        if (x0 >= width || y0 >= height) continue;
        const uint64_t pw = (width - x0 + dx - 1) / dx, ph = (height - y0 + dy - 1) / dy;
        inf.limit += (size_t)(ph * (1 + (pw * channels * depth + 7) / 8));
    }
    inf.out.reserve(inf.limit);
    if (!inf.run()) { err = "corrupt DEFLATE data"; return WF_ERR_INVALID; }
    const std::vector<uint8_t>& raw = inf.out;
    const int bpp = std::max(1, channels * depth / 8);   // filter byte distance
    // samples of the whole image, 16 bits each, in row-major pixel order
    std::vector<uint16_t> smp((size_t)width * height * channels);
    static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
    size_t rp = 0;
    for (int pass = 0; pass < (interlace ? 7 : 1); ++pass) {
        const uint32_t x0 = interlace ? ax0[pass] : 0, y0 = interlace ? ay0[pass] : 0;
        const uint32_t dx = interlace ? adx[pass] : 1, dy = interlace ? ady[pass] : 1;
        if (x0 >= width || y0 >= height) continue;
        const uint32_t pw = (width - x0 + dx - 1) / dx, ph = (height - y0 + dy - 1) / dy;
        const size_t stride = ((size_t)pw * channels * depth + 7) / 8;
        std::vector<uint8_t> prev(stride, 0), cur(stride);
        for (uint32_t y = 0; y < ph; ++y) {
            if (rp + 1 + stride > raw.size()) { err = "image data too short"; return WF_ERR_INVALID; }
            const uint8_t f = raw[rp];
            const uint8_t* src = raw.data() + rp + 1;
            rp += 1 + stride;
            for (size_t i = 0; i < stride; ++i) {
                const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= (size_t)bpp ? prev[i - bpp] : 0;
                int v = src[i];
                switch (f) {
                    case 0: break;
                    case 1: v += a; break;
                    case 2: v += b; break;
                    case 3: v += (a + b) >> 1; break;
                    case 4: {
                        const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                        v += (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                        break;
                    }
                    default: err = "unknown scanline filter"; return WF_ERR_INVALID;
                }
                cur[i] = (uint8_t)v;
            }
            for (uint32_t x = 0; x < pw; ++x) {
                const size_t o = (((size_t)(y0 + y * dy)) * width + (x0 + x * dx)) * channels;
                for (int ch = 0; ch < channels; ++ch) {
                    const size_t k = (size_t)x * channels + ch;
                    uint16_t v;
                    if (depth == 16) v = (uint16_t)((cur[2 * k] << 8) | cur[2 * k + 1]);
                    else if (depth == 8) v = cur[k];
                    else v = (uint16_t)((cur[(k * depth) >> 3] >> (8 - depth - (int)((k * depth) & 7))) & ((1 << depth) - 1));
                    smp[o + ch] = v;
                }
            }
            std::swap(prev, cur);
        }
    }
    // to RGBA8: 16-bit samples keep their high byte; grey below 8 bits is
    // scaled to 0..255; tRNS keys compare with the samples at their own depth
    const int scale = depth == 1 ? 255 : depth == 2 ? 85 : depth == 4 ? 17 : 1;
    rgba.resize((size_t)width * height * 4);
    const size_t npx = (size_t)width * height;
    for (size_t i = 0; i < npx; ++i) {
        const uint16_t* s = smp.data() + i * channels;
        uint8_t* o = rgba.data() + i * 4;
        auto to8 = [&](uint16_t v) { return (uint8_t)(depth == 16 ? (v >> 8) : v * scale); };
        if (ctype == 3) {
            const size_t idx = s[0];
            if (3 * idx + 2 >= plte.size()) { err = "palette index out of range"; return WF_ERR_INVALID; }
            o[0] = plte[3 * idx];
            o[1] = plte[3 * idx + 1];
            o[2] = plte[3 * idx + 2];
            o[3] = idx < trns.size() ? trns[idx] : 255;
        } else if (ctype == 0 || ctype == 4) {
            o[0] = o[1] = o[2] = to8(s[0]);
            if (ctype == 4) o[3] = to8(s[1]);
            else o[3] = (trns.size() >= 2 && s[0] == (((uint16_t)trns[0] << 8) | trns[1])) ? 0 : 255;
        } else {
            for (int ch = 0; ch < 3; ++ch) o[ch] = to8(s[ch]);
            if (ctype == 6) {
                o[3] = to8(s[3]);
            } else {
                const bool key = trns.size() >= 6 && s[0] == (((uint16_t)trns[0] << 8) | trns[1]) &&
                                 s[1] == (((uint16_t)trns[2] << 8) | trns[3]) &&
                                 s[2] == (((uint16_t)trns[4] << 8) | trns[5]);
                o[3] = key ? 0 : 255;
            }
        }
    }
    *w = width;
    *h = height;
    return WF_OK;
}

}  // namespace
}  // namespace wf

extern "C" int wf_image_decode(const void* file, uint64_t file_size, uint32_t* out_width, uint32_t* out_height,
                               uint32_t* out_format, void* out, uint64_t* inout_size) {
    using namespace wf;
    if (!file || !out_width || !out_height || !out_format || !inout_size)
        return report_error(WF_ERR_INVALID, "wf_image_decode: null argument");
    const uint8_t* d = static_cast<const uint8_t*>(file);
    const size_t n = (size_t)file_size;
    std::string err;
    int rc;
    uint32_t w = 0, h = 0, f = 0;
    const uint8_t* src = nullptr;
    uint64_t bytes = 0;
    std::vector<uint8_t> rgba8;
    std::vector<float> rgbaf;
    if (n >= 2 && d[0] == 0xFF && d[1] == 0xD8) {
        rc = decode_jpeg(d, n, &w, &h, rgba8, err);
        f = WF_TEXTURE_RGBA8;
        src = rgba8.data();
        bytes = rgba8.size();
    } else if (n >= 6 && d[0] == '#' && d[1] == '?') {
        rc = decode_hdr(d, n, &w, &h, rgbaf, err);
        f = WF_TEXTURE_RGBA32F;
        src = reinterpret_cast<const uint8_t*>(rgbaf.data());
        bytes = rgbaf.size() * 4ull;
    } else if (n >= 4 && d[0] == 'D' && d[1] == 'D' && d[2] == 'S' && d[3] == ' ') {
        rc = decode_dds(d, n, &w, &h, &f, &src, &bytes, err);
    } else if (n >= 8 && d[0] == 137 && d[1] == 'P' && d[2] == 'N' && d[3] == 'G') {
        rc = decode_png(d, n, &w, &h, rgba8, err);
        f = WF_TEXTURE_RGBA8;
        src = rgba8.data();
        bytes = rgba8.size();
    } else {
        return report_error(WF_ERR_INVALID,
                            "wf_image_decode: unrecognised file (JPEG, PNG, Radiance HDR or DDS expected)");
    }
    if (rc) return report_error(rc, ("wf_image_decode: " + err).c_str());
    *out_width = w;
    *out_height = h;
    *out_format = f;
    if (!out || *inout_size < bytes) {
        *inout_size = bytes;
        return out ? report_error(WF_ERR_CAPACITY, "wf_image_decode: output buffer too small") : WF_OK;
    }
    std::memcpy(out, src, bytes);
    *inout_size = bytes;
    return WF_OK;
}
