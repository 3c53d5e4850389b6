// wf_qbvh.cu — the quantized 4-wide BLAS layout (wf_init_params.blas_layout = 1).
//
// The reference's BLAS is a binary tree of 32-byte nodes whose child pairs
// share a 64-byte line (bvh_builder.cpp:44-45, shared.hlsl.h:106-112): one
// traversal step fetches 64 bytes and tests two boxes.  This layout collapses
// every other level of that tree into one 64-byte node holding up to four
// child boxes quantized to 8 bits per plane, so a step fetches the same 64
// bytes, tests four boxes and a ray takes about half as many dependent
// steps.  The nodes are derived from the binary blob (the builders and the
// blob the C ABI returns are unchanged); leaves keep their triangle ranges in
// the blob's leaf order.
//
// Node (4 x float4, 64-byte aligned):
//   q0 = {origin xyz (the node's box min), meta}  meta = biased exponents
//        ex | ey << 8 | ez << 16 | child count << 24 (scale_a = 2^(e_a - 127))
//   q1 = {lo_x[4], lo_y[4], lo_z[4] (bytes), count_lo[4]}
//   q2 = {hi_x[4], hi_y[4], hi_z[4] (bytes), count_hi[4]}
//   q3 = {child[4]}: leaf = first triangle (leaf order), count > 0;
//        interior = node index, count = 0
// A child box is origin + q * scale per plane: q * scale is exact (an 8-bit
// integer times a power of two) and the sum rounds once; the quantizer checks
// the rounded value in float exactly as the kernel computes it, so every
// quantized box contains its exact box plane by plane.  The traversal over
// these boxes therefore visits every leaf the exact boxes would, and with the
// order-independent tie rule (closest hit = smallest t, then smallest
// (instance, primitive)) its hits equal those of the exact binary traversal.
//
// The exact 4-wide layout (blas_layout = 2) collapses the same levels without
// quantizing: 128 bytes per node (8 x float4: the four children's lo_x, hi_x,
// lo_y, hi_y, lo_z, hi_z planes as float4 lanes, then child[4], then
// count[4] with the child count in count[0]'s top byte), so a step tests four
// exact boxes for two 64-byte lines and no decoding.  A grandchild's box lies
// inside its parent's in float as well (the same coordinates, and rounding is
// monotone), so skipping the parent's test only adds visits, and with the tie
// rule the hits equal the binary traversal's.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/wf.h"
#include "wf_kernels.h"

namespace wf {
namespace {

struct BNode {
    float mn[3];
    uint32_t left_first;
    float mx[3];
    uint32_t prim_count;
};

// The dequantized plane as the kernel computes it.
inline float plane(float origin, uint32_t q, uint32_t biased) {
    float scale;
    const uint32_t bits = biased << 23;
    std::memcpy(&scale, &bits, 4);
    return origin + (float)q * scale;
}

// Quantizes one axis of up to four child boxes against the parent's min
// (origin).  Returns false when no exponent in range covers them.
bool quantize_axis(float origin, float pmax, const float* cmin, const float* cmax, int n, uint8_t* lo, uint8_t* hi,
                   uint32_t* biased) {
    const double extent = (double)pmax - (double)origin;
    if (!(extent >= 0.0) || !std::isfinite(extent)) return false;
    int e = -126;
    if (extent > 0.0) {
        e = (int)std::ceil(std::log2(extent / 255.0));
        if (e < -126) e = -126;
    }
    for (; e <= 127; ++e) {
        const uint32_t b = (uint32_t)(e + 127);
        const double s = std::ldexp(1.0, e);
        bool ok = true;
        for (int i = 0; i < n && ok; ++i) {
            double ql = std::floor(((double)cmin[i] - (double)origin) / s);
            double qh = std::ceil(((double)cmax[i] - (double)origin) / s);
            int l = (int)std::fmax(0.0, std::fmin(255.0, ql));
            int h = (int)std::fmax(0.0, std::fmin(255.0, qh));
            while (l > 0 && plane(origin, (uint32_t)l, b) > cmin[i]) --l;
            while (h < 255 && plane(origin, (uint32_t)h, b) < cmax[i]) ++h;
            if (plane(origin, (uint32_t)l, b) > cmin[i] || plane(origin, (uint32_t)h, b) < cmax[i]) {
                ok = false;
            } else {
                lo[i] = (uint8_t)l;
                hi[i] = (uint8_t)h;
            }
        }
        if (ok) {
            *biased = b;
            return true;
        }
    }
    return false;
}

struct Converter {
    const uint8_t* nodes;
    uint64_t node_count;
    bool exact = false;            // the exact layout (32 words per node) instead of the quantized one
    std::vector<uint32_t> words;   // 16 (quantized) or 32 (exact) words per node
    const char* error = nullptr;
    uint32_t stride() const { return exact ? 32u : 16u; }

    BNode get(uint32_t i) const {
        BNode b;
        std::memcpy(&b, nodes + 32ull * i, 32);
        return b;
    }

    // Emits the node for binary interior node bi; returns its index.
    uint32_t emit(uint32_t bi, int depth) {
        if (depth > 64) { error = "BLAS deeper than the traversal stack"; return 0; }
        const uint32_t me = (uint32_t)(words.size() / stride());
        words.resize(words.size() + stride(), 0u);
        const BNode p = get(bi);
        uint32_t kid[4];
        int n = 0;
        for (uint32_t c = p.left_first; c < p.left_first + 2u; ++c) {
            if ((uint64_t)c + 1 > node_count) { error = "BLAS child index out of range"; return 0; }
            const BNode b = get(c);
            if (b.prim_count > 0) {
                kid[n++] = c;
            } else {
                if ((uint64_t)b.left_first + 2 > node_count) { error = "BLAS child index out of range"; return 0; }
                kid[n++] = b.left_first;
                kid[n++] = b.left_first + 1;
            }
        }
        float cmin[3][4], cmax[3][4];
        uint32_t entry[4], count[4];
        for (int i = 0; i < n; ++i) {
            const BNode b = get(kid[i]);
            for (int a = 0; a < 3; ++a) { cmin[a][i] = b.mn[a]; cmax[a][i] = b.mx[a]; }
            count[i] = b.prim_count;
            if (b.prim_count > 0xFFFFu) { error = "a BLAS leaf holds more than 65535 triangles"; return 0; }
            // a leaf's first triangle; an interior child's own binary index (emitted below)
            entry[i] = b.prim_count > 0 ? b.left_first : kid[i];
        }
        if (exact) {
            for (int i = 0; i < n; ++i)
                if (count[i] == 0) entry[i] = emit(entry[i], depth + 1);
            if (error) return 0;
            uint32_t* w = words.data() + 32ull * me;
            for (int i = 0; i < 4; ++i) {
                for (int a = 0; a < 3; ++a) {
                    const float lo_v = i < n ? cmin[a][i] : 0.0f, hi_v = i < n ? cmax[a][i] : 0.0f;
                    std::memcpy(&w[8 * a + i], &lo_v, 4);
                    std::memcpy(&w[8 * a + 4 + i], &hi_v, 4);
                }
                w[24 + i] = i < n ? entry[i] : 0xFFFFFFFFu;
                w[28 + i] = i < n ? count[i] : 0u;
            }
            w[28] |= (uint32_t)n << 24;
            return me;
        }
        // the node's box: the union of its children (the binary node's box)
        uint8_t lo[3][4] = {}, hi[3][4] = {};
        uint32_t be[3];
        float origin[3];
        for (int a = 0; a < 3; ++a) {
            float mn = cmin[a][0], mx = cmax[a][0];
            for (int i = 1; i < n; ++i) { mn = std::fmin(mn, cmin[a][i]); mx = std::fmax(mx, cmax[a][i]); }
            origin[a] = mn;
            if (!quantize_axis(mn, mx, cmin[a], cmax[a], n, lo[a], hi[a], &be[a])) {
                error = "a BLAS box cannot be quantized (non-finite bounds)";
                return 0;
            }
        }
        for (int i = 0; i < n; ++i)
            if (count[i] == 0) entry[i] = emit(entry[i], depth + 1);
        if (error) return 0;
        uint32_t* w = words.data() + 16ull * me;
        std::memcpy(&w[0], &origin[0], 4);
        std::memcpy(&w[1], &origin[1], 4);
        std::memcpy(&w[2], &origin[2], 4);
        w[3] = be[0] | (be[1] << 8) | (be[2] << 16) | ((uint32_t)n << 24);
        for (int i = 0; i < 4; ++i) {
            const uint32_t c = i < n ? count[i] : 0u;
            w[4] |= (uint32_t)lo[0][i] << (8 * i);
            w[5] |= (uint32_t)lo[1][i] << (8 * i);
            w[6] |= (uint32_t)lo[2][i] << (8 * i);
            w[7] |= (c & 0xFFu) << (8 * i);
            w[8] |= (uint32_t)hi[0][i] << (8 * i);
            w[9] |= (uint32_t)hi[1][i] << (8 * i);
            w[10] |= (uint32_t)hi[2][i] << (8 * i);
            w[11] |= (c >> 8) << (8 * i);
            w[12 + i] = i < n ? entry[i] : 0xFFFFFFFFu;
        }
        return me;
    }
};

}  // namespace

// Builds the quantized nodes of a BLAS blob; *root_count = the root's
// triangle count when the whole BLAS is one leaf (no nodes then), else 0.
int qbvh_convert(const uint8_t* blob, uint64_t size, std::vector<uint32_t>& out, uint32_t* root_count,
                 const char** error, bool exact) {
    bvh_header_t h;
    if (size < 12 + 32) { *error = "BLAS blob too small"; return WF_ERR_INVALID; }
    std::memcpy(&h, blob, 12);
    if (h.nodes_offset != 12 || h.triangles_offset < 12 + 32 || h.triangles_offset > size) {
        *error = "bad BLAS header";
        return WF_ERR_INVALID;
    }
    Converter cv;
    cv.exact = exact;
    cv.nodes = blob + 12;
    cv.node_count = (h.triangles_offset - 12) / 32;
    const BNode root = cv.get(0);
    out.clear();
    *root_count = 0;
    if (root.prim_count > 0) {
        *root_count = root.prim_count;
        return WF_OK;
    }
    cv.emit(0, 0);
    if (cv.error) { *error = cv.error; return WF_ERR_INVALID; }
    out.swap(cv.words);
    return WF_OK;
}

}  // namespace wf

// The quantized 4-wide nodes of a BLAS blob, on the host (tests and tools):
// writes 64 bytes per node into out_nodes (NULL = size query) and the root
// triangle count when the BLAS is a single leaf.
extern "C" int wf_bvh_quantize(const void* blob, uint64_t blob_size, void* out_nodes, uint64_t* inout_size,
                               uint32_t* out_root_count) {
    if (!blob || !inout_size || !out_root_count) return wf::report_error(WF_ERR_INVALID, "wf_bvh_quantize: null argument");
    std::vector<uint32_t> words;
    const char* err = nullptr;
    int rc = wf::qbvh_convert(static_cast<const uint8_t*>(blob), blob_size, words, out_root_count, &err, false);
    if (rc) return wf::report_error(rc, err);
    const uint64_t bytes = words.size() * 4ull;
    if (!out_nodes || *inout_size < bytes) {
        *inout_size = bytes;
        return out_nodes ? wf::report_error(WF_ERR_CAPACITY, "wf_bvh_quantize: output buffer too small") : WF_OK;
    }
    std::memcpy(out_nodes, words.data(), bytes);
    *inout_size = bytes;
    return WF_OK;
}

// The exact 4-wide nodes of a BLAS blob (blas_layout 2), on the host: 128
// bytes per node into out_nodes (NULL = size query).
extern "C" int wf_bvh_widen(const void* blob, uint64_t blob_size, void* out_nodes, uint64_t* inout_size,
                            uint32_t* out_root_count) {
    if (!blob || !inout_size || !out_root_count) return wf::report_error(WF_ERR_INVALID, "wf_bvh_widen: null argument");
    std::vector<uint32_t> words;
    const char* err = nullptr;
    int rc = wf::qbvh_convert(static_cast<const uint8_t*>(blob), blob_size, words, out_root_count, &err, true);
    if (rc) return wf::report_error(rc, err);
    const uint64_t bytes = words.size() * 4ull;
    if (!out_nodes || *inout_size < bytes) {
        *inout_size = bytes;
        return out_nodes ? wf::report_error(WF_ERR_CAPACITY, "wf_bvh_widen: output buffer too small") : WF_OK;
    }
    std::memcpy(out_nodes, words.data(), bytes);
    *inout_size = bytes;
    return WF_OK;
}
