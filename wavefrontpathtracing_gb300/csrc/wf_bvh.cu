// wf_bvh.cu — GPU binned-SAH BLAS builder, byte-identical to the reference's
// recursive CPU builder (bvh_builder.cpp:6-264) at equal options.
//
// Why the output matches:
//  * every float is computed with the reference's operations: centroid
//    ((p0 + p1) + p2) * 0.3333f, bin (int)((c - cmin) * (bins / (cmax - cmin)))
//    clamped to bins-1, and the SAH sweep's per-plane costs (half area,
//    count * area) with the first minimum over axis 0..2, then plane
//    0..bins-2, as the reference's strict "<" picks it (one thread per node in
//    the large phase, a warp scan over the bins in the small phase);
//  * bin and node bounds are min/max reductions, whose value does not depend
//    on the order (a -0.0/+0.0 tie is the one case where the reference keeps
//    the first operand it saw; a bound holding both zero signs may differ in
//    that bit only);
//  * the reference's in-place two-pointer partition (:121-137) is not stable,
//    but its permutation has a closed form that two scans reproduce in
//    parallel.  With nL left-going triangles, p = nL + [element nL goes
//    right], front = [0, p), back = [p, count):
//       front left-goer at i                 -> i
//       back right-goer at i                 -> i - 1
//       m-th front right-goer                -> g(m-1) - 1   (g(0) = count)
//       m-th back left-goer counted from the end, g(m) -> f(m), the position
//                                               of the m-th front right-goer
//    which also reproduces the left rotation the loop applies when no plane
//    exists and every triangle "goes right";
//  * nodes are created breadth-first or per warp, then renumbered: the
//    reference allocates each split node's child pair when it visits that node
//    in pre-order, so the pair of internal node X sits at
//    2 + 2 * (pre-order rank of X among internal nodes).
//
// Phases: nodes with more than kSmall triangles are processed level by level
// by many CTAs (chunked binning into shared-memory bins, chunked scans for the
// partition); subtrees of at most kSmall triangles are built by one warp each,
// entirely in shared memory.  The host side makes one scratch allocation,
// gathers the positions on several threads and writes the blob straight into
// the caller's buffer when it fits.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "wf_bvh.h"
#include "wf_device.cuh"

namespace wf {

namespace {

constexpr uint32_t kMaxBins = 64;
constexpr uint32_t kChunk = 4096;      // positions per CTA in the large-node phase
constexpr uint32_t kChunkThreads = 256;
#ifndef WF_BVH_SMALL
#define WF_BVH_SMALL 128
#endif
constexpr uint32_t kSmall = WF_BVH_SMALL;   // subtrees at most this large are built by one warp
static_assert(kSmall >= 32 && kSmall <= 65536, "16-bit local positions");
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kBinWords = 7;      // count, min xyz, max xyz (order-preserving keys)
constexpr uint32_t kBoxWords = 18;     // node min/max, centroid min/max keys, first-zero positions

thread_local std::string g_err;

// Order-preserving float <-> uint32 keys for atomicMin / atomicMax.
__device__ __forceinline__ uint32_t fenc(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fdec(uint32_t k) { return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k); }
// glm::min / glm::max (func_common.inl:17-35)
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float half_area(const float* mn, const float* mx) {
    float ex = mx[0] - mn[0], ey = mx[1] - mn[1], ez = mx[2] - mn[2];
    return ex * ey + ey * ez + ez * ex;
}
__device__ __forceinline__ float comp(float4 v, uint32_t a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

struct Ctx {
    uint32_t n, bins, single, max_leaf;
    const float* pos;        // 9 floats per triangle (original order)
    float4* cen;             // centroid
    float4* tmn;             // triangle min corner
    float4* tmx;             // triangle max corner
    uint32_t* idx;           // current index permutation
    uint32_t* idx_tmp;       // partition target
    uint32_t* F;             // per-position scratch: front right-goers by rank
    uint32_t* G;             // per-position scratch: back left-goers by rank
    float4* ta;              // temporary nodes {min xyz, first}
    float4* tb;              //                 {max xyz, count}
    uint32_t* tleft;         // left child (kNone for leaves); right child = left + 1
    uint32_t* tdepth;
    uint32_t* tcount;        // [0] nodes allocated, [1] maximum depth, [2] small roots, [3] error
    uint32_t* small_list;
};

// Split plan of one node, shared by the large and the small phase.
struct Plan {
    uint32_t axis, pos, nl, p, partition, children;
    float lo, scale;
};

// c = the triangle's centroid component on P.axis.
__device__ __forceinline__ bool goes_left_c(const Ctx& C, const Plan& P, float c) {
    if (P.pos == 0) return false;
    int32_t bin = (int32_t)((c - P.lo) * P.scale);
    if ((int32_t)C.bins - 1 < bin) bin = (int32_t)C.bins - 1;
    return (uint32_t)bin < P.pos;
}
__device__ __forceinline__ bool goes_left(const Ctx& C, const Plan& P, uint32_t t) {
    return goes_left_c(C, P, comp(C.cen[t], P.axis));
}

// find_best_split_plane's sweep (bvh_builder.cpp:196-249) over bins laid out
// [axis][bin][count, min xyz key, max xyz key].
__device__ float sah_sweep(const uint32_t* bins, uint32_t B, const float* cmn, const float* cmx, uint32_t& axis,
                           uint32_t& pos) {
    float cheapest = FLT_MAX;
    float larea[kMaxBins], rarea[kMaxBins];
    for (uint32_t a = 0; a < 3; ++a) {
        if (cmn[a] == cmx[a]) continue;
        const uint32_t* ab = bins + a * B * kBinWords;
        float lmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        float rmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t lsum = 0, rsum = 0;
        for (uint32_t i = 0; i < B - 1; ++i) {
            const uint32_t* lb = ab + i * kBinWords;
            lsum += lb[0];
            for (int k = 0; k < 3; ++k) {
                lmn[k] = gmin(lmn[k], fdec(lb[1 + k]));
                lmx[k] = gmax(lmx[k], fdec(lb[4 + k]));
            }
            larea[i] = (float)lsum * half_area(lmn, lmx);
            const uint32_t* rb = ab + (B - 1 - i) * kBinWords;
            rsum += rb[0];
            for (int k = 0; k < 3; ++k) {
                rmn[k] = gmin(rmn[k], fdec(rb[1 + k]));
                rmx[k] = gmax(rmx[k], fdec(rb[4 + k]));
            }
            rarea[B - 2 - i] = (float)rsum * half_area(rmn, rmx);
        }
        for (uint32_t i = 0; i < B - 1; ++i) {
            float cost = larea[i] + rarea[i];
            if (cost < cheapest) { axis = a; pos = i + 1; cheapest = cost; }
        }
    }
    return cheapest;
}

// subdivide_node's decision (bvh_builder.cpp:104-118, 139-143) plus the
// max_leaf_prims extension, without the split position p (which needs the
// element at position nL: the caller places it).
__device__ Plan make_plan_bins(const Ctx& C, const uint32_t* bins, uint32_t count, const float* nmn,
                               const float* nmx, const float* cmn, const float* cmx) {
    Plan P{};
    uint32_t axis = 0, pos = 0;
    float cost = sah_sweep(bins, C.bins, cmn, cmx, axis, pos);
    bool leaf;
    if (C.single) {
        leaf = count == 1;
    } else {
        bool force = C.max_leaf > 0 && count > C.max_leaf;
        float parent = (float)count * half_area(nmn, nmx);
        leaf = !force && cost >= parent;
    }
    P.axis = axis;
    P.pos = pos;
    P.partition = leaf ? 0u : 1u;
    if (leaf) return P;
    P.lo = cmn[axis];
    P.scale = pos > 0 ? (float)C.bins / (cmx[axis] - cmn[axis]) : 0.0f;
    uint32_t nl = 0;
    if (pos > 0) {
        const uint32_t* ab = bins + axis * C.bins * kBinWords;
        for (uint32_t b = 0; b < pos; ++b) nl += ab[b * kBinWords];
    }
    P.nl = nl;
    P.p = count;
    P.children = (nl > 0 && nl < count) ? 1u : 0u;
    return P;
}

// The same, reading the element at nL from the position list.
__device__ Plan make_plan(const Ctx& C, const uint32_t* bins, uint32_t first, uint32_t count, const float* nmn,
                          const float* nmx, const float* cmn, const float* cmx) {
    Plan P = make_plan_bins(C, bins, count, nmn, nmx, cmn, cmx);
    if (P.partition && P.nl < count) P.p = P.nl + (goes_left(C, P, C.idx[first + P.nl]) ? 0u : 1u);
    return P;
}

// Warp-parallel form of sah_sweep for the small phase: every lane returns the
// same (cheapest, axis, pos) and nl = the triangles in bins [0, pos).  Lane l
// holds bins [q*l, q*l + q) (q = 1 for up to 32 bins, else 2); shuffle scans
// give each plane its left prefix and right suffix.  Prefix and suffix boxes
// are min/max folds and counts are integer sums, so every plane's box, area
// and cost are the same floats the sequential sweep computes (a bound that
// folds -0.0 with +0.0 may keep the other zero, which changes no area); the
// first minimum in (axis, plane) order wins, as with the strict "<".
__device__ float warp_sweep(const uint32_t* bins, uint32_t B, const float* cmn, const float* cmx, uint32_t lane,
                            uint32_t& axis, uint32_t& pos, uint32_t& nl) {
    float cheapest = FLT_MAX;
    axis = 0;
    pos = 0;
    nl = 0;
    const uint32_t q = (B + 31) >> 5;
    for (uint32_t a = 0; a < 3; ++a) {
        if (cmn[a] == cmx[a]) continue;
        const uint32_t* ab = bins + a * B * kBinWords;
        uint32_t cnt[2];
        float bmn[2][3], bmx[2][3];
        for (uint32_t k = 0; k < 2; ++k) {
            const uint32_t j = lane * q + k;
            const bool have = k < q && j < B;
            const uint32_t* e = ab + j * kBinWords;
            cnt[k] = have ? e[0] : 0u;
            for (int c = 0; c < 3; ++c) {
                bmn[k][c] = have ? fdec(e[1 + c]) : FLT_MAX;
                bmx[k][c] = have ? fdec(e[4 + c]) : -FLT_MAX;
            }
        }
        // lane totals, then inclusive scans up (prefix) and down (suffix)
        uint32_t pc = cnt[0] + cnt[1], sc = pc;
        float pmn[3], pmx[3], smn[3], smx[3];
        for (int c = 0; c < 3; ++c) {
            pmn[c] = smn[c] = gmin(bmn[0][c], bmn[1][c]);
            pmx[c] = smx[c] = gmax(bmx[0][c], bmx[1][c]);
        }
        for (uint32_t off = 1; off < 32; off <<= 1) {
            const uint32_t oc = __shfl_up_sync(0xffffffffu, pc, off), uc = __shfl_down_sync(0xffffffffu, sc, off);
            float omn[3], omx[3], umn[3], umx[3];
            for (int c = 0; c < 3; ++c) {
                omn[c] = __shfl_up_sync(0xffffffffu, pmn[c], off);
                omx[c] = __shfl_up_sync(0xffffffffu, pmx[c], off);
                umn[c] = __shfl_down_sync(0xffffffffu, smn[c], off);
                umx[c] = __shfl_down_sync(0xffffffffu, smx[c], off);
            }
            if (lane >= off) {
                pc += oc;
                for (int c = 0; c < 3; ++c) { pmn[c] = gmin(pmn[c], omn[c]); pmx[c] = gmax(pmx[c], omx[c]); }
            }
            if (lane + off < 32) {
                sc += uc;
                for (int c = 0; c < 3; ++c) { smn[c] = gmin(smn[c], umn[c]); smx[c] = gmax(smx[c], umx[c]); }
            }
        }
        // exclusive: lanes below (prefix) and above (suffix)
        uint32_t ec = __shfl_up_sync(0xffffffffu, pc, 1), xc = __shfl_down_sync(0xffffffffu, sc, 1);
        float emn[3], emx[3], xmn[3], xmx[3];
        for (int c = 0; c < 3; ++c) {
            emn[c] = __shfl_up_sync(0xffffffffu, pmn[c], 1);
            emx[c] = __shfl_up_sync(0xffffffffu, pmx[c], 1);
            xmn[c] = __shfl_down_sync(0xffffffffu, smn[c], 1);
            xmx[c] = __shfl_down_sync(0xffffffffu, smx[c], 1);
        }
        if (lane == 0) {
            ec = 0;
            for (int c = 0; c < 3; ++c) { emn[c] = FLT_MAX; emx[c] = -FLT_MAX; }
        }
        if (lane == 31) {
            xc = 0;
            for (int c = 0; c < 3; ++c) { xmn[c] = FLT_MAX; xmx[c] = -FLT_MAX; }
        }
        // planes j (between bin j and j + 1) held by this lane, first minimum
        float bc = INFINITY;
        uint32_t bi = 0xFFFFFFFFu, bl = 0;
        for (uint32_t k = 0; k < 2; ++k) {
            const uint32_t j = lane * q + k;
            if (k >= q || j + 1 >= B) continue;
            uint32_t lc = ec + cnt[0], rc = xc;
            float lmn[3], lmx[3], rmn[3], rmx[3];
            for (int c = 0; c < 3; ++c) {
                lmn[c] = gmin(emn[c], bmn[0][c]);
                lmx[c] = gmax(emx[c], bmx[0][c]);
                rmn[c] = xmn[c];
                rmx[c] = xmx[c];
            }
            if (k == 1) {
                lc += cnt[1];
                for (int c = 0; c < 3; ++c) { lmn[c] = gmin(lmn[c], bmn[1][c]); lmx[c] = gmax(lmx[c], bmx[1][c]); }
            } else if (q == 2) {
                rc += cnt[1];
                for (int c = 0; c < 3; ++c) { rmn[c] = gmin(rmn[c], bmn[1][c]); rmx[c] = gmax(rmx[c], bmx[1][c]); }
            }
            const float cost = (float)lc * half_area(lmn, lmx) + (float)rc * half_area(rmn, rmx);
            if (cost < FLT_MAX && cost < bc) { bc = cost; bi = j; bl = lc; }
        }
        for (uint32_t off = 16; off > 0; off >>= 1) {
            const float oc = __shfl_xor_sync(0xffffffffu, bc, off);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, off), ol = __shfl_xor_sync(0xffffffffu, bl, off);
            if (oc < bc || (oc == bc && oi < bi)) { bc = oc; bi = oi; bl = ol; }
        }
        if (bc < cheapest) { axis = a; pos = bi + 1; cheapest = bc; nl = bl; }
    }
    return cheapest;
}

// make_plan_bins for a whole warp over shared-memory bins (all lanes return
// the same plan, p not yet placed).
__device__ Plan make_plan_warp(const Ctx& C, const uint32_t* bins, uint32_t count, const float* nmn,
                               const float* nmx, const float* cmn, const float* cmx, uint32_t lane) {
    Plan P{};
    uint32_t axis, pos, nl;
    const float cost = warp_sweep(bins, C.bins, cmn, cmx, lane, axis, pos, nl);
    bool leaf;
    if (C.single) {
        leaf = count == 1;
    } else {
        bool force = C.max_leaf > 0 && count > C.max_leaf;
        float parent = (float)count * half_area(nmn, nmx);
        leaf = !force && cost >= parent;
    }
    P.axis = axis;
    P.pos = pos;
    P.partition = leaf ? 0u : 1u;
    if (leaf) return P;
    P.lo = cmn[axis];
    P.scale = pos > 0 ? (float)C.bins / (cmx[axis] - cmn[axis]) : 0.0f;
    P.nl = pos > 0 ? nl : 0u;
    P.p = count;
    P.children = (P.nl > 0 && P.nl < count) ? 1u : 0u;
    return P;
}

// Destination of local position i (closed form of the two-pointer loop).
__device__ __forceinline__ uint32_t partition_dst(const Ctx& C, const Plan& P, uint32_t first, uint32_t count,
                                                  uint32_t i, bool left, uint32_t lpre) {
    if (i < P.p) {
        if (left) return i;
        uint32_t m = i - lpre + 1;
        return (m == 1 ? count : C.G[first + m - 2]) - 1;
    }
    if (!left) return i - 1;
    uint32_t m = P.nl - lpre;
    return C.F[first + m - 1];
}

__device__ __forceinline__ void partition_rank(const Ctx& C, const Plan& P, uint32_t first, uint32_t i, bool left,
                                               uint32_t lpre) {
    if (i < P.p && !left) {
        C.F[first + (i - lpre)] = i;               // m = i - lpre + 1
    } else if (i >= P.p && left) {
        C.G[first + (P.nl - lpre) - 1] = i;        // m = nL - lpre
    }
}

// ---------------------------------------------------------------- preparation
__global__ void k_prep(Ctx C) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < C.n; t += stride) {
        const float* p = C.pos + 9ull * t;
        float c[3], mn[3], mx[3];
        for (int a = 0; a < 3; ++a) {
            float p0 = p[a], p1 = p[3 + a], p2 = p[6 + a];
            c[a] = ((p0 + p1) + p2) * 0.3333f;
            mn[a] = gmin(gmin(p0, p1), p2);
            mx[a] = gmax(gmax(p0, p1), p2);
        }
        C.cen[t] = make_float4(c[0], c[1], c[2], 0.0f);
        C.tmn[t] = make_float4(mn[0], mn[1], mn[2], 0.0f);
        C.tmx[t] = make_float4(mx[0], mx[1], mx[2], 0.0f);
        C.idx[t] = t;
    }
}

__device__ __forceinline__ void box_init(float* v) {
    for (int k = 0; k < 3; ++k) { v[k] = FLT_MAX; v[3 + k] = -FLT_MAX; v[6 + k] = FLT_MAX; v[9 + k] = -FLT_MAX; }
}
__device__ __forceinline__ void box_add(float* v, const Ctx& C, uint32_t t) {
    float4 mn = C.tmn[t], mx = C.tmx[t], c = C.cen[t];
    v[0] = gmin(v[0], mn.x); v[1] = gmin(v[1], mn.y); v[2] = gmin(v[2], mn.z);
    v[3] = gmax(v[3], mx.x); v[4] = gmax(v[4], mx.y); v[5] = gmax(v[5], mx.z);
    v[6] = gmin(v[6], c.x); v[7] = gmin(v[7], c.y); v[8] = gmin(v[8], c.z);
    v[9] = gmax(v[9], c.x); v[10] = gmax(v[10], c.y); v[11] = gmax(v[11], c.z);
}
// Signed zeros.  A bound equal to zero is +0.0 or -0.0 in the reference
// depending on which zero its glm fold met first (calc_node_min_max walks the
// node's triangles in index-list order and keeps the running value on ties).
// Alongside the value reductions the builder records, per box component, the
// first index-list position whose triangle bound is zero; a zero result takes
// that triangle's bits.
__device__ __forceinline__ float tri_comp(const Ctx& C, uint32_t t, int k) {
    const float4 v = k < 3 ? C.tmn[t] : C.tmx[t];
    return comp(v, (uint32_t)(k % 3));
}
__device__ __forceinline__ void zero_init(uint32_t* zp) {
    for (int k = 0; k < 6; ++k) zp[k] = kNone;
}
__device__ __forceinline__ void zero_add(uint32_t* zp, const Ctx& C, uint32_t t, uint32_t position) {
    const float4 mn = C.tmn[t], mx = C.tmx[t];
    const float v[6] = {mn.x, mn.y, mn.z, mx.x, mx.y, mx.z};
    for (int k = 0; k < 6; ++k)
        if (v[k] == 0.0f && zp[k] == kNone) zp[k] = position;
}
__device__ __forceinline__ void zero_warp_reduce(uint32_t* zp) {
    for (int off = 16; off > 0; off >>= 1)
        for (int k = 0; k < 6; ++k) zp[k] = min(zp[k], __shfl_xor_sync(0xffffffffu, zp[k], off));
}
__device__ __forceinline__ void zero_fix(const Ctx& C, float* v, const uint32_t* zp) {
    for (int k = 0; k < 6; ++k)
        if (v[k] == 0.0f && zp[k] != kNone) v[k] = tri_comp(C, C.idx[zp[k]], k);
}

__device__ __forceinline__ void box_warp_reduce(float* v) {
    for (int off = 16; off > 0; off >>= 1) {
        for (int k = 0; k < 12; ++k) {
            float o = __shfl_xor_sync(0xffffffffu, v[k], off);
            v[k] = ((k % 6) < 3) ? gmin(v[k], o) : gmax(v[k], o);
        }
    }
}
__device__ __forceinline__ void box_atomic(uint32_t* keys, const float* v, const uint32_t* zp) {
    for (int k = 0; k < 12; ++k) {
        if ((k % 6) < 3) atomicMin(&keys[k], fenc(v[k]));
        else atomicMax(&keys[k], fenc(v[k]));
    }
    for (int k = 0; k < 6; ++k)
        if (zp[k] != kNone) atomicMin(&keys[12 + k], zp[k]);
}

__device__ __forceinline__ uint32_t key_init(uint32_t k) {
    return k >= 12 ? kNone : (((k % 6) < 3) ? fenc(FLT_MAX) : fenc(-FLT_MAX));
}

// Bounds of the root (all positions) into slot keys.
__global__ void k_root_bounds(Ctx C, uint32_t* keys) {
    float v[12];
    uint32_t zp[6];
    box_init(v);
    zero_init(zp);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < C.n; i += stride) {
        const uint32_t t = C.idx[i];
        box_add(v, C, t);
        zero_add(zp, C, t, i);
    }
    box_warp_reduce(v);
    zero_warp_reduce(zp);
    if ((threadIdx.x & 31) == 0) box_atomic(keys, v, zp);
}

__global__ void k_keys_init(uint32_t* keys, uint32_t count_words) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count_words; i += stride)
        keys[i] = key_init(i % kBoxWords);
}

// ---------------------------------------------------------------- large-node phase
struct Level {
    uint32_t nslots;
    const uint32_t* slot_tmp;   // tmp node id per slot
    const uint32_t* slot_box;   // 12 keys per slot
    uint32_t* bins;             // slot x 3 x B x 7
    uint32_t* chunk_off;        // exclusive prefix of chunks per slot, [nslots] = total
    uint32_t* chunk_l;          // left-goers per chunk, then their per-slot exclusive prefix
    Plan* plan;                 // per slot
    uint32_t* child_slot;       // per slot x 2: next-level slot or kNone
    uint32_t* next_tmp;
    uint32_t* next_box;
    uint32_t* next_count;
};

__global__ void k_chunk_scan(Ctx C, Level Lv) {
    // one block of 1024 threads; each thread owns a contiguous run of slots
    __shared__ uint32_t part[1024];
    const uint32_t per = (Lv.nslots + 1023) / 1024;
    const uint32_t s0 = threadIdx.x * per, s1 = min(Lv.nslots, s0 + per);
    uint32_t sum = 0;
    for (uint32_t s = s0; s < s1; ++s) sum += (__float_as_uint(C.tb[Lv.slot_tmp[s]].w) + kChunk - 1) / kChunk;
    part[threadIdx.x] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {
        uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (uint32_t s = s0; s < s1; ++s) {
        Lv.chunk_off[s] = run;
        run += (__float_as_uint(C.tb[Lv.slot_tmp[s]].w) + kChunk - 1) / kChunk;
    }
    if (threadIdx.x == 1023) Lv.chunk_off[Lv.nslots] = part[1023];
}

// Maps a block to (slot, first, count, local range); false if past the end.
__device__ __forceinline__ bool chunk_of(const Ctx& C, const Level& Lv, uint32_t b, uint32_t& slot, uint32_t& first,
                                         uint32_t& count, uint32_t& i0, uint32_t& i1) {
    if (b >= Lv.chunk_off[Lv.nslots]) return false;
    uint32_t lo = 0, hi = Lv.nslots - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (Lv.chunk_off[mid] <= b) lo = mid; else hi = mid - 1;
    }
    slot = lo;
    const uint32_t t = Lv.slot_tmp[slot];
    first = __float_as_uint(C.ta[t].w);
    count = __float_as_uint(C.tb[t].w);
    i0 = (b - Lv.chunk_off[slot]) * kChunk;
    i1 = min(count, i0 + kChunk);
    return true;
}

__device__ __forceinline__ void bins_reset(uint32_t* sb, uint32_t words, uint32_t tid, uint32_t nthreads) {
    for (uint32_t w = tid; w < words; w += nthreads) {
        uint32_t k = w % kBinWords;
        sb[w] = k == 0 ? 0u : (k < 4 ? fenc(FLT_MAX) : fenc(-FLT_MAX));
    }
}

__device__ __forceinline__ void bin_element(const Ctx& C, uint32_t* sb, uint32_t t, const bool* deg, const float* lo,
                                            const float* scale) {
    const float4 c = C.cen[t], mn = C.tmn[t], mx = C.tmx[t];
    for (uint32_t a = 0; a < 3; ++a) {
        if (deg[a]) continue;
        int32_t bin = (int32_t)((comp(c, a) - lo[a]) * scale[a]);
        if ((int32_t)C.bins - 1 < bin) bin = (int32_t)C.bins - 1;
        uint32_t* e = sb + (a * C.bins + (uint32_t)bin) * kBinWords;
        atomicAdd(&e[0], 1u);
        atomicMin(&e[1], fenc(mn.x)); atomicMin(&e[2], fenc(mn.y)); atomicMin(&e[3], fenc(mn.z));
        atomicMax(&e[4], fenc(mx.x)); atomicMax(&e[5], fenc(mx.y)); atomicMax(&e[6], fenc(mx.z));
    }
}

__global__ void k_bins_reset(Ctx C, Level Lv) {
    const uint32_t words = Lv.nslots * 3 * C.bins * kBinWords;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += stride) {
        uint32_t k = w % kBinWords;
        Lv.bins[w] = k == 0 ? 0u : (k < 4 ? fenc(FLT_MAX) : fenc(-FLT_MAX));
    }
}

__global__ void __launch_bounds__(kChunkThreads) k_bin_chunks(Ctx C, Level Lv) {
    __shared__ uint32_t sb[3 * kMaxBins * kBinWords];
    uint32_t slot, first, count, i0, i1;
    if (!chunk_of(C, Lv, blockIdx.x, slot, first, count, i0, i1)) return;
    const uint32_t* key = Lv.slot_box + kBoxWords * slot;
    bool deg[3];
    float lo[3], scale[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = fdec(key[6 + a]);
        float hi = fdec(key[9 + a]);
        deg[a] = lo[a] == hi;
        scale[a] = deg[a] ? 0.0f : (float)C.bins / (hi - lo[a]);
    }
    const uint32_t words = 3 * C.bins * kBinWords;
    bins_reset(sb, words, threadIdx.x, blockDim.x);
    __syncthreads();
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) bin_element(C, sb, C.idx[first + i], deg, lo, scale);
    __syncthreads();
    uint32_t* gb = Lv.bins + (size_t)slot * words;
    for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) {
        const uint32_t k = w % kBinWords;
        if (deg[w / (C.bins * kBinWords)]) continue;
        if (k == 0) { if (sb[w]) atomicAdd(&gb[w], sb[w]); }
        else if (k < 4) atomicMin(&gb[w], sb[w]);
        else atomicMax(&gb[w], sb[w]);
    }
}

__global__ void k_plan(Ctx C, Level Lv) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= Lv.nslots) return;
    const uint32_t t = Lv.slot_tmp[s];
    const uint32_t* key = Lv.slot_box + kBoxWords * s;
    float box[6], cmn[3], cmx[3];
    for (int a = 0; a < 3; ++a) {
        box[a] = fdec(key[a]); box[3 + a] = fdec(key[3 + a]);
        cmn[a] = fdec(key[6 + a]); cmx[a] = fdec(key[9 + a]);
    }
    zero_fix(C, box, key + 12);
    const float* nmn = box;
    const float* nmx = box + 3;
    const uint32_t first = __float_as_uint(C.ta[t].w), count = __float_as_uint(C.tb[t].w);
    C.ta[t] = make_float4(nmn[0], nmn[1], nmn[2], __uint_as_float(first));
    C.tb[t] = make_float4(nmx[0], nmx[1], nmx[2], __uint_as_float(count));
    Lv.plan[s] = make_plan(C, Lv.bins + (size_t)s * 3 * C.bins * kBinWords, first, count, nmn, nmx, cmn, cmx);
}

// Block-wide exclusive prefix of a flag (blockDim.x <= 1024); returns the prefix
// and writes the block total to *total.
__device__ __forceinline__ uint32_t block_prefix(bool flag, uint32_t* warp_sums, uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    const uint32_t in_warp = __popc(m & ((1u << lane) - 1u));
    if (lane == 0) warp_sums[warp] = __popc(m);
    __syncthreads();
    uint32_t before = 0, all = 0;
    for (uint32_t w = 0; w < nw; ++w) {
        if (w < warp) before += warp_sums[w];
        all += warp_sums[w];
    }
    __syncthreads();
    *total = all;
    return before + in_warp;
}

__global__ void __launch_bounds__(kChunkThreads) k_part_count(Ctx C, Level Lv) {
    __shared__ uint32_t ws[32];
    uint32_t slot, first, count, i0, i1;
    if (!chunk_of(C, Lv, blockIdx.x, slot, first, count, i0, i1)) return;
    const Plan P = Lv.plan[slot];
    if (!P.partition) return;
    uint32_t sum = 0;
    for (uint32_t base = i0; base < i1; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool left = i < i1 && goes_left(C, P, C.idx[first + i]);
        uint32_t tot;
        block_prefix(left, ws, &tot);
        sum += tot;
    }
    if (threadIdx.x == 0) Lv.chunk_l[blockIdx.x] = sum;
}

__global__ void k_part_slot_scan(Ctx C, Level Lv) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= Lv.nslots || !Lv.plan[s].partition) return;
    uint32_t run = 0;
    for (uint32_t b = Lv.chunk_off[s]; b < Lv.chunk_off[s + 1]; ++b) {
        uint32_t v = Lv.chunk_l[b];
        Lv.chunk_l[b] = run;
        run += v;
    }
}

template <bool MOVE>
__global__ void __launch_bounds__(kChunkThreads) k_part_pass(Ctx C, Level Lv) {
    __shared__ uint32_t ws[32];
    uint32_t slot, first, count, i0, i1;
    if (!chunk_of(C, Lv, blockIdx.x, slot, first, count, i0, i1)) return;
    const Plan P = Lv.plan[slot];
    if (!P.partition) return;
    uint32_t run = Lv.chunk_l[blockIdx.x];
    for (uint32_t base = i0; base < i1; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < i1;
        const uint32_t t = valid ? C.idx[first + i] : 0u;
        const bool left = valid && goes_left(C, P, t);
        uint32_t tot;
        const uint32_t lpre = run + block_prefix(left, ws, &tot);
        if (valid) {
            if (MOVE) C.idx_tmp[first + partition_dst(C, P, first, count, i, left, lpre)] = t;
            else partition_rank(C, P, first, i, left, lpre);
        }
        run += tot;
    }
}

__global__ void __launch_bounds__(kChunkThreads) k_part_copy(Ctx C, Level Lv) {
    uint32_t slot, first, count, i0, i1;
    if (!chunk_of(C, Lv, blockIdx.x, slot, first, count, i0, i1)) return;
    if (!Lv.plan[slot].partition) return;
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) C.idx[first + i] = C.idx_tmp[first + i];
}

__device__ __forceinline__ void new_children(const Ctx& C, uint32_t X, uint32_t first, uint32_t count, uint32_t nl,
                                             uint32_t& L) {
    L = atomicAdd(&C.tcount[0], 2u);
    const uint32_t d = C.tdepth[X] + 1;
    C.ta[L] = make_float4(0, 0, 0, __uint_as_float(first));
    C.tb[L] = make_float4(0, 0, 0, __uint_as_float(nl));
    C.ta[L + 1] = make_float4(0, 0, 0, __uint_as_float(first + nl));
    C.tb[L + 1] = make_float4(0, 0, 0, __uint_as_float(count - nl));
    C.tleft[L] = kNone;
    C.tleft[L + 1] = kNone;
    C.tdepth[L] = d;
    C.tdepth[L + 1] = d;
    C.tleft[X] = L;
    atomicMax(&C.tcount[1], d);
}

__global__ void k_children(Ctx C, Level Lv) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= Lv.nslots) return;
    const Plan P = Lv.plan[s];
    Lv.child_slot[2 * s] = kNone;
    Lv.child_slot[2 * s + 1] = kNone;
    if (!P.children) return;
    const uint32_t X = Lv.slot_tmp[s];
    const uint32_t first = __float_as_uint(C.ta[X].w), count = __float_as_uint(C.tb[X].w);
    uint32_t L;
    new_children(C, X, first, count, P.nl, L);
    const uint32_t cnt[2] = {P.nl, count - P.nl};
    for (uint32_t side = 0; side < 2; ++side) {
        if (cnt[side] > kSmall) {
            const uint32_t j = atomicAdd(Lv.next_count, 1u);
            Lv.next_tmp[j] = L + side;
            uint32_t* key = Lv.next_box + kBoxWords * j;
            for (uint32_t k = 0; k < kBoxWords; ++k) key[k] = key_init(k);
            Lv.child_slot[2 * s + side] = j;
        } else {
            C.small_list[atomicAdd(&C.tcount[2], 1u)] = L + side;
        }
    }
}

__global__ void __launch_bounds__(kChunkThreads) k_child_bounds(Ctx C, Level Lv) {
    uint32_t slot, first, count, i0, i1;
    if (!chunk_of(C, Lv, blockIdx.x, slot, first, count, i0, i1)) return;
    const Plan P = Lv.plan[slot];
    if (!P.children) return;
    const uint32_t j0 = Lv.child_slot[2 * slot], j1 = Lv.child_slot[2 * slot + 1];
    if (j0 == kNone && j1 == kNone) return;
    float v0[12], v1[12];
    uint32_t z0[6], z1[6];
    box_init(v0);
    box_init(v1);
    zero_init(z0);
    zero_init(z1);
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const uint32_t t = C.idx[first + i];
        if (i < P.nl) {
            if (j0 != kNone) { box_add(v0, C, t); zero_add(z0, C, t, first + i); }
        } else if (j1 != kNone) {
            box_add(v1, C, t);
            zero_add(z1, C, t, first + i);
        }
    }
    box_warp_reduce(v0);
    box_warp_reduce(v1);
    zero_warp_reduce(z0);
    zero_warp_reduce(z1);
    if ((threadIdx.x & 31) == 0) {
        if (j0 != kNone && i0 < P.nl) box_atomic(Lv.next_box + kBoxWords * j0, v0, z0);
        if (j1 != kNone && i1 > P.nl) box_atomic(Lv.next_box + kBoxWords * j1, v1, z1);
    }
}

// ---------------------------------------------------------------- small-subtree phase
// One warp (one CTA) builds a whole subtree of at most kSmall triangles with
// the subtree held in shared memory: each triangle's centroid, min and max
// corner (component k of local triangle j at d[k * kSmall + j]), its index,
// and a 16-bit permutation of local triangles that the partitions reorder.
// Only the node records and the final index list go to global memory.  Node
// ids come from one reservation of 2 * (count - 1) per subtree (a subtree of
// count triangles splits at most count - 1 times); ids a subtree does not use
// keep tdepth = kNone and are skipped by the renumbering.  The warp descends
// into the smaller child and keeps the larger on a lane-distributed stack, so
// at most log2(kSmall) + 1 entries are pending.
struct SmallSmem {
    float* d;
    uint32_t* oidx;
    uint16_t *perm, *ptmp, *F, *G;
    uint32_t* bins;
};

__host__ __device__ constexpr size_t small_smem_bytes(uint32_t bins) {
    return (9ull + 1ull) * 4ull * kSmall + 4ull * 2ull * kSmall + 4ull * 3ull * bins * kBinWords;
}

__global__ void __launch_bounds__(32) k_small(Ctx C, uint32_t nsmall, uint32_t tcap) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    SmallSmem S;
    S.d = reinterpret_cast<float*>(smem_raw);
    S.oidx = reinterpret_cast<uint32_t*>(S.d + 9 * kSmall);
    S.perm = reinterpret_cast<uint16_t*>(S.oidx + kSmall);
    S.ptmp = S.perm + kSmall;
    S.F = S.ptmp + kSmall;
    S.G = S.F + kSmall;
    S.bins = reinterpret_cast<uint32_t*>(S.G + kSmall);
    const uint32_t lane = threadIdx.x;
    const uint32_t words = 3 * C.bins * kBinWords;
    for (uint32_t w = blockIdx.x; w < nsmall; w += gridDim.x) {
        const uint32_t R = C.small_list[w];
        const uint32_t gfirst = __float_as_uint(C.ta[R].w), count = __float_as_uint(C.tb[R].w);
        const uint32_t depth0 = C.tdepth[R];
        for (uint32_t i = lane; i < count; i += 32) {
            const uint32_t t = C.idx[gfirst + i];
            const float4 c = C.cen[t], mn = C.tmn[t], mx = C.tmx[t];
            S.d[0 * kSmall + i] = c.x;  S.d[1 * kSmall + i] = c.y;  S.d[2 * kSmall + i] = c.z;
            S.d[3 * kSmall + i] = mn.x; S.d[4 * kSmall + i] = mn.y; S.d[5 * kSmall + i] = mn.z;
            S.d[6 * kSmall + i] = mx.x; S.d[7 * kSmall + i] = mx.y; S.d[8 * kSmall + i] = mx.z;
            S.oidx[i] = t;
            S.perm[i] = (uint16_t)i;
        }
        uint32_t L0 = 0;
        if (lane == 0) L0 = atomicAdd(&C.tcount[0], 2u * (count - 1));
        L0 = __shfl_sync(0xffffffffu, L0, 0);
        if ((uint64_t)L0 + 2ull * (count - 1) > tcap) {   // cannot happen for tcap = 2n + 2n / kSmall + 4
            if (lane == 0) atomicOr(&C.tcount[3], 1u);
            continue;
        }
        __syncwarp();
        uint32_t splits = 0, maxd = depth0, sp = 0;
        uint32_t sX = 0, sf = 0, sc = 0, sd = 0;   // stack entry `lane`
        uint32_t X = R, f = 0, c = count, dep = depth0;
        for (;;) {
            // node bounds, centroid bounds and first zero positions
            float v[12];
            uint32_t zp[6];
            box_init(v);
            zero_init(zp);
            for (uint32_t i = lane; i < c; i += 32) {
                const uint32_t j = S.perm[f + i];
                float e[9];
                for (int k = 0; k < 9; ++k) e[k] = S.d[k * kSmall + j];
                v[0] = gmin(v[0], e[3]); v[1] = gmin(v[1], e[4]); v[2] = gmin(v[2], e[5]);
                v[3] = gmax(v[3], e[6]); v[4] = gmax(v[4], e[7]); v[5] = gmax(v[5], e[8]);
                v[6] = gmin(v[6], e[0]); v[7] = gmin(v[7], e[1]); v[8] = gmin(v[8], e[2]);
                v[9] = gmax(v[9], e[0]); v[10] = gmax(v[10], e[1]); v[11] = gmax(v[11], e[2]);
                for (int k = 0; k < 6; ++k)
                    if (e[3 + k] == 0.0f && zp[k] == kNone) zp[k] = i;
            }
            box_warp_reduce(v);
            zero_warp_reduce(zp);
            for (int k = 0; k < 6; ++k)
                if (v[k] == 0.0f && zp[k] != kNone) v[k] = S.d[(3 + k) * kSmall + S.perm[f + zp[k]]];
            if (lane == 0) {
                C.ta[X] = make_float4(v[0], v[1], v[2], __uint_as_float(gfirst + f));
                C.tb[X] = make_float4(v[3], v[4], v[5], __uint_as_float(c));
                C.tleft[X] = kNone;
                C.tdepth[X] = dep;
            }
            bool deg[3];
            float lo[3], scale[3];
            for (int a = 0; a < 3; ++a) {
                lo[a] = v[6 + a];
                deg[a] = v[6 + a] == v[9 + a];
                scale[a] = deg[a] ? 0.0f : (float)C.bins / (v[9 + a] - v[6 + a]);
            }
            bins_reset(S.bins, words, lane, 32);
            __syncwarp();
            for (uint32_t i = lane; i < c; i += 32) {
                const uint32_t j = S.perm[f + i];
                for (uint32_t a = 0; a < 3; ++a) {
                    if (deg[a]) continue;
                    int32_t bin = (int32_t)((S.d[a * kSmall + j] - lo[a]) * scale[a]);
                    if ((int32_t)C.bins - 1 < bin) bin = (int32_t)C.bins - 1;
                    uint32_t* e = S.bins + (a * C.bins + (uint32_t)bin) * kBinWords;
                    atomicAdd(&e[0], 1u);
                    atomicMin(&e[1], fenc(S.d[3 * kSmall + j]));
                    atomicMin(&e[2], fenc(S.d[4 * kSmall + j]));
                    atomicMin(&e[3], fenc(S.d[5 * kSmall + j]));
                    atomicMax(&e[4], fenc(S.d[6 * kSmall + j]));
                    atomicMax(&e[5], fenc(S.d[7 * kSmall + j]));
                    atomicMax(&e[6], fenc(S.d[8 * kSmall + j]));
                }
            }
            __syncwarp();
            Plan P = make_plan_warp(C, S.bins, c, v, v + 3, v + 6, v + 9, lane);
            if (P.partition && P.nl < c)
                P.p = P.nl + (goes_left_c(C, P, S.d[P.axis * kSmall + S.perm[f + P.nl]]) ? 0u : 1u);
            __syncwarp();
            if (P.partition) {
                // the closed form of the two-pointer partition (see the file head),
                // positions relative to the node's first position f
                for (int pass = 0; pass < 2; ++pass) {
                    uint32_t run = 0;
                    for (uint32_t base = 0; base < c; base += 32) {
                        const uint32_t i = base + lane;
                        const bool valid = i < c;
                        const uint32_t j = valid ? S.perm[f + i] : 0u;
                        const bool left = valid && goes_left_c(C, P, S.d[P.axis * kSmall + j]);
                        const unsigned m = __ballot_sync(0xffffffffu, left);
                        const uint32_t lpre = run + __popc(m & ((1u << lane) - 1u));
                        if (valid) {
                            if (pass == 0) {
                                if (i < P.p && !left) S.F[f + (i - lpre)] = (uint16_t)i;
                                else if (i >= P.p && left) S.G[f + (P.nl - lpre) - 1] = (uint16_t)i;
                            } else {
                                uint32_t dst;
                                if (i < P.p) {
                                    const uint32_t mm = i - lpre + 1;
                                    dst = left ? i : (mm == 1 ? c : (uint32_t)S.G[f + mm - 2]) - 1;
                                } else {
                                    dst = !left ? i - 1 : (uint32_t)S.F[f + (P.nl - lpre) - 1];
                                }
                                S.ptmp[f + dst] = (uint16_t)j;
                            }
                        }
                        run += __popc(m);
                    }
                    __syncwarp();
                }
                for (uint32_t i = lane; i < c; i += 32) S.perm[f + i] = S.ptmp[f + i];
                __syncwarp();
            }
            if (P.children) {
                const uint32_t L = L0 + 2 * splits++;
                if (lane == 0) C.tleft[X] = L;
                const uint32_t nl = P.nl, nr = c - P.nl;
                maxd = max(maxd, dep + 1);
                // descend into the smaller child, push the larger
                const bool go_left = nl <= nr;
                if (lane == sp) {
                    sX = go_left ? L + 1 : L;
                    sf = go_left ? f + nl : f;
                    sc = go_left ? nr : nl;
                    sd = dep + 1;
                }
                ++sp;
                X = go_left ? L : L + 1;
                f = go_left ? f : f + nl;
                c = go_left ? nl : nr;
                dep = dep + 1;
                continue;
            }
            if (sp == 0) break;
            --sp;
            X = __shfl_sync(0xffffffffu, sX, sp);
            f = __shfl_sync(0xffffffffu, sf, sp);
            c = __shfl_sync(0xffffffffu, sc, sp);
            dep = __shfl_sync(0xffffffffu, sd, sp);
        }
        for (uint32_t i = lane; i < count; i += 32) C.idx[gfirst + i] = S.oidx[S.perm[i]];
        if (lane == 0) atomicMax(&C.tcount[1], maxd);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- renumbering and output
__global__ void k_internal_count(Ctx C, uint32_t T, uint32_t depth, uint32_t* ic) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t X = blockIdx.x * blockDim.x + threadIdx.x; X < T; X += stride) {
        if (C.tdepth[X] != depth) continue;
        const uint32_t L = C.tleft[X];
        ic[X] = L == kNone ? 0u : 1u + ic[L] + ic[L + 1];
    }
}

__global__ void k_rank(Ctx C, uint32_t T, uint32_t depth, const uint32_t* ic, uint32_t* rank, uint32_t* fidx) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t X = blockIdx.x * blockDim.x + threadIdx.x; X < T; X += stride) {
        if (C.tdepth[X] != depth) continue;
        const uint32_t L = C.tleft[X];
        if (L == kNone) continue;
        const uint32_t r = rank[X];
        fidx[L] = 2 + 2 * r;
        fidx[L + 1] = 3 + 2 * r;
        rank[L] = r + 1;
        rank[L + 1] = r + 1 + ic[L];
    }
}

__global__ void k_emit(Ctx C, uint32_t T, const uint32_t* rank, const uint32_t* fidx, float4* out) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t X = blockIdx.x * blockDim.x + threadIdx.x; X < T; X += stride) {
        if (C.tdepth[X] == kNone) continue;   // id reserved by a small subtree but not used
        const float4 a = C.ta[X], b = C.tb[X];
        const bool internal = C.tleft[X] != kNone;
        const uint32_t f = fidx[X];
        out[2ull * f] = make_float4(a.x, a.y, a.z, internal ? __uint_as_float(2 + 2 * rank[X]) : a.w);
        out[2ull * f + 1] = make_float4(b.x, b.y, b.z, internal ? __uint_as_float(0u) : b.w);
    }
}

__global__ void k_leaf_tris(Ctx C, float4* out) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < C.n; i += stride) {
        const uint32_t t = C.idx[i];
        const float* p = C.pos + 9ull * t;
        out[3ull * i] = make_float4(p[0], p[1], p[2], __uint_as_float(t));
        out[3ull * i + 1] = make_float4(p[3] - p[0], p[4] - p[1], p[5] - p[2], 0.0f);
        out[3ull * i + 2] = make_float4(p[6] - p[0], p[7] - p[1], p[8] - p[2], 0.0f);
    }
}

// ---------------------------------------------------------------- host side
// One device allocation for all of a build's scratch, carved into 256-byte
// aligned parts (one cudaMalloc / cudaFree per build instead of one per array).
struct Arena {
    size_t bytes = 0;
    template <typename T>
    size_t part(size_t count) {
        const size_t off = bytes;
        bytes += (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~size_t(255);
        return off;
    }
};

struct DeviceBlock {
    void* p = nullptr;
    ~DeviceBlock() { dfree(p); }
};

unsigned blocks_for(uint64_t n, unsigned threads, unsigned cap = 152u * 16u) {
    uint64_t b = (n + threads - 1) / threads;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, cap));
}

#define BVH_CUDA(call)                                                               \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            g_err = std::string(#call) + ": " + cudaGetErrorString(e_);              \
            return e_ == cudaErrorMemoryAllocation ? WF_ERR_OOM : WF_ERR_CUDA;       \
        }                                                                            \
    } while (0)

}  // namespace

const char* bvh_last_error() { return g_err.c_str(); }

int gpu_bvh_build(const triangle_t* tris, uint32_t n, const wf_bvh_options& o, cudaStream_t st, BvhBuildOut* out) {
    if (n == 0 || !tris || !out) { g_err = "gpu_bvh_build: empty mesh"; return WF_ERR_INVALID; }
    if (o.interval_count < 2 || o.interval_count > kMaxBins) {
        g_err = "gpu_bvh_build: interval_count must be 2..64";
        return WF_ERR_INVALID;
    }
    if (n > (1u << 30)) { g_err = "gpu_bvh_build: too many triangles"; return WF_ERR_CAPACITY; }
    const uint32_t B = o.interval_count;
    // 2n + 2 ids hold any binary tree over n triangles; the small phase reserves
    // 2 * (count - 1) per subtree, which can leave up to 2 * (large leaves) more
    const uint64_t tcap = 2ull * n + 2ull * (n / kSmall) + 4;
    const uint32_t maxslots = n / kSmall + 2;
    const uint32_t maxchunks = n / kChunk + maxslots + 1;
    const uint64_t max_nodes = 2ull * n;   // 2 + 2 * (internal nodes <= n - 1)

    Arena A;
    const size_t o_pos = A.part<float>(9ull * n), o_cen = A.part<float4>(n), o_tmn = A.part<float4>(n),
                 o_tmx = A.part<float4>(n), o_idx = A.part<uint32_t>(n), o_idx_tmp = A.part<uint32_t>(n),
                 o_F = A.part<uint32_t>(n), o_G = A.part<uint32_t>(n), o_ta = A.part<float4>(tcap),
                 o_tb = A.part<float4>(tcap), o_tleft = A.part<uint32_t>(tcap), o_tdepth = A.part<uint32_t>(tcap),
                 o_tcount = A.part<uint32_t>(4), o_small = A.part<uint32_t>(n);
    const size_t o_st0 = A.part<uint32_t>(maxslots), o_st1 = A.part<uint32_t>(maxslots),
                 o_sb0 = A.part<uint32_t>(kBoxWords * maxslots), o_sb1 = A.part<uint32_t>(kBoxWords * maxslots),
                 o_bins = A.part<uint32_t>((size_t)maxslots * 3 * B * kBinWords),
                 o_choff = A.part<uint32_t>(maxslots + 1), o_chl = A.part<uint32_t>(maxchunks),
                 o_plan = A.part<Plan>(maxslots), o_child = A.part<uint32_t>(2ull * maxslots),
                 o_next = A.part<uint32_t>(1), o_ic = A.part<uint32_t>(tcap), o_rank = A.part<uint32_t>(tcap),
                 o_fidx = A.part<uint32_t>(tcap);
    const size_t o_nodes = out->keep_device ? 0 : A.part<float4>(2 * max_nodes);
    DeviceBlock scratch;
    {
        const cudaError_t e = dmalloc(&scratch.p, A.bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            g_err = std::string("gpu_bvh_build: cudaMalloc: ") + cudaGetErrorString(e);
            return WF_ERR_OOM;
        }
    }
    uint8_t* base = static_cast<uint8_t*>(scratch.p);
    auto at = [base](size_t off) { return static_cast<void*>(base + off); };

    // triangle positions, gathered on the host threads
    std::unique_ptr<float[]> hpos(new (std::nothrow) float[9ull * n]);
    if (!hpos) { g_err = "gpu_bvh_build: host allocation failed"; return WF_ERR_OOM; }
    host_parallel(n, 1u << 16, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            std::memcpy(&hpos[9 * i], tris[i].v0.position, 12);
            std::memcpy(&hpos[9 * i + 3], tris[i].v1.position, 12);
            std::memcpy(&hpos[9 * i + 6], tris[i].v2.position, 12);
        }
    });

    Ctx C{};
    C.n = n; C.bins = B; C.single = o.subdivide_single_prim ? 1u : 0u; C.max_leaf = o.max_leaf_prims;
    float* d_pos = static_cast<float*>(at(o_pos));
    C.pos = d_pos;
    C.cen = static_cast<float4*>(at(o_cen)); C.tmn = static_cast<float4*>(at(o_tmn));
    C.tmx = static_cast<float4*>(at(o_tmx));
    C.idx = static_cast<uint32_t*>(at(o_idx)); C.idx_tmp = static_cast<uint32_t*>(at(o_idx_tmp));
    C.F = static_cast<uint32_t*>(at(o_F)); C.G = static_cast<uint32_t*>(at(o_G));
    C.ta = static_cast<float4*>(at(o_ta)); C.tb = static_cast<float4*>(at(o_tb));
    C.tleft = static_cast<uint32_t*>(at(o_tleft)); C.tdepth = static_cast<uint32_t*>(at(o_tdepth));
    C.tcount = static_cast<uint32_t*>(at(o_tcount));
    C.small_list = static_cast<uint32_t*>(at(o_small));
    uint32_t* slot_tmp[2] = {static_cast<uint32_t*>(at(o_st0)), static_cast<uint32_t*>(at(o_st1))};
    uint32_t* slot_box[2] = {static_cast<uint32_t*>(at(o_sb0)), static_cast<uint32_t*>(at(o_sb1))};
    uint32_t* bins = static_cast<uint32_t*>(at(o_bins));
    uint32_t* chunk_off = static_cast<uint32_t*>(at(o_choff));
    uint32_t* chunk_l = static_cast<uint32_t*>(at(o_chl));
    Plan* plan = static_cast<Plan*>(at(o_plan));
    uint32_t* child_slot = static_cast<uint32_t*>(at(o_child));
    uint32_t* next_count = static_cast<uint32_t*>(at(o_next));
    uint32_t* ic = static_cast<uint32_t*>(at(o_ic));
    uint32_t* rank = static_cast<uint32_t*>(at(o_rank));
    uint32_t* fidx = static_cast<uint32_t*>(at(o_fidx));

    BVH_CUDA(cudaMemcpyAsync(d_pos, hpos.get(), 36ull * n, cudaMemcpyHostToDevice, st));
    k_prep<<<blocks_for(n, 256), 256, 0, st>>>(C);
    // root = temporary node 0
    {
        const float4 a = make_float4(0, 0, 0, 0);
        float4 b = make_float4(0, 0, 0, 0);
        uint32_t nn = n;
        std::memcpy(&b.w, &nn, 4);
        const uint32_t init[4] = {1u, 0u, 0u, 0u}, none = kNone, zero = 0u;
        BVH_CUDA(cudaMemcpyAsync(C.ta, &a, 16, cudaMemcpyHostToDevice, st));
        BVH_CUDA(cudaMemcpyAsync(C.tb, &b, 16, cudaMemcpyHostToDevice, st));
        BVH_CUDA(cudaMemcpyAsync(C.tleft, &none, 4, cudaMemcpyHostToDevice, st));
        BVH_CUDA(cudaMemcpyAsync(C.tdepth, &zero, 4, cudaMemcpyHostToDevice, st));
        BVH_CUDA(cudaMemcpyAsync(C.tcount, init, 16, cudaMemcpyHostToDevice, st));
        BVH_CUDA(cudaStreamSynchronize(st));   // the host copies above read stack variables
    }
    uint32_t nslots = 0;
    if (n > kSmall) {
        const uint32_t zero = 0u;
        BVH_CUDA(cudaMemcpyAsync(slot_tmp[0], &zero, 4, cudaMemcpyHostToDevice, st));
        k_keys_init<<<1, 32, 0, st>>>(slot_box[0], kBoxWords);
        k_root_bounds<<<blocks_for(n, 256), 256, 0, st>>>(C, slot_box[0]);
        BVH_CUDA(cudaStreamSynchronize(st));
        nslots = 1;
    } else {
        const uint32_t zero = 0u, one = 1u;
        BVH_CUDA(cudaMemcpyAsync(C.small_list, &zero, 4, cudaMemcpyHostToDevice, st));
        BVH_CUDA(cudaMemcpyAsync(C.tcount + 2, &one, 4, cudaMemcpyHostToDevice, st));
        BVH_CUDA(cudaStreamSynchronize(st));
    }
    int cur = 0;
    while (nslots > 0) {
        Level Lv;
        Lv.nslots = nslots;
        Lv.slot_tmp = slot_tmp[cur];
        Lv.slot_box = slot_box[cur];
        Lv.bins = bins;
        Lv.chunk_off = chunk_off;
        Lv.chunk_l = chunk_l;
        Lv.plan = plan;
        Lv.child_slot = child_slot;
        Lv.next_tmp = slot_tmp[cur ^ 1];
        Lv.next_box = slot_box[cur ^ 1];
        Lv.next_count = next_count;
        // chunks in this level: sum of ceil(count / kChunk) <= n / kChunk + nslots
        const unsigned grid = (unsigned)std::min<uint64_t>(maxchunks, (uint64_t)n / kChunk + nslots + 1);
        const unsigned sgrid = (nslots + 127) / 128;
        BVH_CUDA(cudaMemsetAsync(next_count, 0, 4, st));
        k_chunk_scan<<<1, 1024, 0, st>>>(C, Lv);
        k_bins_reset<<<blocks_for((uint64_t)nslots * 3 * B * kBinWords, 256), 256, 0, st>>>(C, Lv);
        k_bin_chunks<<<grid, kChunkThreads, 0, st>>>(C, Lv);
        k_plan<<<sgrid, 128, 0, st>>>(C, Lv);
        k_part_count<<<grid, kChunkThreads, 0, st>>>(C, Lv);
        k_part_slot_scan<<<sgrid, 128, 0, st>>>(C, Lv);
        k_part_pass<false><<<grid, kChunkThreads, 0, st>>>(C, Lv);
        k_part_pass<true><<<grid, kChunkThreads, 0, st>>>(C, Lv);
        k_part_copy<<<grid, kChunkThreads, 0, st>>>(C, Lv);
        k_children<<<sgrid, 128, 0, st>>>(C, Lv);
        k_child_bounds<<<grid, kChunkThreads, 0, st>>>(C, Lv);
        BVH_CUDA(cudaGetLastError());
        BVH_CUDA(cudaMemcpyAsync(&nslots, next_count, 4, cudaMemcpyDeviceToHost, st));
        BVH_CUDA(cudaStreamSynchronize(st));
        cur ^= 1;
    }
    uint32_t counts[4];
    BVH_CUDA(cudaMemcpyAsync(counts, C.tcount, 12, cudaMemcpyDeviceToHost, st));
    BVH_CUDA(cudaStreamSynchronize(st));
    if (counts[2] > 0) {
        // ids from counts[0] on are reserved per small subtree; unused ones keep depth kNone
        BVH_CUDA(cudaMemsetAsync(C.tdepth + counts[0], 0xFF, 4ull * (tcap - counts[0]), st));
        const size_t smem = small_smem_bytes(B);
        BVH_CUDA(cudaFuncSetAttribute(k_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_small<<<counts[2], 32, smem, st>>>(C, counts[2], (uint32_t)tcap);
        BVH_CUDA(cudaGetLastError());
    }
    BVH_CUDA(cudaMemcpyAsync(counts, C.tcount, 16, cudaMemcpyDeviceToHost, st));
    BVH_CUDA(cudaStreamSynchronize(st));
    if (counts[3] != 0) {
        g_err = "gpu_bvh_build: small-subtree node ids exceeded the reserved range";
        return WF_ERR_CAPACITY;
    }
    const uint32_t T = counts[0], maxd = counts[1];
    const unsigned tgrid = blocks_for(T, 256);
    for (int d = (int)maxd; d >= 0; --d) k_internal_count<<<tgrid, 256, 0, st>>>(C, T, (uint32_t)d, ic);
    BVH_CUDA(cudaMemsetAsync(rank, 0, 4, st));
    BVH_CUDA(cudaMemsetAsync(fidx, 0, 4, st));
    for (uint32_t d = 0; d < maxd; ++d) k_rank<<<tgrid, 256, 0, st>>>(C, T, d, ic, rank, fidx);
    uint32_t internal = 0;
    BVH_CUDA(cudaMemcpyAsync(&internal, ic, 4, cudaMemcpyDeviceToHost, st));
    BVH_CUDA(cudaStreamSynchronize(st));
    const uint32_t nc = 2 + 2 * internal;
    float4* d_nodes = nullptr;
    float4* d_tris = nullptr;
    if (out->keep_device) {
        BVH_CUDA(dmalloc(reinterpret_cast<void**>(&d_nodes), 32ull * nc));
        if (dmalloc(reinterpret_cast<void**>(&d_tris), 48ull * n) != cudaSuccess) {
            dfree(d_nodes);
            cudaGetLastError();
            g_err = "gpu_bvh_build: cudaMalloc failed";
            return WF_ERR_OOM;
        }
    } else {
        d_nodes = static_cast<float4*>(at(o_nodes));
    }
    auto drop = [&]() {
        if (out->keep_device) {
            dfree(d_nodes);
            dfree(d_tris);
        }
    };
    cudaError_t e = cudaMemsetAsync(d_nodes, 0, 32ull * nc, st);
    k_emit<<<tgrid, 256, 0, st>>>(C, T, rank, fidx, d_nodes);
    if (d_tris) k_leaf_tris<<<blocks_for(n, 256), 256, 0, st>>>(C, d_tris);
    if (e == cudaSuccess) e = cudaGetLastError();
    // blob: [header | nodes | bvh_triangle_t (original order) | index list], written
    // straight into the caller's buffer when it is large enough
    const uint64_t nodes_bytes = 32ull * nc, tri_bytes = 36ull * n, idx_bytes = 4ull * n;
    const uint64_t size = 12 + nodes_bytes + tri_bytes + idx_bytes;
    uint8_t* blob;
    if (out->dst && out->dst_capacity >= size) {
        blob = out->dst;
        out->in_dst = true;
    } else {
        out->blob.resize(size);
        blob = out->blob.data();
        out->in_dst = false;
    }
    out->blob_size = size;
    if (e == cudaSuccess) e = cudaMemcpyAsync(blob + 12, d_nodes, nodes_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(blob + 12 + nodes_bytes + tri_bytes, C.idx, idx_bytes, cudaMemcpyDeviceToHost, st);
    uint8_t* tri_dst = blob + 12 + nodes_bytes;
    host_parallel(tri_bytes, 1u << 22, [&](uint64_t lo, uint64_t hi) {
        std::memcpy(tri_dst + lo, reinterpret_cast<const uint8_t*>(hpos.get()) + lo, hi - lo);
    });
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        drop();
        g_err = std::string("gpu_bvh_build: ") + cudaGetErrorString(e);
        return WF_ERR_CUDA;
    }
    bvh_header_t h;
    h.nodes_offset = 12;
    h.triangles_offset = (uint32_t)(12 + nodes_bytes);
    h.indices_offset = (uint32_t)(12 + nodes_bytes + tri_bytes);
    std::memcpy(blob, &h, 12);
    bvh_node_t root;
    std::memcpy(&root, blob + 12, 32);
    std::memcpy(out->root_min, root.aabb_min, 12);
    std::memcpy(out->root_max, root.aabb_max, 12);
    out->node_count = nc;
    out->d_nodes = out->keep_device ? d_nodes : nullptr;
    out->d_tris = d_tris;
    return WF_OK;
}

}  // namespace wf
