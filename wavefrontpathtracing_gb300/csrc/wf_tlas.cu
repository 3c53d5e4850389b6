// wf_tlas.cu — agglomerative TLAS builder on the GPU, node-for-node identical
// to tlas_builder_t::build (tlas_builder.cpp:6-68).
//
// The reference's A/B/C walk is inherently sequential: each step asks
// find_best_match (:86-110) for the partner of one node among the remaining
// ones.  One warp runs the walk; every find_best_match is a warp-parallel scan
// of the remaining list (each lane scans a strided slice in increasing order,
// keeping its first strict minimum, then a shuffle reduction takes the
// smallest value and, on equal values, the smallest list position — exactly
// the element the reference's sequential "area < smallest" loop keeps).  The
// remaining list and its boxes live in shared memory when they fit.
#include <mutex>

#include "../../include/wf.h"
#include "wf_kernels.h"

namespace wf {

namespace {

constexpr uint32_t kSmemInstances = 7168;   // 7 words per list entry -> 200,704 bytes

__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }   // glm::min
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }   // glm::max

struct List {
    uint32_t* idx;   // node index per list position
    float* bmn;      // 3 floats per position
    float* bmx;
};

// find_best_match: partner of list position X among positions [0, count).
__device__ uint32_t best_match(const List& L, uint32_t X, uint32_t count, uint32_t metric) {
    const uint32_t lane = threadIdx.x;
    const float ax0 = L.bmn[3 * X], ax1 = L.bmn[3 * X + 1], ax2 = L.bmn[3 * X + 2];
    const float bx0 = L.bmx[3 * X], bx1 = L.bmx[3 * X + 1], bx2 = L.bmx[3 * X + 2];
    float best = FLT_MAX;
    uint32_t bi = 0xFFFFFFFFu;
    for (uint32_t j = lane; j < count; j += 32u) {
        if (j == X) continue;
        float hx, hy, hz, lx, ly, lz;
        if (metric == 0) {
            // the reference's corners: "max" = max(A.min, B.min), "min" = max(A.max, B.max)
            hx = gmax(ax0, L.bmn[3 * j]); hy = gmax(ax1, L.bmn[3 * j + 1]); hz = gmax(ax2, L.bmn[3 * j + 2]);
            lx = gmax(bx0, L.bmx[3 * j]); ly = gmax(bx1, L.bmx[3 * j + 1]); lz = gmax(bx2, L.bmx[3 * j + 2]);
        } else {
            // the merged box
            lx = gmin(ax0, L.bmn[3 * j]); ly = gmin(ax1, L.bmn[3 * j + 1]); lz = gmin(ax2, L.bmn[3 * j + 2]);
            hx = gmax(bx0, L.bmx[3 * j]); hy = gmax(bx1, L.bmx[3 * j + 1]); hz = gmax(bx2, L.bmx[3 * j + 2]);
        }
        float ex = hx - lx, ey = hy - ly, ez = hz - lz;
        float area = ex * ey + ey * ez + ez * ex;
        if (area < best) { best = area; bi = j; }
    }
    for (int off = 16; off > 0; off >>= 1) {
        float ob = __shfl_down_sync(0xffffffffu, best, off);
        uint32_t oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    return __shfl_sync(0xffffffffu, bi, 0);
}

__device__ __forceinline__ void store_node(float4* nodes, uint32_t k, const float* mn, uint32_t lr, const float* mx,
                                           uint32_t inst) {
    nodes[2 * k] = make_float4(mn[0], mn[1], mn[2], __uint_as_float(lr));
    nodes[2 * k + 1] = make_float4(mx[0], mx[1], mx[2], __uint_as_float(inst));
}

// The reference's A/B/C walk (tlas_builder.cpp:18-67) for one warp.  aabbs:
// 6 floats per instance (min xyz, max xyz); nodes: 2n nodes; base: the
// working list, 7 words per instance (node index, box min, box max), in
// shared memory, a scratch buffer or the allocation-free build's static array.
__device__ __forceinline__ void tlas_walk(const float* __restrict__ aabbs, uint32_t n, float4* nodes, uint32_t* base,
                                          uint32_t metric) {
    List L;
    L.idx = base;
    L.bmn = reinterpret_cast<float*>(base + n);
    L.bmx = reinterpret_cast<float*>(base + 4 * n);
    const uint32_t lane = threadIdx.x;
    for (uint32_t i = lane; i < n; i += 32u) {
        float mn[3] = {aabbs[6 * i], aabbs[6 * i + 1], aabbs[6 * i + 2]};
        float mx[3] = {aabbs[6 * i + 3], aabbs[6 * i + 4], aabbs[6 * i + 5]};
        store_node(nodes, 1 + i, mn, 0u, mx, i);
        L.idx[i] = 1 + i;
        for (int a = 0; a < 3; ++a) { L.bmn[3 * i + a] = mn[a]; L.bmx[3 * i + a] = mx[a]; }
    }
    __syncwarp();
    uint32_t remaining = n, at = n + 1;
    uint32_t A = 0;
    uint32_t B = best_match(L, A, remaining, metric);
    while (remaining > 1) {
        const uint32_t C = best_match(L, B, remaining, metric);
        if (A == C) {
            if (lane == 0) {
                const uint32_t ia = L.idx[A], ib = L.idx[B];
                float mn[3], mx[3];
                for (int a = 0; a < 3; ++a) {
                    mn[a] = gmin(L.bmn[3 * A + a], L.bmn[3 * B + a]);
                    mx[a] = gmax(L.bmx[3 * A + a], L.bmx[3 * B + a]);
                }
                store_node(nodes, at, mn, ia + (ib << 16), mx, 0u);
                L.idx[A] = at;
                for (int a = 0; a < 3; ++a) { L.bmn[3 * A + a] = mn[a]; L.bmx[3 * A + a] = mx[a]; }
                const uint32_t last = remaining - 1;
                L.idx[B] = L.idx[last];
                for (int a = 0; a < 3; ++a) { L.bmn[3 * B + a] = L.bmn[3 * last + a]; L.bmx[3 * B + a] = L.bmx[3 * last + a]; }
            }
            __syncwarp();
            at++;
            remaining--;
            B = best_match(L, A, remaining, metric);
        } else {
            A = B;
            B = C;
        }
    }
    __syncwarp();
    if (lane == 0) {
        const uint32_t r = L.idx[A];
        const float4 a = nodes[2 * r], b = nodes[2 * r + 1];
        nodes[0] = a;
        nodes[1] = b;
    }
}

// One warp; the list in shared memory when it fits, else in gscratch.
__global__ void __launch_bounds__(32) k_tlas_build(const float* __restrict__ aabbs, uint32_t n, float4* nodes,
                                                   uint32_t* gscratch, uint32_t metric) {
    extern __shared__ uint32_t smem[];
    tlas_walk(aabbs, n, nodes, (n <= kSmemInstances) ? smem : gscratch, metric);
}

}  // namespace

// ---------------------------------------------------------------------------
// metric 2: parallel locally-ordered clustering (Meister and Bittner 2018).
// One block of 1024 threads, its working set in shared memory up to 2048
// instances: Morton order of the box centres by a bitonic sort,
// then rounds of nearest-neighbour search within kPlocRadius list positions
// (smallest merged half area, ties to the lower position), merging of mutual
// pairs (new nodes numbered in list order by a block scan) and in-order
// compaction.  Identical, node for node, to the oracle's tlas_ploc.
namespace {

constexpr uint32_t kPlocThreads = 1024;
// Neighbour window in list positions: on the 1,025-instance scene radius 2
// gives the cheapest tree (30.3 TLAS node loads per extension ray and 55.1
// per shadow ray against 33.0 / 59.2 at 16; radii 1-4 within 0.3 %, 8 / 16 /
// 32 / 64 worse) and the fastest build.
#ifndef WF_PLOC_RADIUS
#define WF_PLOC_RADIUS 2
#endif
constexpr uint32_t kPlocRadius = WF_PLOC_RADIUS;

__device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t code = 0;
    for (int b = 0; b < 10; ++b) {
        code |= ((x >> b) & 1u) << (3 * b + 2);
        code |= ((y >> b) & 1u) << (3 * b + 1);
        code |= ((z >> b) & 1u) << (3 * b);
    }
    return code;
}
__device__ __forceinline__ uint32_t quantize10(float c, float lo, float ext) {
    float q = (ext > 0.0f) ? (c - lo) / ext : 0.0f;
    if (!(q >= 0.0f)) q = 0.0f;
    if (q > 1.0f) q = 1.0f;
    return (uint32_t)(q * 1023.0f);
}

// The build's working arrays: in dynamic shared memory when they fit
// (n <= kPlocSmemMax), else in the caller's global scratch, same layout.
struct PlocScratch {
    unsigned long long* key;   // P (power of two >= n)
    uint32_t* cl[2];           // node id per list position
    uint32_t* nn;              // nearest neighbour per position
    uint32_t* flag;            // per position: 1 = creates a node
    uint32_t* keep;            // per position: 1 = stays in the list
    float* box[2];             // per position: the cluster's box (min xyz, max xyz)
};

constexpr uint32_t kPlocSmemMax = 2048;

__host__ __device__ inline size_t ploc_bytes(uint32_t n, uint32_t P) {
    return 8ull * P + 4ull * 5 * n + 4ull * 12 * n;
}

__device__ inline PlocScratch ploc_carve(void* base, uint32_t n, uint32_t P) {
    PlocScratch S;
    S.key = static_cast<unsigned long long*>(base);
    uint32_t* w = reinterpret_cast<uint32_t*>(S.key + P);
    S.cl[0] = w;
    S.cl[1] = w + n;
    S.nn = w + 2 * n;
    S.flag = w + 3 * n;
    S.keep = w + 4 * n;
    S.box[0] = reinterpret_cast<float*>(w + 5 * n);
    S.box[1] = S.box[0] + 6 * n;
    return S;
}

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t x) {
    const uint32_t lane = threadIdx.x & 31u;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, x, off);
        if ((int)lane >= off) x += o;
    }
    return x;
}

// Exclusive scan of v[0, count) in place by the whole block (each thread a
// contiguous chunk); returns the total.  s_wt: 33 words of shared memory.
__device__ uint32_t block_scan(uint32_t* v, uint32_t count, uint32_t* s_wt) {
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint32_t per = (count + kPlocThreads - 1) / kPlocThreads;
    const uint32_t b = t * per, e = min(count, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += v[i];
    const uint32_t incl = warp_inclusive_scan(sum);
    if (lane == 31u) s_wt[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t y = s_wt[lane];
        const uint32_t iw = warp_inclusive_scan(y);
        s_wt[lane] = iw - y;
        if (lane == 31u) s_wt[32] = iw;
    }
    __syncthreads();
    uint32_t run = (incl - sum) + s_wt[warp];
    for (uint32_t i = b; i < e; ++i) { const uint32_t x = v[i]; v[i] = run; run += x; }
    const uint32_t total = s_wt[32];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(kPlocThreads) k_tlas_ploc(const float* __restrict__ aabbs, uint32_t n,
                                                            float4* nodes, uint32_t* scratch, uint32_t P,
                                                            bool smem) {
    extern __shared__ unsigned long long s_dyn[];
    __shared__ uint32_t s_part[33];
    __shared__ float s_red[6][32];
    const PlocScratch S = ploc_carve(smem ? static_cast<void*>(s_dyn) : static_cast<void*>(scratch), n, P);
    const uint32_t t = threadIdx.x;
    // leaves and the centre bounds
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = t; i < n; i += kPlocThreads) {
        const float* b = aabbs + 6ull * i;
        nodes[2 * (1 + i)] = make_float4(b[0], b[1], b[2], __uint_as_float(0u));
        nodes[2 * (1 + i) + 1] = make_float4(b[3], b[4], b[5], __uint_as_float(i));
        for (int a = 0; a < 3; ++a) {
            const float c = (b[a] + b[3 + a]) * 0.5f;
            lo[a] = gmin(lo[a], c);
            hi[a] = gmax(hi[a], c);
        }
    }
    // gmin / gmax are order-insensitive for the finite centres here: the
    // result is the smallest / largest value, whichever order combines them
    for (int a = 0; a < 3; ++a)
        for (int off = 16; off > 0; off >>= 1) {
            lo[a] = gmin(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
            hi[a] = gmax(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
        }
    if ((t & 31u) == 0)
        for (int a = 0; a < 3; ++a) { s_red[a][t >> 5] = lo[a]; s_red[3 + a][t >> 5] = hi[a]; }
    __syncthreads();
    for (int a = 0; a < 3; ++a) {
        lo[a] = s_red[a][0];
        hi[a] = s_red[3 + a][0];
        for (int w = 1; w < 32; ++w) { lo[a] = gmin(lo[a], s_red[a][w]); hi[a] = gmax(hi[a], s_red[3 + a][w]); }
    }
    const float ext0 = hi[0] - lo[0], ext1 = hi[1] - lo[1], ext2 = hi[2] - lo[2];
    for (uint32_t i = t; i < P; i += kPlocThreads) {
        if (i < n) {
            const float* b = aabbs + 6ull * i;
            const uint32_t code = morton3(quantize10((b[0] + b[3]) * 0.5f, lo[0], ext0),
                                          quantize10((b[1] + b[4]) * 0.5f, lo[1], ext1),
                                          quantize10((b[2] + b[5]) * 0.5f, lo[2], ext2));
            S.key[i] = ((unsigned long long)code << 32) | i;
        } else {
            S.key[i] = ~0ull;
        }
    }
    __syncthreads();
    // bitonic sort of the P keys, ascending
    for (uint32_t size = 2; size <= P; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = t; i < P; i += kPlocThreads) {
                const uint32_t j = i ^ stride;
                if (j > i) {
                    const unsigned long long x = S.key[i], y = S.key[j];
                    const bool up = (i & size) == 0;
                    if (up ? (x > y) : (x < y)) { S.key[i] = y; S.key[j] = x; }
                }
            }
            __syncthreads();
        }
    for (uint32_t k = t; k < n; k += kPlocThreads) {
        const uint32_t leaf = (uint32_t)(S.key[k] & 0xFFFFFFFFull);
        S.cl[0][k] = 1u + leaf;
        for (int a = 0; a < 6; ++a) S.box[0][6 * k + a] = aabbs[6ull * leaf + a];
    }
    __syncthreads();
    uint32_t count = n, next = n + 1, cur = 0;
    while (count > 1) {
        const uint32_t* cl = S.cl[cur];
        uint32_t* ncl = S.cl[cur ^ 1];
        const float* bx = S.box[cur];
        float* nbx = S.box[cur ^ 1];
        for (uint32_t k = t; k < count; k += kPlocThreads) {
            const float* A = bx + 6 * k;
            const float anx = A[0], any_ = A[1], anz = A[2], axx = A[3], axy = A[4], axz = A[5];
            const uint32_t j0 = k > kPlocRadius ? k - kPlocRadius : 0u;
            const uint32_t j1 = k + kPlocRadius < count - 1 ? k + kPlocRadius : count - 1;
            float best = FLT_MAX;
            uint32_t bj = (k == 0) ? 1u : k - 1;
            for (uint32_t j = j0; j <= j1; ++j) {
                if (j == k) continue;
                const float* Bj = bx + 6 * j;
                const float ex = gmax(axx, Bj[3]) - gmin(anx, Bj[0]);
                const float ey = gmax(axy, Bj[4]) - gmin(any_, Bj[1]);
                const float ez = gmax(axz, Bj[5]) - gmin(anz, Bj[2]);
                const float d = ex * ey + ey * ez + ez * ex;
                if (d < best) { best = d; bj = j; }
            }
            S.nn[k] = bj;
        }
        __syncthreads();
        // a round without a mutual pair (not seen in practice) merges positions 0 and 1
        for (uint32_t k = t; k < count; k += kPlocThreads) S.flag[k] = (S.nn[S.nn[k]] == k && k < S.nn[k]) ? 1u : 0u;
        __syncthreads();
        uint32_t any = 0;
        for (uint32_t k = t; k < count; k += kPlocThreads) any |= S.flag[k];
        any = __syncthreads_or(any);
        if (!any) {
            if (t == 0) { S.nn[0] = 1; S.nn[1] = 0; }
            __syncthreads();
        }
        for (uint32_t k = t; k < count; k += kPlocThreads) {
            const uint32_t m = S.nn[k];
            const bool mutual = S.nn[m] == k;
            S.flag[k] = (mutual && k < m) ? 1u : 0u;
            S.keep[k] = (mutual && k > m) ? 0u : 1u;
        }
        __syncthreads();
        const uint32_t made = block_scan(S.flag, count, s_part);
        const uint32_t kept = block_scan(S.keep, count, s_part);
        for (uint32_t k = t; k < count; k += kPlocThreads) {
            const uint32_t m = S.nn[k];
            const bool mutual = S.nn[m] == k;
            if (mutual && k > m) continue;
            const uint32_t pos = S.keep[k];
            const float* A = bx + 6 * k;
            float* O = nbx + 6 * pos;
            if (mutual) {
                const uint32_t id = next + S.flag[k];
                const float* Bm = bx + 6 * m;
                const float mn[3] = {gmin(A[0], Bm[0]), gmin(A[1], Bm[1]), gmin(A[2], Bm[2])};
                const float mx[3] = {gmax(A[3], Bm[3]), gmax(A[4], Bm[4]), gmax(A[5], Bm[5])};
                nodes[2 * id] = make_float4(mn[0], mn[1], mn[2], __uint_as_float((cl[k] << 16) | cl[m]));
                nodes[2 * id + 1] = make_float4(mx[0], mx[1], mx[2], __uint_as_float(0u));
                ncl[pos] = id;
                for (int a = 0; a < 3; ++a) { O[a] = mn[a]; O[3 + a] = mx[a]; }
            } else {
                ncl[pos] = cl[k];
                for (int a = 0; a < 6; ++a) O[a] = A[a];
            }
        }
        __syncthreads();
        count = kept;
        next += made;
        cur ^= 1;
    }
    if (t == 0 && n > 0) {
        const uint32_t r = S.cl[cur][0];
        nodes[0] = nodes[2 * r];
        nodes[1] = nodes[2 * r + 1];
    }
}

// ---------------------------------------------------------------------------
// metric 3: top-down full-sweep SAH, one block of 1024 threads.  Three lists
// of the instances by box centre along x, y, z (one bitonic network over the
// three axes' (sortable centre bits, index) keys, its strides below 32 in
// warp shuffles); then level by level: on a level of at most two ranges the
// whole block sweeps each range in turn (sweep_block), else a range [s, e)
// of 3 to 10 instances goes to one warp (sweep_warp_small) and a larger one
// to a team of three warps, one
// per axis (warp scans of the prefix union boxes, their half areas kept per
// position, then of the suffix boxes, each boundary's cost A(left) * |left|
// + A(right) * |right| in float), which takes the cheapest boundary (ties to
// the lower axis, then the lower position), partitions the other two lists
// stably and queues the two halves for the next level; a range of 2 goes to
// one thread, which builds its whole subtree the same way.  The interior node of a range split after position k is node
// n + 1 + k (every boundary is split once), so node numbers do not depend on
// which warp takes which range; a child sets its half of the parent's
// left_right word.  Identical, node for node, to the oracle's tlas_sweep.
__device__ __forceinline__ uint32_t sortable_bits(float x) {
    const uint32_t u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

constexpr uint32_t kSweepSmemMax = 2048;

// Boxes live as sortable bits (an unsigned order equal to float order, -0
// below +0), so a union is an integer min / max: order-independent, and one
// instruction.  A box: min x, y, z then max x, y, z.
__device__ __forceinline__ float from_sortable(uint32_t s) {
    return __uint_as_float((s & 0x80000000u) ? (s & 0x7FFFFFFFu) : ~s);
}
__device__ __forceinline__ float half_area_sb(const uint32_t* b) {
    const float ex = from_sortable(b[3]) - from_sortable(b[0]);
    const float ey = from_sortable(b[4]) - from_sortable(b[1]);
    const float ez = from_sortable(b[5]) - from_sortable(b[2]);
    return ex * ey + ey * ez + ez * ex;
}

struct SweepScratch {
    uint32_t* list[3];    // n each
    uint32_t* tmp;        // n
    uint32_t* left;       // n: 1 = the instance is in its range's left part
    float* area[3];       // per axis and position: the half area of the prefix union box
    float* sarea[3];      // per axis and position: the half area of the suffix union box (block mode)
    unsigned long long* key;   // 3 P sort keys (the same words as area and sarea, before the sweep)
    uint32_t* box;        // 6 per instance
    uint32_t* task[2];    // per level: (s | e << 16, parent | slot << 16), n / 2 + 1 each
};

__host__ __device__ inline size_t sweep_words(uint32_t n, uint32_t P) {
    return 6ull * P + 3ull * n + n + n + 6ull * n + 2ull * 2 * (n / 2 + 1);
}

__device__ inline SweepScratch sweep_carve(uint32_t* base, uint32_t n, uint32_t P) {
    SweepScratch S;
    S.key = reinterpret_cast<unsigned long long*>(base);   // first: 8-byte aligned
    for (int a = 0; a < 3; ++a) {
        S.area[a] = reinterpret_cast<float*>(base) + (size_t)a * n;
        S.sarea[a] = reinterpret_cast<float*>(base) + (size_t)(3 + a) * n;   // 6 n <= 6 P words
    }
    uint32_t* w = base + 6ull * P;
    S.list[0] = w; S.list[1] = w + n; S.list[2] = w + 2 * n;
    S.tmp = w + 3 * n;
    S.left = w + 4 * n;
    S.box = w + 5 * n;
    S.task[0] = w + 11 * n;
    S.task[1] = S.task[0] + 2 * (n / 2 + 1);
    return S;
}

struct Split {
    float cost;
    uint32_t ax, k;
};
__device__ __forceinline__ bool better(const Split& a, const Split& b) {
    return a.cost < b.cost || (a.cost == b.cost && (a.ax < b.ax || (a.ax == b.ax && a.k < b.k)));
}

// the identity of a box union: min fields at the top of the order, max at the bottom
constexpr uint32_t kSbEmptyMin = 0xFFFFFFFFu, kSbEmptyMax = 0u;

// Stable partition of list ax over [s, e) by S.left (nleft left instances), by one thread.
__device__ void partition_serial(const SweepScratch& S, uint32_t s, uint32_t e, uint32_t ax) {
    uint32_t* L = S.list[ax];
    uint32_t p = s;
    for (uint32_t i = s; i < e; ++i) if (S.left[L[i]]) S.tmp[p++] = L[i];
    for (uint32_t i = s; i < e; ++i) if (!S.left[L[i]]) S.tmp[p++] = L[i];
    for (uint32_t i = s; i < e; ++i) L[i] = S.tmp[i];
}

// One thread: the split of range [s, e) (e - s >= 2) by a sequential sweep,
// the same candidates as the warps' sweeps; the lists left partitioned, the
// range's box in rb.
__device__ uint32_t sweep_serial(const SweepScratch& S, uint32_t s, uint32_t e, uint32_t* rb) {
    Split best{FLT_MAX, 3u, 0u};
    for (uint32_t ax = 0; ax < 3; ++ax) {
        const uint32_t* L = S.list[ax];
        float* A = S.area[ax];
        uint32_t c[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
        for (uint32_t i = s; i < e; ++i) {
            const uint32_t* b = S.box + 6ull * L[i];
            for (int a = 0; a < 3; ++a) { c[a] = min(c[a], b[a]); c[3 + a] = max(c[3 + a], b[3 + a]); }
            A[i] = half_area_sb(c);
        }
        if (ax == 0)
            for (int a = 0; a < 6; ++a) rb[a] = c[a];
        uint32_t q[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
        for (uint32_t i = e - 1; i > s; --i) {
            const uint32_t* b = S.box + 6ull * L[i];
            for (int a = 0; a < 3; ++a) { q[a] = min(q[a], b[a]); q[3 + a] = max(q[3 + a], b[3 + a]); }
            const uint32_t k = i - 1;
            const float cost = A[k] * (float)(k - s + 1) + half_area_sb(q) * (float)(e - 1 - k);
            const Split cand{cost, ax, k};
            if (cost < FLT_MAX && better(cand, best)) best = cand;
        }
    }
    uint32_t bax = best.ax, bk = best.k;
    if (bax == 3u) { bax = 0u; bk = s; }   // no cost below FLT_MAX (not for finite boxes)
    for (uint32_t i = s; i < e; ++i) S.left[S.list[bax][i]] = i <= bk ? 1u : 0u;
    for (uint32_t ax = 0; ax < 3; ++ax)
        if (ax != bax) partition_serial(S, s, e, ax);
    return bk;
}

__device__ __forceinline__ void store_sweep_node(float4* nodes, uint32_t id, const uint32_t* rb) {
    nodes[2 * id] = make_float4(from_sortable(rb[0]), from_sortable(rb[1]), from_sortable(rb[2]), __uint_as_float(0u));
    nodes[2 * id + 1] = make_float4(from_sortable(rb[3]), from_sortable(rb[4]), from_sortable(rb[5]), __uint_as_float(0u));
}
__device__ __forceinline__ void link_child(float4* nodes, uint32_t parent, uint32_t slot, uint32_t id) {
    atomicOr(reinterpret_cast<uint32_t*>(nodes + 2 * parent) + 3, slot == 0u ? (id << 16) : id);
}

// One thread builds the whole subtree of a small range [s, e) (2 <= e - s
// <= kSweepSerial) below parent / slot, depth-first.
#ifndef WF_SWEEP_SERIAL
#define WF_SWEEP_SERIAL 2
#endif
constexpr uint32_t kSweepSerial = WF_SWEEP_SERIAL;
__device__ void sweep_subtree(const SweepScratch& S, float4* nodes, uint32_t n, uint32_t s0, uint32_t e0,
                              uint32_t parent0, uint32_t slot0, uint32_t* root) {
    uint32_t st[3 * kSweepSerial];
    uint32_t top = 0;
    st[0] = s0 | (e0 << 16); st[1] = parent0; st[2] = slot0;
    top = 1;
    while (top) {
        --top;
        const uint32_t s = st[3 * top] & 0xFFFFu, e = st[3 * top] >> 16, parent = st[3 * top + 1], slot = st[3 * top + 2];
        uint32_t id;
        if (e - s == 1) {
            id = 1 + S.list[0][s];
        } else {
            uint32_t rb[6];
            const uint32_t k = sweep_serial(S, s, e, rb);
            id = n + 1 + k;
            store_sweep_node(nodes, id, rb);
            st[3 * top] = (k + 1) | (e << 16); st[3 * top + 1] = id; st[3 * top + 2] = 1u;
            ++top;
            st[3 * top] = s | ((k + 1) << 16); st[3 * top + 1] = id; st[3 * top + 2] = 0u;
            ++top;
        }
        if (slot == 2u) *root = id;
        else link_child(nodes, parent, slot, id);
    }
}

// Inclusive warp scan of a sortable box (min fields by min, max fields by max).
__device__ __forceinline__ void warp_scan_box(uint32_t* v, uint32_t lane) {
    for (int off = 1; off < 32; off <<= 1)
        for (int a = 0; a < 6; ++a) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, v[a], off);
            if ((int)lane >= off) v[a] = a < 3 ? min(o, v[a]) : max(o, v[a]);
        }
}

// One warp, one axis of range [s, e) (e - s >= 2): the prefix areas, then
// the cheapest boundary along the axis (ties to the lower position); the
// range's box in rb (every lane).
__device__ Split sweep_axis(const SweepScratch& S, uint32_t ax, uint32_t s, uint32_t e, uint32_t* rb) {
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned FULL = 0xffffffffu;
    const uint32_t* L = S.list[ax];
    float* A = S.area[ax];
    Split best{FLT_MAX, 3u, 0u};
    uint32_t cb[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
    for (uint32_t c = s; c < e; c += 32) {
        const uint32_t i = c + lane;
        uint32_t v[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
        if (i < e) {
            const uint32_t* b = S.box + 6ull * L[i];
            for (int a = 0; a < 6; ++a) v[a] = b[a];
        }
        warp_scan_box(v, lane);
        for (int a = 0; a < 6; ++a) v[a] = a < 3 ? min(cb[a], v[a]) : max(cb[a], v[a]);
        if (i < e) A[i] = half_area_sb(v);
        const uint32_t last = min(31u, e - 1 - c);
        for (int a = 0; a < 6; ++a) cb[a] = __shfl_sync(FULL, v[a], last);
    }
    for (int a = 0; a < 6; ++a) rb[a] = cb[a];
    __syncwarp();
    // suffix boxes from the end; position i's suffix pairs with the prefix at i - 1
    for (int a = 0; a < 6; ++a) cb[a] = a < 3 ? kSbEmptyMin : kSbEmptyMax;
    for (uint32_t c = 0; c < e - s; c += 32) {
        const uint32_t j = c + lane;   // j-th position from the end
        const bool valid = j < e - s;
        const uint32_t i = e - 1 - j;
        uint32_t v[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
        if (valid) {
            const uint32_t* b = S.box + 6ull * L[i];
            for (int a = 0; a < 6; ++a) v[a] = b[a];
        }
        warp_scan_box(v, lane);
        for (int a = 0; a < 6; ++a) v[a] = a < 3 ? min(cb[a], v[a]) : max(cb[a], v[a]);
        if (valid && i > s) {
            const uint32_t k = i - 1;
            const float cost = A[k] * (float)(k - s + 1) + half_area_sb(v) * (float)(e - 1 - k);
            const Split cand{cost, ax, k};
            if (cost < FLT_MAX && better(cand, best)) best = cand;
        }
        const uint32_t last = min(31u, e - s - 1 - c);
        for (int a = 0; a < 6; ++a) cb[a] = __shfl_sync(FULL, v[a], last);
    }
    for (int off = 16; off > 0; off >>= 1) {
        const Split o{__shfl_xor_sync(FULL, best.cost, off), __shfl_xor_sync(FULL, best.ax, off),
                      __shfl_xor_sync(FULL, best.k, off)};
        if (better(o, best)) best = o;
    }
    return best;
}

// One warp: stable partition of list ax over [s, e) by S.left (nleft left
// instances), through the axis's own prefix-area words (free once the split
// is chosen; the two lists of a range are partitioned at the same time).
__device__ void partition_warp(const SweepScratch& S, uint32_t ax, uint32_t s, uint32_t e, uint32_t nleft) {
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned FULL = 0xffffffffu;
    uint32_t* L = S.list[ax];
    uint32_t* T = reinterpret_cast<uint32_t*>(S.area[ax]);
    uint32_t nl = 0, nr = 0;
    for (uint32_t c = s; c < e; c += 32) {
        const uint32_t i = c + lane;
        const bool valid = i < e;
        const uint32_t id = valid ? L[i] : 0u;
        const bool isl = valid && S.left[id] != 0u;
        const unsigned ml = __ballot_sync(FULL, isl), mr = __ballot_sync(FULL, valid && !isl);
        const unsigned below = (1u << lane) - 1u;
        if (isl) T[s + nl + __popc(ml & below)] = id;
        else if (valid) T[s + nleft + nr + __popc(mr & below)] = id;
        nl += __popc(ml);
        nr += __popc(mr);
    }
    __syncwarp();
    for (uint32_t i = s + lane; i < e; i += 32) L[i] = T[i];
    __syncwarp();
}

__device__ __forceinline__ void team_sync(uint32_t team) {
    asm volatile("bar.sync %0, %1;" ::"r"(team + 1u), "r"(96) : "memory");
}

// Block mode, for the top levels where a few large ranges would leave most
// teams idle: the whole block on one range [s, e) (e - s > kSweepSerial), ten
// warps per axis, each on a contiguous chunk of the range.  Chunk union boxes
// first; then each warp scans its chunk starting from the union of the chunks
// before it (prefix areas) and after it (suffix areas); then every boundary's
// cost, the cheapest over the block, and a stable partition of the other two
// lists from per-chunk left counts.  Unions of sortable bits do not depend on
// grouping, so the areas, the costs (the same float expression) and the split
// equal the team's.  Called by every thread; returns k, the range's box in rb.
constexpr uint32_t kAxisWarps = kPlocThreads / 96;   // 10: warps 30 and 31 only keep the barriers
#ifndef WF_SWEEP_BLOCK_TASKS
#define WF_SWEEP_BLOCK_TASKS 2
#endif
constexpr uint32_t kSweepBlockTasks = WF_SWEEP_BLOCK_TASKS;   // block mode on levels of at most this many ranges

struct SweepBlockShared {
    uint32_t tot[3][kAxisWarps][6];   // per axis and chunk: the chunk's union box
    Split best[3 * kAxisWarps];       // per warp: its chunk's cheapest boundary
    uint32_t cnt[3][kAxisWarps];      // per axis and chunk: instances in the left part
};

__device__ __forceinline__ void box_union(uint32_t* d, const uint32_t* b) {
    for (int a = 0; a < 3; ++a) { d[a] = min(d[a], b[a]); d[3 + a] = max(d[3 + a], b[3 + a]); }
}

__device__ uint32_t sweep_block(const SweepScratch& S, SweepBlockShared& B, uint32_t s, uint32_t e, uint32_t* rb) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned FULL = 0xffffffffu;
    const bool active = warp < 3 * kAxisWarps;
    const uint32_t ax = active ? warp / kAxisWarps : 0u, ch = warp % kAxisWarps;
    const uint32_t clen = (e - s + kAxisWarps - 1) / kAxisWarps;
    const uint32_t c0 = min(e, s + ch * clen), c1 = min(e, c0 + clen);   // this warp's chunk [c0, c1)
    const uint32_t* L = S.list[ax];
    if (active) {
        uint32_t v[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
        for (uint32_t i = c0 + lane; i < c1; i += 32) box_union(v, S.box + 6ull * L[i]);
        for (int off = 16; off > 0; off >>= 1)
            for (int a = 0; a < 6; ++a) {
                const uint32_t o = __shfl_xor_sync(FULL, v[a], off);
                v[a] = a < 3 ? min(o, v[a]) : max(o, v[a]);
            }
        if (lane == 0)
            for (int a = 0; a < 6; ++a) B.tot[ax][ch][a] = v[a];
    }
    __syncthreads();
    if (active) {
        uint32_t pre[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
        uint32_t post[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
        for (uint32_t c = 0; c < kAxisWarps; ++c) {
            if (c < ch) box_union(pre, B.tot[ax][c]);
            if (c > ch) box_union(post, B.tot[ax][c]);
        }
        uint32_t cb[6];
        for (int a = 0; a < 6; ++a) cb[a] = pre[a];
        for (uint32_t c = c0; c < c1; c += 32) {
            const uint32_t i = c + lane;
            uint32_t v[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
            if (i < c1) {
                const uint32_t* b = S.box + 6ull * L[i];
                for (int a = 0; a < 6; ++a) v[a] = b[a];
            }
            warp_scan_box(v, lane);
            box_union(v, cb);
            if (i < c1) S.area[ax][i] = half_area_sb(v);
            const uint32_t last = min(31u, c1 - 1 - c);
            for (int a = 0; a < 6; ++a) cb[a] = __shfl_sync(FULL, v[a], last);
        }
        for (int a = 0; a < 6; ++a) cb[a] = post[a];
        for (uint32_t c = 0; c < c1 - c0; c += 32) {
            const uint32_t j = c + lane;   // j-th position from the chunk's end
            const bool valid = j < c1 - c0;
            const uint32_t i = c1 - 1 - j;
            uint32_t v[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
            if (valid) {
                const uint32_t* b = S.box + 6ull * L[i];
                for (int a = 0; a < 6; ++a) v[a] = b[a];
            }
            warp_scan_box(v, lane);
            box_union(v, cb);
            if (valid) S.sarea[ax][i] = half_area_sb(v);
            const uint32_t last = min(31u, c1 - c0 - 1 - c);
            for (int a = 0; a < 6; ++a) cb[a] = __shfl_sync(FULL, v[a], last);
        }
    }
    __syncthreads();
    if (active) {
        // boundary k (after position k) pairs the prefix at k with the suffix at k + 1
        Split best{FLT_MAX, 3u, 0u};
        for (uint32_t k = c0 + lane; k < c1; k += 32) {
            if (k + 1 >= e) continue;
            const float cost = S.area[ax][k] * (float)(k - s + 1) + S.sarea[ax][k + 1] * (float)(e - 1 - k);
            const Split cand{cost, ax, k};
            if (cost < FLT_MAX && better(cand, best)) best = cand;
        }
        for (int off = 16; off > 0; off >>= 1) {
            const Split o{__shfl_xor_sync(FULL, best.cost, off), __shfl_xor_sync(FULL, best.ax, off),
                          __shfl_xor_sync(FULL, best.k, off)};
            if (better(o, best)) best = o;
        }
        if (lane == 0) B.best[warp] = best;
    }
    __syncthreads();
    // every candidate's cost is below FLT_MAX, so better() orders them totally
    // and the reduction's order does not matter
    Split best = B.best[0];
    for (uint32_t w = 1; w < 3 * kAxisWarps; ++w)
        if (better(B.best[w], best)) best = B.best[w];
    uint32_t bax = best.ax, k = best.k;
    if (bax == 3u) { bax = 0u; k = s; }   // no cost below FLT_MAX (not for finite boxes)
    for (int a = 0; a < 6; ++a) rb[a] = a < 3 ? kSbEmptyMin : kSbEmptyMax;
    for (uint32_t c = 0; c < kAxisWarps; ++c) box_union(rb, B.tot[0][c]);
    if (active && ax == bax)
        for (uint32_t i = c0 + lane; i < c1; i += 32) S.left[L[i]] = i <= k ? 1u : 0u;
    __syncthreads();
    const bool part = active && ax != bax;
    if (part) {
        uint32_t nl = 0;
        for (uint32_t c = c0; c < c1; c += 32) {
            const uint32_t i = c + lane;
            nl += __popc(__ballot_sync(FULL, i < c1 && S.left[L[i]] != 0u));
        }
        if (lane == 0) B.cnt[ax][ch] = nl;
    }
    __syncthreads();
    // the stable partition goes through the axis's prefix-area words (free now)
    uint32_t* T = reinterpret_cast<uint32_t*>(S.area[ax]);
    if (part) {
        uint32_t nl = 0;
        for (uint32_t c = 0; c < ch; ++c) nl += B.cnt[ax][c];
        uint32_t nr = (c0 - s) - nl;
        const uint32_t nleft = k + 1 - s;
        for (uint32_t c = c0; c < c1; c += 32) {
            const uint32_t i = c + lane;
            const bool valid = i < c1;
            const uint32_t id = valid ? L[i] : 0u;
            const bool isl = valid && S.left[id] != 0u;
            const unsigned ml = __ballot_sync(FULL, isl), mr = __ballot_sync(FULL, valid && !isl);
            const unsigned below = (1u << lane) - 1u;
            if (isl) T[s + nl + __popc(ml & below)] = id;
            else if (valid) T[s + nleft + nr + __popc(mr & below)] = id;
            nl += __popc(ml);
            nr += __popc(mr);
        }
    }
    __syncthreads();
    if (part)
        for (uint32_t i = c0 + lane; i < c1; i += 32) S.list[ax][i] = T[i];
    __syncthreads();
    return k;
}

// Warp mode, for ranges of kSweepSerial + 1 to kSweepWarpMax instances: one
// warp, the three axes side by side in segments of kSeg lanes (lane a kSeg + j
// holds list a's position s + j in the prefix scan and e - 1 - j in the
// suffix scan); each boundary's cost from its own prefix area and a shuffled
// suffix area, the cheapest over the warp, a stable partition of the other
// two lists by ballots within their segments, and the node emitted.  The
// same areas, costs and split as the team's.
constexpr uint32_t kSeg = 10;
#ifndef WF_SWEEP_WARP_MAX
#define WF_SWEEP_WARP_MAX 10
#endif
constexpr uint32_t kSweepWarpMax = WF_SWEEP_WARP_MAX;
static_assert(kSweepWarpMax <= kSeg, "a warp-mode range fits one segment");

__device__ __forceinline__ void seg_scan_box(uint32_t* v, uint32_t j) {
    for (uint32_t off = 1; off < kSeg; off <<= 1)
        for (int a = 0; a < 6; ++a) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, v[a], off);
            if (j >= off) v[a] = a < 3 ? min(o, v[a]) : max(o, v[a]);
        }
}

__device__ void emit_split(const SweepScratch& S, float4* nodes, uint32_t n, uint32_t s, uint32_t e, uint32_t k,
                           uint32_t parent, uint32_t slot, const uint32_t* rb, uint32_t* next_count,
                           uint32_t* next_task, uint32_t* root);

__device__ void sweep_warp_small(const SweepScratch& S, float4* nodes, uint32_t n, uint32_t s, uint32_t e,
                                 uint32_t parent, uint32_t slot, uint32_t* next_count, uint32_t* next_task,
                                 uint32_t* root) {
    const unsigned FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t a = lane / kSeg, j = lane - a * kSeg, m = e - s;
    const bool in = a < 3u && j < m;
    const uint32_t id = in ? S.list[a][s + j] : 0u;
    uint32_t v[6] = {kSbEmptyMin, kSbEmptyMin, kSbEmptyMin, kSbEmptyMax, kSbEmptyMax, kSbEmptyMax};
    if (in)
        for (int c = 0; c < 6; ++c) v[c] = S.box[6ull * id + c];
    seg_scan_box(v, j);
    const float pa = half_area_sb(v);          // prefix area at s + j
    uint32_t rb[6];                            // the range's box: list 0's last prefix
    for (int c = 0; c < 6; ++c) rb[c] = __shfl_sync(FULL, v[c], m - 1);
    for (int c = 0; c < 6; ++c) v[c] = c < 3 ? kSbEmptyMin : kSbEmptyMax;
    if (in) {
        const uint32_t* b = S.box + 6ull * S.list[a][e - 1 - j];
        for (int c = 0; c < 6; ++c) v[c] = b[c];
    }
    seg_scan_box(v, j);
    const float sa = half_area_sb(v);          // suffix area at e - 1 - j
    // boundary k = s + j pairs the prefix at k with the suffix at k + 1,
    // held by lane a kSeg + (m - 2 - j)
    const bool cand_ok = in && j + 1 < m;
    const float sa1 = __shfl_sync(FULL, sa, cand_ok ? a * kSeg + (m - 2 - j) : lane);
    Split best{FLT_MAX, 3u, 0u};
    if (cand_ok) {
        const uint32_t k = s + j;
        const float cost = pa * (float)(k - s + 1) + sa1 * (float)(e - 1 - k);
        const Split cand{cost, a, k};
        if (cost < FLT_MAX && better(cand, best)) best = cand;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const Split o{__shfl_xor_sync(FULL, best.cost, off), __shfl_xor_sync(FULL, best.ax, off),
                      __shfl_xor_sync(FULL, best.k, off)};
        if (better(o, best)) best = o;
    }
    uint32_t bax = best.ax, k = best.k;
    if (bax == 3u) { bax = 0u; k = s; }   // no cost below FLT_MAX (not for finite boxes)
    if (in && a == bax) S.left[id] = (s + j <= k) ? 1u : 0u;
    __syncwarp();
    const bool part = in && a != bax;
    const bool isl = part && S.left[id] != 0u;
    const unsigned seg = a < 3u ? (((1u << m) - 1u) << (a * kSeg)) : 0u;
    const unsigned ml = __ballot_sync(FULL, isl) & seg, mr = __ballot_sync(FULL, part && !isl) & seg;
    const unsigned below = (1u << lane) - 1u;
    __syncwarp();
    if (part) S.list[a][isl ? s + __popc(ml & below) : s + (k + 1 - s) + __popc(mr & below)] = id;
    __syncwarp();
    if (lane == 0) emit_split(S, nodes, n, s, e, k, parent, slot, rb, next_count, next_task, root);
    __syncwarp();
}

// A compare-exchange of the bitonic network between lanes lane and lane ^ st
// of a warp holding keys i (this lane's position in its axis) for stage
// (size, st): an ascending pair (bit `size` of i clear) leaves the smaller key
// at the lower position.
__device__ __forceinline__ unsigned long long cx_lanes(unsigned long long x, uint32_t i, uint32_t size, uint32_t st,
                                                       uint32_t lane) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, st);
    const bool up = (i & size) == 0, low = (lane & st) == 0;
    return (low == up) ? min(x, y) : max(x, y);
}

// Every window of 32 consecutive keys (P >= 32, so a window lies within one
// axis's keys), one warp each: ALL = the stages of sizes 2-32, else the
// strides 16-1 of stage `size`.
template <bool ALL>
__device__ void sort_windows(unsigned long long* key, uint32_t P, uint32_t size) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t w = warp; w < 3 * (P >> 5); w += kPlocThreads / 32) {
        const uint32_t q = 32 * w + lane, i = q & (P - 1);
        unsigned long long x = key[q];
        if (ALL) {
#pragma unroll
            for (uint32_t sz = 2; sz <= 32; sz <<= 1)
#pragma unroll
                for (uint32_t st = sz >> 1; st > 0; st >>= 1) x = cx_lanes(x, i, sz, st, lane);
        } else {
#pragma unroll
            for (uint32_t st = 16; st > 0; st >>= 1) x = cx_lanes(x, i, size, st, lane);
        }
        key[q] = x;
    }
}

// One thread, once range [s, e) is split after k and its lists partitioned:
// the interior node n + 1 + k with the range's box, its single-instance
// halves linked as leaves, the node linked into its parent (slot 2: the
// root), and the larger halves queued for the next level.
__device__ void emit_split(const SweepScratch& S, float4* nodes, uint32_t n, uint32_t s, uint32_t e, uint32_t k,
                           uint32_t parent, uint32_t slot, const uint32_t* rb, uint32_t* next_count,
                           uint32_t* next_task, uint32_t* root) {
    const uint32_t id = n + 1 + k;
    store_sweep_node(nodes, id, rb);
    if (k == s) link_child(nodes, id, 0u, 1u + S.list[0][s]);
    if (k + 2 == e) link_child(nodes, id, 1u, 1u + S.list[0][e - 1]);
    if (slot == 2u) *root = id;
    else link_child(nodes, parent, slot, id);
    if (k > s) {
        const uint32_t p = atomicAdd(next_count, 1u);
        next_task[2 * p] = s | ((k + 1) << 16);
        next_task[2 * p + 1] = id | (0u << 16);
    }
    if (k + 2 < e) {
        const uint32_t p = atomicAdd(next_count, 1u);
        next_task[2 * p] = (k + 1) | (e << 16);
        next_task[2 * p + 1] = id | (1u << 16);
    }
}

__global__ void __launch_bounds__(kPlocThreads) k_tlas_sweep(const float* __restrict__ aabbs, uint32_t n,
                                                             float4* nodes, uint32_t* scratch, uint32_t P,
                                                             bool smem) {
    extern __shared__ unsigned long long s_dyn[];
    constexpr uint32_t kTeams = kPlocThreads / 96;   // three warps each
    __shared__ uint32_t s_count[2], s_root, s_next;
    __shared__ Split s_split[kTeams][3];
    __shared__ uint32_t s_box[kTeams][6];
    __shared__ SweepBlockShared s_blk;
    const SweepScratch S = sweep_carve(smem ? reinterpret_cast<uint32_t*>(s_dyn) : scratch, n, P);
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint32_t team = warp / 3u, axw = warp % 3u;
    for (uint32_t i = t; i < n; i += kPlocThreads) {
        const float* b = aabbs + 6ull * i;
        nodes[2 * (1 + i)] = make_float4(b[0], b[1], b[2], __uint_as_float(0u));
        nodes[2 * (1 + i) + 1] = make_float4(b[3], b[4], b[5], __uint_as_float(i));
        for (int a = 0; a < 6; ++a) S.box[6ull * i + a] = sortable_bits(b[a]);
    }
    // the three sorted lists, sorted together: keys of axis a at [a P, (a + 1) P)
    unsigned long long* key = S.key;
    const uint32_t lgP = 31u - __clz(P);
    for (uint32_t q = t; q < 3 * P; q += kPlocThreads) {
        const uint32_t ax = q >> lgP, i = q & (P - 1);
        if (i < n) {
            const float c = (aabbs[6ull * i + ax] + aabbs[6ull * i + 3 + ax]) * 0.5f;
            key[q] = ((unsigned long long)sortable_bits(c) << 32) | i;
        } else {
            key[q] = ~0ull;
        }
    }
    __syncthreads();
    // a bitonic network: strides of 32 and more as pairs in shared memory
    // between barriers; the strides below 32 (and sizes 2-32 whole) in warp
    // windows of 32 consecutive keys, through shuffles (P >= 32; a smaller P
    // takes every stride as pairs)
    const uint32_t G = P >= 32u ? 32u : 1u;
    if (G == 32u) {
        sort_windows<true>(key, P, 0u);
        __syncthreads();
    }
    for (uint32_t size = 2 * G; size <= P; size <<= 1) {
        for (uint32_t stride = size >> 1; stride >= G; stride >>= 1) {
            const uint32_t lgs = 31u - __clz(stride);
            for (uint32_t p = t; p < 3 * (P >> 1); p += kPlocThreads) {
                const uint32_t ax = p >> (lgP - 1), pi = p & ((P >> 1) - 1);
                const uint32_t i = ((pi >> lgs) << (lgs + 1)) | (pi & (stride - 1)), j = i | stride;
                const uint32_t o = ax << lgP;
                const unsigned long long x = key[o + i], y = key[o + j];
                const bool up = (i & size) == 0;
                if (up ? (x > y) : (x < y)) { key[o + i] = y; key[o + j] = x; }
            }
            __syncthreads();
        }
        if (G == 32u) {
            sort_windows<false>(key, P, size);
            __syncthreads();
        }
    }
    // (the keys' words become the prefix areas after the next barrier)
    for (uint32_t q = t; q < 3 * P; q += kPlocThreads) {
        const uint32_t ax = q >> lgP, i = q & (P - 1);
        if (i < n) S.list[ax][i] = (uint32_t)(key[q] & 0xFFFFFFFFull);
    }
    if (t == 0) {
        s_root = 1u;   // a single instance is its own root
        s_count[0] = n >= 2 ? 1u : 0u;
        s_next = 0u;
        s_count[1] = 0u;
        S.task[0][0] = 0u | (n << 16);
        S.task[0][1] = 0u | (2u << 16);   // slot 2: the root
    }
    __syncthreads();
    uint32_t cur = 0;
    while (s_count[cur] > 0) {
        const uint32_t ntask = s_count[cur];
        // small ranges: one thread builds each one's whole subtree
        for (uint32_t q = t; q < ntask; q += kPlocThreads) {
            const uint32_t r0 = S.task[cur][2 * q], r1 = S.task[cur][2 * q + 1];
            const uint32_t s = r0 & 0xFFFFu, e = r0 >> 16;
            if (e - s <= kSweepSerial) sweep_subtree(S, nodes, n, s, e, r1 & 0xFFFFu, r1 >> 16, &s_root);
        }
        if (ntask <= kSweepBlockTasks) {
            // a level of few ranges: the whole block on each larger range in turn
            for (uint32_t q = 0; q < ntask; ++q) {
                const uint32_t r0 = S.task[cur][2 * q], r1 = S.task[cur][2 * q + 1];
                const uint32_t s = r0 & 0xFFFFu, e = r0 >> 16;
                if (e - s <= kSweepSerial) continue;
                uint32_t rb[6];
                const uint32_t k = sweep_block(S, s_blk, s, e, rb);
                if (t == 0)
                    emit_split(S, nodes, n, s, e, k, r1 & 0xFFFFu, r1 >> 16, rb, &s_count[cur ^ 1], S.task[cur ^ 1],
                               &s_root);
            }
        } else {
            if (team < kTeams) {
                // larger ranges: a team of three warps each, one axis per warp; the
                // halves queued for the next level
                for (uint32_t q = team; q < ntask; q += kTeams) {
                    const uint32_t r0 = S.task[cur][2 * q], r1 = S.task[cur][2 * q + 1];
                    const uint32_t s = r0 & 0xFFFFu, e = r0 >> 16, parent = r1 & 0xFFFFu, slot = r1 >> 16;
                    if (e - s <= kSweepWarpMax) continue;
                    uint32_t rb[6];
                    const Split mine = sweep_axis(S, axw, s, e, rb);
                    if (lane == 0) {
                        s_split[team][axw] = mine;
                        if (axw == 0)
                            for (int a = 0; a < 6; ++a) s_box[team][a] = rb[a];
                    }
                    team_sync(team);
                    Split best = s_split[team][0];
                    for (int a = 1; a < 3; ++a)
                        if (better(s_split[team][a], best)) best = s_split[team][a];
                    uint32_t bax = best.ax, k = best.k;
                    if (bax == 3u) { bax = 0u; k = s; }   // no cost below FLT_MAX (not for finite boxes)
                    if (axw == bax)
                        for (uint32_t i = s + lane; i < e; i += 32) S.left[S.list[bax][i]] = i <= k ? 1u : 0u;
                    team_sync(team);
                    if (axw != bax) partition_warp(S, axw, s, e, k + 1 - s);
                    team_sync(team);
                    if (axw == 0 && lane == 0) {
                        uint32_t box[6];
                        for (int a = 0; a < 6; ++a) box[a] = s_box[team][a];
                        emit_split(S, nodes, n, s, e, k, parent, slot, box, &s_count[cur ^ 1], S.task[cur ^ 1], &s_root);
                    }
                    team_sync(team);   // the team's shared slots free for its next range
                }
            }
            // ranges of kSweepSerial + 1 to kSweepWarpMax: one warp each, taken
            // in turn by whichever warp is free
            for (;;) {
                uint32_t q = 0;
                if (lane == 0) q = atomicAdd(&s_next, 1u);
                q = __shfl_sync(0xffffffffu, q, 0);
                if (q >= ntask) break;
                const uint32_t r0 = S.task[cur][2 * q], r1 = S.task[cur][2 * q + 1];
                const uint32_t s = r0 & 0xFFFFu, e = r0 >> 16;
                if (e - s <= kSweepSerial || e - s > kSweepWarpMax) continue;
                sweep_warp_small(S, nodes, n, s, e, r1 & 0xFFFFu, r1 >> 16, &s_count[cur ^ 1], S.task[cur ^ 1],
                                 &s_root);
            }
        }
        __syncthreads();
        if (t == 0) { s_count[cur] = 0u; s_next = 0u; }
        cur ^= 1;
        __syncthreads();
    }
    if (t == 0 && n > 0) {
        nodes[0] = nodes[2 * s_root];
        nodes[1] = nodes[2 * s_root + 1];
    }
}

// instance_bounds 1: one block per instance.  Each frontier box's world box
// is its transformed centre +/- its half extents through |M| (the exact box of
// the transformed box), widened by 2^-19 of the magnitudes of the terms summed
// so that float rounding cannot shrink it; the instance box is their union.
// sinst rows 0-3 of an instance hold the columns of its local-to-world matrix
// (the mesh index in row 0's w).
constexpr int kBoundsThreads = 256;
__global__ void __launch_bounds__(kBoundsThreads) k_instance_bounds(const float4* __restrict__ sinst, uint32_t rows,
                                                                   const HullRef* __restrict__ hulls,
                                                                   uint32_t mesh_count, float* __restrict__ aabbs) {
    const uint32_t i = blockIdx.x;
    const float4* r = sinst + (size_t)rows * i;
    const float4 m0 = r[0], m1 = r[1], m2 = r[2], m3 = r[3];
    const uint32_t mesh = __float_as_uint(m0.w);
    const HullRef H = mesh < mesh_count ? hulls[mesh] : HullRef{nullptr, 0u, 0u};
    const float col[4][3] = {{m0.x, m0.y, m0.z}, {m1.x, m1.y, m1.z}, {m2.x, m2.y, m2.z}, {m3.x, m3.y, m3.z}};
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t j = threadIdx.x; j < H.count; j += kBoundsThreads) {
        const float4 mn = H.boxes[2ull * j], mx = H.boxes[2ull * j + 1];
        const float c[3] = {0.5f * (mn.x + mx.x), 0.5f * (mn.y + mx.y), 0.5f * (mn.z + mx.z)};
        const float h[3] = {0.5f * (mx.x - mn.x), 0.5f * (mx.y - mn.y), 0.5f * (mx.z - mn.z)};
        for (int a = 0; a < 3; ++a) {
            float wc = col[3][a], wh = 0.0f, mag = fabsf(col[3][a]);
            for (int k = 0; k < 3; ++k) {
                wc = wc + col[k][a] * c[k];
                wh = wh + fabsf(col[k][a]) * h[k];
                mag = mag + fabsf(col[k][a]) * (fabsf(c[k]) + h[k]);
            }
            const float pad = mag * 0x1p-19f;
            lo[a] = fminf(lo[a], wc - wh - pad);
            hi[a] = fmaxf(hi[a], wc + wh + pad);
        }
    }
    __shared__ float s[kBoundsThreads / 32][6];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (int a = 0; a < 3; ++a) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
        }
    }
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { s[warp][a] = lo[a]; s[warp][3 + a] = hi[a]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        const bool is_lo = threadIdx.x < 3;
        float v = s[0][threadIdx.x];
        for (int w = 1; w < kBoundsThreads / 32; ++w) v = is_lo ? fminf(v, s[w][threadIdx.x]) : fmaxf(v, s[w][threadIdx.x]);
        aabbs[6ull * i + threadIdx.x] = v;
    }
}

uint32_t pow2_at_least(uint32_t n) {
    uint32_t p = 1;
    while (p < n) p <<= 1;
    return p;
}

}  // namespace

cudaError_t launch_instance_bounds(const float4* sinst, uint32_t rows, uint32_t n, const HullRef* hulls,
                                   uint32_t mesh_count, float* aabbs, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    k_instance_bounds<<<n, kBoundsThreads, 0, stream>>>(sinst, rows, hulls, mesh_count, aabbs);
    return cudaGetLastError();
}

size_t tlas_scratch_words(uint32_t n, uint32_t metric) {
    if (metric == 2) return (n <= kPlocSmemMax) ? 8 : ploc_bytes(n, pow2_at_least(n ? n : 1)) / 4 + 8;
    if (metric == 3) return (n <= kSweepSmemMax) ? 8 : sweep_words(n, pow2_at_least(n ? n : 1)) + 8;
    return 7ull * n + 1;
}

cudaError_t launch_tlas_build(const float* aabbs, uint32_t n, float4* nodes, uint32_t* scratch, uint32_t metric,
                              cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (metric == 2) {
        // the working set in shared memory up to kPlocSmemMax instances
        // (152 KiB at 2048), else in the scratch (8-byte aligned: cudaMalloc)
        const uint32_t P = pow2_at_least(n);
        const bool smem = n <= kPlocSmemMax;
        const size_t bytes = smem ? ploc_bytes(n, P) : 0;
        if (bytes > 48u * 1024u) {
            cudaError_t e = cudaFuncSetAttribute(k_tlas_ploc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            if (e != cudaSuccess) return e;
        }
        k_tlas_ploc<<<1, kPlocThreads, bytes, stream>>>(aabbs, n, nodes, scratch, P, smem);
        return cudaGetLastError();
    }
    if (metric == 3) {
        // the working set in shared memory up to kSweepSmemMax instances
        // (152 KiB at 2048), else in the scratch
        const uint32_t P = pow2_at_least(n);
        const bool smem = n <= kSweepSmemMax;
        const size_t bytes = smem ? 4 * sweep_words(n, P) : 0;
        if (bytes > 48u * 1024u) {
            cudaError_t e = cudaFuncSetAttribute(k_tlas_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
            if (e != cudaSuccess) return e;
        }
        k_tlas_sweep<<<1, kPlocThreads, bytes, stream>>>(aabbs, n, nodes, scratch, P, smem);
        return cudaGetLastError();
    }
    size_t smem = (n <= kSmemInstances) ? (size_t)n * 7u * 4u : 0u;
    if (smem > 48u * 1024u) {
        cudaError_t e = cudaFuncSetAttribute(k_tlas_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_tlas_build<<<1, 32, smem, stream>>>(aabbs, n, nodes, scratch, metric);
    return cudaGetLastError();
}

// ============================================================================
// Allocation-free TLAS build (wf_tlas_build_noalloc).
//
// Some callers cannot allocate device memory: a per-frame render thread where
// an allocation's implicit device-wide synchronisation would stall the frame,
// or an engine that hands out all of its device memory from a budget fixed up
// front (its own pool, a hard memory cap).  They pass their own
// device buffers for the instance boxes and the output nodes; the build's
// working list (7 words per instance) lives in one fixed-size static device
// array that every call on a device shares.

namespace {

constexpr uint32_t kNoAllocMaxInstances = 8192;
constexpr int kNoAllocMaxContexts = 64;

// 7 x 8192 words = 224 KiB, resident on every GPU that loads the library.
static __device__ __align__(256) uint32_t g_tlas_noalloc_list[7u * kNoAllocMaxInstances];

// The array's device address per CUDA context (a module global has its own
// address in each context: the device's primary context, or one an engine
// created and made current itself).
struct NoAllocAddr {
    void* ctx;
    uint32_t* list;
};
std::mutex g_noalloc_mu;
NoAllocAddr g_noalloc_addr[kNoAllocMaxContexts] = {};
int g_noalloc_count = 0;

// cuCtxGetCurrent, looked up through the runtime (no link against the driver library).
typedef int (*CtxGetCurrentFn)(void** ctx);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<CtxGetCurrentFn>(f);
    }();
    return fn;
}

// The walk of k_tlas_build with the list in the static array (`list` is its
// device address).
__global__ void __launch_bounds__(32) k_tlas_build_noalloc(const float* __restrict__ aabbs, uint32_t n,
                                                           float4* nodes, uint32_t* list, uint32_t metric) {
    tlas_walk(aabbs, n, nodes, list, metric);
}

}  // namespace

}  // namespace wf

extern "C" int wf_tlas_build_noalloc(const float* device_aabbs, uint32_t instance_count, void* device_nodes,
                                     uint32_t tlas_metric, void* stream) {
    using namespace wf;
    if (instance_count > kNoAllocMaxInstances)
        return report_error(WF_ERR_CAPACITY, "wf_tlas_build_noalloc: at most 8192 instances (static working list)");
    if (!device_nodes || (instance_count > 0 && !device_aabbs))
        return report_error(WF_ERR_INVALID, "wf_tlas_build_noalloc: null device pointer");
    if (tlas_metric > 1) return report_error(WF_ERR_INVALID, "wf_tlas_build_noalloc: tlas_metric must be 0 or 1");
    if ((reinterpret_cast<uintptr_t>(device_aabbs) & 3u) || (reinterpret_cast<uintptr_t>(device_nodes) & 15u))
        return report_error(WF_ERR_INVALID, "wf_tlas_build_noalloc: boxes must be 4-byte, nodes 16-byte aligned");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return report_error(WF_ERR_CUDA, "wf_tlas_build_noalloc: no usable current CUDA device");
    }
    // The current context.  It is still null when no call has made the
    // device's primary context current yet; cudaGetSymbolAddress below does,
    // and the entry is keyed by the context current after it.
    CtxGetCurrentFn get_ctx = ctx_get_current();
    void* ctx = nullptr;
    if (get_ctx) get_ctx(&ctx);
    uint32_t* list = nullptr;
    {
        // Set-up, once per context, with that context current: the host-side
        // name g_tlas_noalloc_list is only a stand-in, so the kernel gets the
        // array's device address.
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        for (int i = 0; ctx && i < g_noalloc_count; ++i)
            if (g_noalloc_addr[i].ctx == ctx) list = g_noalloc_addr[i].list;
        if (!list) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_tlas_noalloc_list);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return report_error(WF_ERR_CUDA, "wf_tlas_build_noalloc: cudaGetSymbolAddress failed");
            }
            list = static_cast<uint32_t*>(p);
            if (get_ctx && !ctx) get_ctx(&ctx);   // the lookup made the primary context current
            if (ctx && g_noalloc_count < kNoAllocMaxContexts) g_noalloc_addr[g_noalloc_count++] = {ctx, list};
        }
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (instance_count == 0) {
        e = cudaMemsetAsync(device_nodes, 0, 32, st);   // one zero node, as tlas_builder_t leaves it
    } else {
        k_tlas_build_noalloc<<<1, 32, 0, st>>>(device_aabbs, instance_count, static_cast<float4*>(device_nodes),
                                                list, tlas_metric);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return report_error(WF_ERR_CUDA, cudaGetErrorString(e));
    return WF_OK;
}

