// wf_sort.cu — ray reordering for the stand-alone ray query (wf_trace with
// WF_TRACE_REORDER): rays are traced in the order of their origins' Morton
// codes in the scene's bounding box, so the rays a GPU holds at once start
// close together and read the same BVH nodes from L2 instead of each going to
// DRAM.  The order comes from a stable LSD radix sort of (code, ray index)
// pairs written here: three 8-bit passes of upsweep (digit counts per tile),
// an exclusive scan of the counts (digit-major, so equal digits keep their
// tiles' order) and a downsweep that ranks each tile's keys in order (warp
// match + per-warp counts) and scatters them.  Rays with equal codes keep
// their input order; when every origin falls in one cell (camera rays) the key
// pass says so in a device flag, the sort passes return at once and the rays
// are traced in their own order.  The hits land at each ray's own index;
// which ray a lane traces never changes a result.
#include "wf_kernels.h"

namespace wf {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;                        // rounds of kSortThreads keys per tile
constexpr uint32_t kTile = kSortThreads * kSortRounds;
constexpr int kRadix = 256;
constexpr int kWarps = kSortThreads / 32;
constexpr int kScanThreads = 1024, kScanItems = 4;   // 4096 counters per scan block

__device__ __forceinline__ uint32_t spread8(uint32_t v) {   // 8 bits -> every third bit of 24
    v &= 0xFFu;
    v = (v | (v << 8)) & 0x0000F00Fu;
    v = (v | (v << 4)) & 0x000C30C3u;
    v = (v | (v << 2)) & 0x00249249u;
    return v;
}

__device__ __forceinline__ uint32_t cell8(float x, float lo, float inv) {
    const float u = (x - lo) * inv;
    if (!(u > 0.0f)) return 0u;                       // also NaN
    if (u >= 1.0f) return 255u;
    return (uint32_t)(u * 256.0f) & 0xFFu;
}

// WF_SORT_DIR_BITS = k > 0: the key's top 24 - 3k bits are the origin's
// Morton code at 8 - k bits per axis and its low 3k bits the Morton code of
// the direction quantised to k bits per axis, so rays that start in one cell
// are also ordered by where they go.
#ifndef WF_SORT_DIR_BITS
#define WF_SORT_DIR_BITS 0
#endif
static_assert(WF_SORT_DIR_BITS >= 0 && WF_SORT_DIR_BITS <= 4, "WF_SORT_DIR_BITS: 0..4");

__device__ __forceinline__ uint32_t ray_key(const float4* __restrict__ rays, uint32_t i, float3 lo, float3 inv) {
    const float4 o = __ldg(rays + 2ull * i);
    constexpr int k = WF_SORT_DIR_BITS;
    uint32_t key = (spread8(cell8(o.x, lo.x, inv.x) >> k) << 2) | (spread8(cell8(o.y, lo.y, inv.y) >> k) << 1) |
                   spread8(cell8(o.z, lo.z, inv.z) >> k);
    if constexpr (k > 0) {
        const float4 d = __ldg(rays + 2ull * i + 1);
        // direction components in [-1, 1] -> [0, 1] -> k bits (cell8 clamps and maps NaN to 0)
        const uint32_t dx = cell8(d.x, -1.0f, 0.5f) >> (8 - k), dy = cell8(d.y, -1.0f, 0.5f) >> (8 - k),
                       dz = cell8(d.z, -1.0f, 0.5f) >> (8 - k);
        key = (key << (3 * k)) | (spread8(dx) << 2) | (spread8(dy) << 1) | spread8(dz);
    }
    return key;
}

// Key = 24-bit Morton code of the origin in the scene box (clamped), value =
// the ray's index.  Without a scene every key is 0 (the input order stays).
// scattered counts the neighbouring rays (i, i + 1, within a warp's 32) whose
// origins lie in different cells of a 16^3 grid over the scene box.
__global__ void k_origin_keys(const float4* __restrict__ rays, uint32_t n, const float4* __restrict__ root,
                              bool has_scene, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                              uint32_t* __restrict__ varied, unsigned long long* __restrict__ scattered) {
    float3 lo = make_float3(0.f, 0.f, 0.f), inv = make_float3(0.f, 0.f, 0.f);
    if (has_scene) {
        const float4 a = root[0], b = root[1];
        lo = make_float3(a.x, a.y, a.z);
        const float ex = b.x - a.x, ey = b.y - a.y, ez = b.z - a.z;
        inv = make_float3(ex > 0.f ? 1.0f / ex : 0.f, ey > 0.f ? 1.0f / ey : 0.f, ez > 0.f ? 1.0f / ez : 0.f);
    }
    const uint32_t key0 = has_scene ? ray_key(rays, 0u, lo, inv) : 0u;
    const uint32_t lane = threadIdx.x & 31u;
    bool differs = false;
    uint32_t far = 0;
    // block-uniform loop, so that every lane takes part in the shuffles
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid && has_scene ? ray_key(rays, i, lo, inv) : 0u;
        if (valid) {
            keys[i] = key;
            vals[i] = i;
            differs |= key != key0;
        }
        const uint32_t next = __shfl_down_sync(0xffffffffu, key, 1);
        const bool apart = valid && lane < 31u && i + 1u < n && ((key ^ next) >> 12) != 0u;
        far += (uint32_t)__popc(__ballot_sync(0xffffffffu, apart));
    }
    if (__any_sync(0xffffffffu, differs) && lane == 0) atomicOr(varied, 1u);
    if (lane == 0 && far) atomicAdd(scattered, (unsigned long long)far);
}

// The rays are sorted only when their origins are scattered: when fewer than
// three in four neighbouring rays share a 16^3 cell, else the input order
// stands (the sort would cost more than the locality it adds).
__global__ void k_sort_decision(uint32_t* __restrict__ varied, const unsigned long long* __restrict__ scattered,
                                uint32_t n) {
    const unsigned long long pairs = (unsigned long long)n - (n + 31u) / 32u;
    if (*varied && 4ull * *scattered < pairs) *varied = 0u;
}

// Digit counts of each tile: hist[digit * tiles + tile].
__global__ void __launch_bounds__(kSortThreads) k_upsweep(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                          uint32_t tiles, uint32_t* __restrict__ hist,
                                                          const uint32_t* __restrict__ varied) {
    if (*varied == 0u) return;   // one cell: the input order stands
    __shared__ uint32_t s_count[kRadix];
    s_count[threadIdx.x] = 0u;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const uint64_t i = base + (uint64_t)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&s_count[(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * tiles + blockIdx.x] = s_count[threadIdx.x];
}

// Exclusive scan of m counters in three steps: per-block scans with block
// totals, a scan of the totals, and the totals added back.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= (uint32_t)off) x += y;
    }
    if (lane == 31u) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const uint32_t nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= (uint32_t)off) w += y;
        }
        if (lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[(blockDim.x >> 5) - 1];
    const uint32_t before = warp ? s_warp[warp - 1] : 0u;
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(uint32_t* __restrict__ a, uint64_t m,
                                                              uint32_t* __restrict__ sums,
                                                              const uint32_t* __restrict__ varied) {
    if (*varied == 0u) return;
    __shared__ uint32_t s_warp[32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanThreads * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], t = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < m ? a[base + k] : 0u;
        t += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(t, s_warp, total);
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < m) a[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t* __restrict__ sums, uint32_t count,
                                                            const uint32_t* __restrict__ varied) {
    if (*varied == 0u) return;
    __shared__ uint32_t s_warp[32];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < count; base += kScanThreads) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < count ? sums[i] : 0u;
        uint32_t total;
        const uint32_t ex = block_exclusive_scan(v, s_warp, total);
        if (i < count) sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(uint32_t* __restrict__ a, uint64_t m,
                                                           const uint32_t* __restrict__ sums,
                                                           const uint32_t* __restrict__ varied) {
    if (*varied == 0u) return;
    const uint64_t base = (uint64_t)blockIdx.x * kScanThreads * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    const uint32_t add = sums[blockIdx.x];
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < m) a[base + k] += add;
}

// Stable scatter of one tile: its keys are ranked in input order, round by
// round (a round = kSortThreads consecutive keys, a warp = 32 of them).
__global__ void __launch_bounds__(kSortThreads) k_downsweep(const uint32_t* __restrict__ kin,
                                                            const uint32_t* __restrict__ vin, uint32_t n, int shift,
                                                            uint32_t tiles, const uint32_t* __restrict__ offsets,
                                                            uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                            const uint32_t* __restrict__ varied) {
    if (*varied == 0u) return;
    __shared__ uint32_t s_run[kRadix];
    __shared__ uint32_t s_warp[kWarps][kRadix];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    s_run[threadIdx.x] = offsets[(size_t)threadIdx.x * tiles + blockIdx.x];
    for (int w = 0; w < kWarps; ++w) s_warp[w][threadIdx.x] = 0u;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const uint64_t i = base + (uint64_t)r * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? kin[i] : 0u;
        const uint32_t val = valid ? vin[i] : 0u;
        const uint32_t d = valid ? (key >> shift) & 0xFFu : kRadix;   // kRadix: no digit
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = (uint32_t)__popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0u) s_warp[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = s_run[d] + rank;
            for (uint32_t w = 0; w < warp; ++w) pos += s_warp[w][d];
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        {
            uint32_t t = 0;
            for (int w = 0; w < kWarps; ++w) {
                t += s_warp[w][threadIdx.x];
                s_warp[w][threadIdx.x] = 0u;
            }
            s_run[threadIdx.x] += t;
        }
        __syncthreads();
    }
}

unsigned grid_for(uint64_t n, unsigned threads) {
    const uint64_t b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : (b > 65535ull * 16 ? 65535ull * 16 : b));
}

cudaError_t exclusive_scan(uint32_t* a, uint64_t m, uint32_t* sums, const uint32_t* varied, cudaStream_t stream) {
    const uint64_t per = (uint64_t)kScanThreads * kScanItems;
    const uint32_t blocks = (uint32_t)((m + per - 1) / per);
    k_scan_blocks<<<blocks, kScanThreads, 0, stream>>>(a, m, sums, varied);
    k_scan_sums<<<1, kScanThreads, 0, stream>>>(sums, blocks, varied);
    k_scan_add<<<blocks, kScanThreads, 0, stream>>>(a, m, sums, varied);
    return cudaGetLastError();
}

}  // namespace

size_t reorder_scratch_words(uint32_t n) {
    const uint64_t tiles = (n + kTile - 1) / kTile;
    const uint64_t hist = (uint64_t)kRadix * tiles;
    const uint64_t sums = (hist + (uint64_t)kScanThreads * kScanItems - 1) / ((uint64_t)kScanThreads * kScanItems);
    return 4ull * n + hist + sums + 4;   // + the flag, the scattered count (8-byte aligned)
}

cudaError_t launch_reorder_rays(const float4* rays, uint32_t n, const float4* root, bool has_scene,
                                uint32_t* scratch, const uint32_t** perm, const uint32_t** varied_out,
                                cudaStream_t stream) {
    const uint32_t tiles = (uint32_t)((n + kTile - 1) / kTile);
    uint32_t* k0 = scratch;
    uint32_t* v0 = k0 + n;
    uint32_t* k1 = v0 + n;
    uint32_t* v1 = k1 + n;
    uint32_t* hist = v1 + n;
    uint32_t* sums = hist + (size_t)kRadix * tiles;
    const size_t words = reorder_scratch_words(n);
    uint32_t* varied = scratch + words - 4;
    unsigned long long* scattered = reinterpret_cast<unsigned long long*>(scratch + ((words - 2) & ~size_t(1)));
    cudaError_t e = cudaMemsetAsync(varied, 0, 4 * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    k_origin_keys<<<grid_for(n, 256), 256, 0, stream>>>(rays, n, root, has_scene, k0, v0, varied, scattered);
    k_sort_decision<<<1, 1, 0, stream>>>(varied, scattered, n);
    e = cudaGetLastError();
    for (int pass = 0; pass < 3 && e == cudaSuccess; ++pass) {
        const int shift = 8 * pass;
        k_upsweep<<<tiles, kSortThreads, 0, stream>>>(k0, n, shift, tiles, hist, varied);
        e = exclusive_scan(hist, (uint64_t)kRadix * tiles, sums, varied, stream);
        if (e != cudaSuccess) break;
        k_downsweep<<<tiles, kSortThreads, 0, stream>>>(k0, v0, n, shift, tiles, hist, k1, v1, varied);
        e = cudaGetLastError();
        uint32_t* t = k0; k0 = k1; k1 = t;
        t = v0; v0 = v1; v1 = t;
    }
    *perm = v0;
    *varied_out = varied;
    return e;
}

}  // namespace wf
