// wf_traverse.cuh — software TLAS -> BLAS traversal (closest hit / any hit).
//
// Per ray it follows trace_ray_tlas / trace_ray_bvh_instance /
// trace_ray_bvh_local (accelstruct.hlsl:58-218) step for step: TLAS root box
// test, near-child-first descent with ties to the left, far child pushed only
// when it was hit, leaf triangles tested in index-list order with strict
// "t < ray.t" acceptance (the first triangle found wins an exact tie),
// instance rays transformed by world_to_local without renormalising.  The
// reference pushes whole node copies; this pushes the 8 bytes a popped node
// needs ({left_first, prim_count} or {left_right, instance_idx}), which visits
// the same nodes in the same order.  Each level keeps its own 64-entry stack,
// as the reference; an overflow abandons the ray (reported as a miss) and
// raises ERRF_STACK where the reference would write past its array.
//
// GPU organisation: a persistent grid; every warp runs one warp-uniform loop
// whose iterations perform one traversal step per lane — an interior visit
// (the same code for TLAS and BLAS nodes: two child boxes, one slab test
// each), an instance entry, or one triangle of a leaf — so lanes stay converged on
// the common interior step instead of drifting apart in nested per-lane loops.
// Lanes whose ray finished take new rays in groups through one atomic per warp
// (kRefill idle lanes, or all of them) from a per-launch counter.
#pragma once
#include <type_traits>
#include "wf_device.cuh"

namespace wf {

struct Hit {
    uint32_t inst, prim;
    float t, u, v;
};

struct LocalCounters {
    uint32_t tlas_nodes, instances, blas_nodes, tris;
};

constexpr uint32_t kNoRay = 0xFFFFFFFFu;
// Threads per block of the persistent traversal kernels.
#ifndef WF_TRACE_BLOCK
#define WF_TRACE_BLOCK 128
#endif
constexpr int kTraceBlock = WF_TRACE_BLOCK;
// Traversal stack: one LIFO for both levels (the TLAS entries below, the
// current instance's BLAS entries above them), 64 entries per level as the
// reference.  Its top WF_TRACE_RING entries live in a shared-memory ring (slot
// index % ring, one column per thread), the older ones in local memory; a
// push into a full ring moves the ring's oldest entry to local memory, a pop
// from an empty ring reads local memory.  WF_TRACE_RING 0 keeps the whole
// stack in local memory.
#ifndef WF_TRACE_RING
#define WF_TRACE_RING 8
#endif
// A warp takes new rays once this many of its lanes are idle (or all are).
#ifndef WF_TRACE_REFILL
#define WF_TRACE_REFILL 12
#endif
constexpr int kRefill = WF_TRACE_REFILL;

// Ray sources / sinks.  load(i, o, d, tmax, no_cull); root(i, S) = the TLAS
// root node of the ray's scene, kInvalid for an empty scene; store(i, hit, ok)
// where ok is false when a traversal stack overflowed.  A source that mixes
// closest-hit and any-hit rays in one launch also has any(i) (true for an
// any-hit ray); the others take the kernel's ANY for every ray.
template <class IO, class = void>
struct MixedIO : std::false_type {};
template <class IO>
struct MixedIO<IO, std::void_t<decltype(std::declval<const IO&>().any(0u))>> : std::true_type {};

struct AosIO {
    const float4* rays;   // RayDesc2
    uint32_t* hits;       // hit_result_t
    bool no_cull;
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        const float4 a = ldg4(rays + 2ull * i), b = ldg4(rays + 2ull * i + 1);
        o = xyz(a); d = xyz(b); tmax = b.w; nc = no_cull;
    }
    __device__ __forceinline__ uint32_t root(uint32_t, const SceneRefs& S) const { return S.inst_count ? 0u : kInvalid; }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool) const {
        uint32_t* o = hits + 5ull * i;
        o[0] = h.inst; o[1] = h.prim; o[2] = __float_as_uint(h.t); o[3] = __float_as_uint(h.u);
        o[4] = __float_as_uint(h.v);
    }
};

// The same rays traced in the order of a permutation (the k-th ray handed
// out is ray perm[k]); each hit still lands at its ray's own index.
struct PermutedAosIO {
    AosIO io;
    const uint32_t* perm;
    const uint32_t* varied;   // 0: the permutation was not built (identity)
    __device__ __forceinline__ uint32_t ray(uint32_t k) const { return *varied ? perm[k] : k; }
    __device__ __forceinline__ void load(uint32_t k, V3& o, V3& d, float& tmax, bool& nc) const {
        io.load(ray(k), o, d, tmax, nc);
    }
    __device__ __forceinline__ uint32_t root(uint32_t, const SceneRefs& S) const { return S.inst_count ? 0u : kInvalid; }
    __device__ __forceinline__ void store(uint32_t k, const Hit& h, bool ok) const { io.store(ray(k), h, ok); }
};

// LAY: the BLAS layout (0 = binary child pairs; 1 = quantized and 2 = exact
// 4-wide nodes, csrc/wf_qbvh.cu).  Over the 4-wide nodes closest-hit rays use
// the order-independent tie rule (smallest t, then smallest (instance,
// primitive); boxes entered at exactly t still visited), so their hits equal
// the binary traversal's whatever order the wider nodes visit leaves in.
// Any-hit rays keep "t < tmax": only whether they hit matters.
template <bool ANY, bool COUNT, int LAY, class IO>
__device__ __forceinline__ void trace_persistent(const SceneRefs& S, const IO& io, uint32_t n, uint32_t* fetch,
                                                 LocalCounters& cnt, bool& overflow) {
    constexpr bool QB = LAY != 0;   // a 4-wide layout, with the tie rule
    const unsigned FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t col = threadIdx.x;
    // State a step rarely touches lives in shared memory, one column per
    // thread, to keep the loop's registers (and so the resident warps) up:
    // the world ray (read back when the ray leaves an instance) and the hit
    // record (written on a hit, read when the ray finishes).
    __shared__ float4 s_wo[kTraceBlock], s_wd[kTraceBlock];
    __shared__ uint32_t s_inst[kTraceBlock], s_prim[kTraceBlock];
    __shared__ float s_t[kTraceBlock], s_u[kTraceBlock], s_v[kTraceBlock];
    uint32_t ri = kNoRay;
    bool exhausted = false;
    bool any_ray = ANY;   // this lane's ray stops at its first hit
    // current-space ray and 1/dir; ct = ray.t (the closest hit so far, shared
    // by world and object space because instance rays are not renormalised)
    V3 co = mk(0, 0, 0), cd = mk(0, 0, 0), ci = mk(0, 0, 0);
    float ct = 0.0f;
    bool no_cull = false, hit_here = false;
    uint32_t level = 0, w0 = 0, w1 = 0, ii = 0;
    BlasRef B;
    B.nodes = nullptr; B.tris = nullptr;
    // stack: entries [0, sp); the TLAS level's are [0, tb) while inside an
    // instance; [lo, sp) are in the ring, [0, lo) in local memory
    int sp = 0, lo = 0, tb = 0;
    uint2 deep[2 * kStack];
#if WF_TRACE_RING > 0
    __shared__ uint2 ring[WF_TRACE_RING][kTraceBlock];
    auto stack_push = [&](uint2 e) {
        if (sp - lo == WF_TRACE_RING) {
            deep[lo] = ring[lo % WF_TRACE_RING][col];
            lo++;
        }
        ring[sp % WF_TRACE_RING][col] = e;
        sp++;
    };
    auto stack_pop = [&]() -> uint2 {
        sp--;
        if (sp >= lo) return ring[sp % WF_TRACE_RING][col];
        lo = sp;
        return deep[sp];
    };
#else
    auto stack_push = [&](uint2 e) { deep[sp++] = e; };
    auto stack_pop = [&]() -> uint2 { return deep[--sp]; };
#endif
    auto hit_record = [&]() {
        Hit h;
        h.inst = s_inst[col]; h.prim = s_prim[col]; h.t = s_t[col]; h.u = s_u[col]; h.v = s_v[col];
        return h;
    };
    auto clear_hit = [&]() {
        s_inst[col] = kInvalid; s_prim[col] = kInvalid; s_t[col] = FLT_MAX; s_u[col] = 0.0f; s_v[col] = 0.0f;
    };

    for (;;) {
        // ---- refill idle lanes (one atomic per warp)
        const bool idle = ri == kNoRay;
        const unsigned want = __ballot_sync(FULL, idle && !exhausted);
        if (want) {
            const unsigned busy = __ballot_sync(FULL, !idle);
            if (busy == 0u || __popc(want) >= kRefill) {
                const int leader = __ffs(want) - 1;
                uint32_t base = 0;
                if ((int)lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(want));
                base = __shfl_sync(FULL, base, leader);
                if (idle && !exhausted) {
                    const uint32_t k = base + (uint32_t)__popc(want & ((1u << lane) - 1u));
                    if (k < n) {
                        ri = k;
                        io.load(k, co, cd, ct, no_cull);
                        if constexpr (MixedIO<IO>::value) any_ray = io.any(k);
                        s_wo[col] = make_float4(co.x, co.y, co.z, 0.0f);
                        s_wd[col] = make_float4(cd.x, cd.y, cd.z, 0.0f);
                        clear_hit();
                        ci = rcp(cd);
                        const uint32_t root = io.root(k, S);
                        bool miss = root == kInvalid;
                        if (!miss && !in_bounds(root, S.tnode_count, S.status)) miss = true;
                        if (!miss) {
                            const float4 n0 = ldg4(S.tnodes + 2ull * root), n1 = ldg4(S.tnodes + 2ull * root + 1);
                            if (COUNT) cnt.tlas_nodes++;
                            miss = ((QB && !any_ray) ? slab_le(xyz(n0), xyz(n1), co, ci, ct)
                                                     : slab(xyz(n0), xyz(n1), co, ci, ct)) == FLT_MAX;
                            level = 0; w0 = __float_as_uint(n0.w); w1 = __float_as_uint(n1.w); sp = 0; lo = 0;
                        }
                        if (miss) { io.store(k, hit_record(), true); ri = kNoRay; }
                    } else {
                        exhausted = true;
                    }
                }
            }
        }
        const unsigned active = __ballot_sync(FULL, ri != kNoRay);
        if (active == 0u) {
            if (__all_sync(FULL, exhausted)) break;
            continue;
        }
        if (ri == kNoRay) continue;

        // ---- one traversal step
        bool finish = false, ok = true;
        bool pop = false;
        if (level == 0u && w0 == 0u) {
            // TLAS leaf: enter the instance (trace_ray_bvh_instance); at level
            // 0 the current ray is the world ray
            ii = w1;
            const float4* ip = S.tinst + 4ull * ii;
            if (!in_bounds(ii, S.inst_count, S.status)) {
                pop = true;
            } else {
                const float4 c0 = ldg4(ip), c1 = ldg4(ip + 1), c2 = ldg4(ip + 2), c3 = ldg4(ip + 3);
                if (COUNT) cnt.instances++;
                const uint32_t mesh = __float_as_uint(c0.w);
                if (!in_bounds(mesh, S.mesh_count, S.status)) {
                    pop = true;
                } else {
                    co = xform(co, 1.0f, c0, c1, c2, c3);
                    cd = xform(cd, 0.0f, c0, c1, c2, c3);
                    ci = rcp(cd);
                    B = S.blas[mesh];
                    if (QB) {
                        // node 0, or the one leaf of a single-leaf BLAS
                        w0 = 0u;
                        w1 = B.root_count;
                    } else {
                        const float4 r0 = ldg4(B.nodes), r1 = ldg4(B.nodes + 1);
                        if (COUNT) cnt.blas_nodes++;
                        w0 = __float_as_uint(r0.w);
                        w1 = __float_as_uint(r1.w);
                    }
                    level = 1; tb = sp; hit_here = false;
                }
            }
        } else if (level == 1u && w1 > 0u && !in_bounds(w0, B.tri_count, S.status)) {
            w1 = 0u;
            pop = true;
        } else if (level == 1u && w1 > 0u) {
            // BLAS leaf: one triangle per step, in index-list order (w0 = the
            // next triangle, w1 = triangles left), so lanes on interior nodes
            // never wait for a whole leaf
            const float4* tp = B.tris + 3ull * w0;
            const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
            if (COUNT) cnt.tris++;
            float bu, bv;
            bool accepted;
            if (QB && !any_ray) {
                // the current hit: this instance once it has one here, else the outer one
                const uint32_t bi = hit_here ? ii : s_inst[col];
                const uint32_t pr = __float_as_uint(a.w);
                const bool wins = ii < bi || (ii == bi && pr < s_prim[col]);
                accepted = tri_hit_tie(xyz(a), xyz(b), xyz(c), co, cd, ct, bu, bv, no_cull, wins);
            } else {
                accepted = tri_hit(xyz(a), xyz(b), xyz(c), co, cd, ct, bu, bv, no_cull);
            }
            if (accepted) {
                s_prim[col] = __float_as_uint(a.w);
                s_u[col] = bu; s_v[col] = bv;
                hit_here = true;
                if (any_ray) { s_inst[col] = ii; s_t[col] = ct; finish = true; }
            }
            w0++;
            w1--;
            pop = !finish && w1 == 0u;
        } else if (QB && level == 1u) {
            // 4-wide BLAS node: up to four child boxes (quantized: origin + q *
            // 2^e per plane; exact: the planes as stored), visited nearest
            // first, the others pushed
            if (!in_bounds(w0, B.qnode_count, S.status)) {
                pop = true;
            } else {
                const bool tie = !any_ray;
                float d[4];
                uint2 e[4];
                if constexpr (LAY == 1) {
                    const float4* qp = B.qnodes + 4ull * w0;
                    const float4 q0 = ldg4(qp), q1 = ldg4(qp + 1), q2 = ldg4(qp + 2), q3 = ldg4(qp + 3);
                    if (COUNT) cnt.blas_nodes += 2;   // 64 bytes, as a binary child pair
                    const uint32_t meta = __float_as_uint(q0.w);
                    const float sx = __uint_as_float((meta & 0xFFu) << 23);
                    const float sy = __uint_as_float(((meta >> 8) & 0xFFu) << 23);
                    const float sz = __uint_as_float(((meta >> 16) & 0xFFu) << 23);
                    const uint32_t nch = meta >> 24;
                    const uint32_t lx = __float_as_uint(q1.x), ly = __float_as_uint(q1.y), lz = __float_as_uint(q1.z);
                    const uint32_t hx = __float_as_uint(q2.x), hy = __float_as_uint(q2.y), hz = __float_as_uint(q2.z);
                    const uint32_t cl = __float_as_uint(q1.w), chi = __float_as_uint(q2.w);
                    const uint32_t kid[4] = {__float_as_uint(q3.x), __float_as_uint(q3.y), __float_as_uint(q3.z),
                                             __float_as_uint(q3.w)};
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const uint32_t sh = 8u * (uint32_t)i;
                        const V3 bmn = mk(q0.x + (float)((lx >> sh) & 0xFFu) * sx, q0.y + (float)((ly >> sh) & 0xFFu) * sy,
                                          q0.z + (float)((lz >> sh) & 0xFFu) * sz);
                        const V3 bmx = mk(q0.x + (float)((hx >> sh) & 0xFFu) * sx, q0.y + (float)((hy >> sh) & 0xFFu) * sy,
                                          q0.z + (float)((hz >> sh) & 0xFFu) * sz);
                        const float di = tie ? slab_le(bmn, bmx, co, ci, ct) : slab(bmn, bmx, co, ci, ct);
                        d[i] = (uint32_t)i < nch ? di : FLT_MAX;
                        e[i] = make_uint2(kid[i], ((cl >> sh) & 0xFFu) | (((chi >> sh) & 0xFFu) << 8));
                    }
                } else {
                    const float4* wp = B.qnodes + 8ull * w0;
                    const float4 xl = ldg4(wp), xh = ldg4(wp + 1), yl = ldg4(wp + 2), yh = ldg4(wp + 3);
                    const float4 zl = ldg4(wp + 4), zh = ldg4(wp + 5), en = ldg4(wp + 6), cn = ldg4(wp + 7);
                    if (COUNT) cnt.blas_nodes += 4;   // 128 bytes, as two binary child pairs
                    const uint32_t nch = __float_as_uint(cn.x) >> 24;
                    auto lane4 = [](const float4& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; };
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const V3 bmn = mk(lane4(xl, i), lane4(yl, i), lane4(zl, i));
                        const V3 bmx = mk(lane4(xh, i), lane4(yh, i), lane4(zh, i));
                        const float di = tie ? slab_le(bmn, bmx, co, ci, ct) : slab(bmn, bmx, co, ci, ct);
                        d[i] = (uint32_t)i < nch ? di : FLT_MAX;
                        const uint32_t c = __float_as_uint(lane4(cn, i));
                        e[i] = make_uint2(__float_as_uint(lane4(en, i)), i == 0 ? (c & 0x00FFFFFFu) : c);
                    }
                }
                // order the four by entry distance (a five-comparator network)
                auto cswap = [&](int a, int b) {
                    if (d[a] > d[b]) {
                        const float td = d[a]; d[a] = d[b]; d[b] = td;
                        const uint2 te = e[a]; e[a] = e[b]; e[b] = te;
                    }
                };
                cswap(0, 1); cswap(2, 3); cswap(0, 2); cswap(1, 3); cswap(1, 2);
                if (d[0] == FLT_MAX) {
                    pop = true;
                } else {
                    w0 = e[0].x; w1 = e[0].y;
#pragma unroll
                    for (int i = 3; i >= 1; --i) {
                        if (d[i] != FLT_MAX && !finish) {
                            if (sp - tb == kStack) {
                                clear_hit();
                                finish = true; ok = false; overflow = true;
                            } else {
                                stack_push(e[i]);
                            }
                        }
                    }
                }
            }
        } else {
            // interior node, TLAS or BLAS: the two children, nearer first
            const float4* pa;
            const float4* pb;
            if (level == 0u) {
                pa = S.tnodes + 2ull * (w0 >> 16);
                pb = S.tnodes + 2ull * (w0 & 0xFFFFu);
            } else {
                pa = B.nodes + 2ull * w0;
                pb = pa + 2;
            }
            if (level == 0u ? !(in_bounds(w0 >> 16, S.tnode_count, S.status) &&
                                in_bounds(w0 & 0xFFFFu, S.tnode_count, S.status))
                            : !in_bounds(w0 + 1ull, B.node_count, S.status)) {
                pop = true;
            } else {
                const float4 a0 = ldg4(pa), a1 = ldg4(pa + 1), b0 = ldg4(pb), b1 = ldg4(pb + 1);
                if (COUNT) { if (level == 0u) cnt.tlas_nodes += 2; else cnt.blas_nodes += 2; }
                const bool tie = QB && !any_ray;
                float dl = tie ? slab_le(xyz(a0), xyz(a1), co, ci, ct) : slab(xyz(a0), xyz(a1), co, ci, ct);
                float dr = tie ? slab_le(xyz(b0), xyz(b1), co, ci, ct) : slab(xyz(b0), xyz(b1), co, ci, ct);
                uint2 L = make_uint2(__float_as_uint(a0.w), __float_as_uint(a1.w));
                uint2 R = make_uint2(__float_as_uint(b0.w), __float_as_uint(b1.w));
                if (dl > dr) {
                    float td = dl; dl = dr; dr = td;
                    uint2 tn = L; L = R; R = tn;
                }
                if (dl == FLT_MAX) {
                    pop = true;
                } else {
                    w0 = L.x; w1 = L.y;
                    if (dr != FLT_MAX) {
                        if ((level == 0u ? sp : sp - tb) == kStack) {
                            clear_hit();
                            finish = true; ok = false; overflow = true;
                        } else {
                            stack_push(R);
                        }
                    }
                }
            }
        }
        if (pop) {
            if (level == 1u) {
                if (sp > tb) {
                    const uint2 e = stack_pop();
                    w0 = e.x; w1 = e.y;
                    pop = false;
                } else {
                    // leave the instance: ray.t = ray_local.t (accelstruct.hlsl:146, 170-174)
                    if (hit_here) { s_inst[col] = ii; s_t[col] = ct; }
                    level = 0;
                    co = xyz(s_wo[col]); cd = xyz(s_wd[col]); ci = rcp(cd);
                }
            }
            if (pop) {
                if (sp > 0) {
                    const uint2 e = stack_pop();
                    w0 = e.x; w1 = e.y;
                } else {
                    finish = true;
                }
            }
        }
        if (finish) {
            io.store(ri, hit_record(), ok);
            ri = kNoRay;
        }
    }
}

// One ray traced by one thread in nested TLAS / BLAS loops (the structure of
// accelstruct.hlsl:58-218 as written), for the megakernel path.  It visits the
// same nodes and triangles in the same order as trace_persistent and returns
// the same hit; false when a stack overflowed (the hit is then a miss).
template <bool ANY>
__device__ __forceinline__ bool trace_single(const SceneRefs& S, uint32_t root, V3 wo, V3 wd, float tmax,
                                             bool no_cull, Hit& h) {
    h.inst = kInvalid; h.prim = kInvalid; h.t = FLT_MAX; h.u = 0.0f; h.v = 0.0f;
    if (root == kInvalid || !in_bounds(root, S.tnode_count, S.status)) return true;
    const V3 wi = rcp(wd);
    float wt = tmax;
    float4 n0 = ldg4(S.tnodes + 2ull * root), n1 = ldg4(S.tnodes + 2ull * root + 1);
    if (slab(xyz(n0), xyz(n1), wo, wi, wt) == FLT_MAX) return true;
    uint32_t t0 = __float_as_uint(n0.w), t1 = __float_as_uint(n1.w);
    uint2 tstack[kStack];
    int tsp = 0;
    for (;;) {
        if (t0 == 0u) {
            // trace_ray_bvh_instance: the ray in object space, t shared
            const uint32_t ii = t1;
            const float4* ip = S.tinst + 4ull * ii;
            const float4 c0 = in_bounds(ii, S.inst_count, S.status) ? ldg4(ip) : make_float4(0.f, 0.f, 0.f, 0.f);
            if (!in_bounds(ii, S.inst_count, nullptr) || !in_bounds(__float_as_uint(c0.w), S.mesh_count, S.status)) {
                if (tsp == 0) break;
                const uint2 e = tstack[--tsp];
                t0 = e.x; t1 = e.y;
                continue;
            }
            const float4 c1 = ldg4(ip + 1), c2 = ldg4(ip + 2), c3 = ldg4(ip + 3);
            const V3 co = xform(wo, 1.0f, c0, c1, c2, c3);
            const V3 cd = xform(wd, 0.0f, c0, c1, c2, c3);
            const V3 ci = rcp(cd);
            float ct = wt;
            const BlasRef B = S.blas[__float_as_uint(c0.w)];
            const float4 r0 = ldg4(B.nodes), r1 = ldg4(B.nodes + 1);
            uint32_t b0 = __float_as_uint(r0.w), b1 = __float_as_uint(r1.w);
            uint2 bstack[kStack];
            int bsp = 0;
            bool hit_here = false;
            for (;;) {
                bool pop = false;
                if (b1 > 0u && !in_bounds((uint64_t)b0 + b1 - 1u, B.tri_count, S.status)) {
                    pop = true;
                } else if (b1 > 0u) {
                    for (uint32_t i = b0; i < b0 + b1; ++i) {
                        const float4* tp = B.tris + 3ull * i;
                        const float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
                        float bu, bv;
                        if (tri_hit(xyz(a), xyz(b), xyz(c), co, cd, ct, bu, bv, no_cull)) {
                            h.prim = __float_as_uint(a.w);
                            h.u = bu; h.v = bv;
                            hit_here = true;
                            if (ANY) { h.inst = ii; h.t = ct; return true; }
                        }
                    }
                    pop = true;
                } else if (!in_bounds(b0 + 1ull, B.node_count, S.status)) {
                    pop = true;
                } else {
                    const float4* pa = B.nodes + 2ull * b0;
                    const float4 a0 = ldg4(pa), a1 = ldg4(pa + 1), q0 = ldg4(pa + 2), q1 = ldg4(pa + 3);
                    float dl = slab(xyz(a0), xyz(a1), co, ci, ct);
                    float dr = slab(xyz(q0), xyz(q1), co, ci, ct);
                    uint2 L = make_uint2(__float_as_uint(a0.w), __float_as_uint(a1.w));
                    uint2 R = make_uint2(__float_as_uint(q0.w), __float_as_uint(q1.w));
                    if (dl > dr) { float td = dl; dl = dr; dr = td; uint2 tn = L; L = R; R = tn; }
                    if (dl == FLT_MAX) {
                        pop = true;
                    } else {
                        b0 = L.x; b1 = L.y;
                        if (dr != FLT_MAX) {
                            if (bsp == kStack) {
                                h.inst = kInvalid; h.prim = kInvalid; h.t = FLT_MAX; h.u = 0.0f; h.v = 0.0f;
                                return false;
                            }
                            bstack[bsp++] = R;
                        }
                    }
                }
                if (pop) {
                    if (bsp == 0) break;
                    const uint2 e = bstack[--bsp];
                    b0 = e.x; b1 = e.y;
                }
            }
            wt = ct;
            if (hit_here) { h.inst = ii; h.t = wt; }
            if (tsp == 0) break;
            const uint2 e = tstack[--tsp];
            t0 = e.x; t1 = e.y;
            continue;
        }
        if (!(in_bounds(t0 >> 16, S.tnode_count, S.status) && in_bounds(t0 & 0xFFFFu, S.tnode_count, S.status))) {
            if (tsp == 0) break;
            const uint2 e = tstack[--tsp];
            t0 = e.x; t1 = e.y;
            continue;
        }
        const float4* pa = S.tnodes + 2ull * (t0 >> 16);
        const float4* pb = S.tnodes + 2ull * (t0 & 0xFFFFu);
        const float4 a0 = ldg4(pa), a1 = ldg4(pa + 1), q0 = ldg4(pb), q1 = ldg4(pb + 1);
        float dl = slab(xyz(a0), xyz(a1), wo, wi, wt);
        float dr = slab(xyz(q0), xyz(q1), wo, wi, wt);
        uint2 L = make_uint2(__float_as_uint(a0.w), __float_as_uint(a1.w));
        uint2 R = make_uint2(__float_as_uint(q0.w), __float_as_uint(q1.w));
        if (dl > dr) { float td = dl; dl = dr; dr = td; uint2 tn = L; L = R; R = tn; }
        if (dl == FLT_MAX) {
            if (tsp == 0) break;
            const uint2 e = tstack[--tsp];
            t0 = e.x; t1 = e.y;
        } else {
            t0 = L.x; t1 = L.y;
            if (dr != FLT_MAX) {
                if (tsp == kStack) {
                    h.inst = kInvalid; h.prim = kInvalid; h.t = FLT_MAX; h.u = 0.0f; h.v = 0.0f;
                    return false;
                }
                tstack[tsp++] = R;
            }
        }
    }
    return true;
}

// Adds a thread's fetch counts to the global counters (one atomic per warp).
__device__ __forceinline__ void flush_counters(const LocalCounters& c, Counters* g) {
    unsigned long long a = c.tlas_nodes, b = c.instances, x = c.blas_nodes, y = c.tris;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
        x += __shfl_down_sync(0xffffffffu, x, off);
        y += __shfl_down_sync(0xffffffffu, y, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&g->tlas_node_loads, a);
        atomicAdd(&g->instance_loads, b);
        atomicAdd(&g->blas_node_loads, x);
        atomicAdd(&g->triangle_tests, y);
    }
}

// Minimum resident blocks per SM asked of the compiler for the traversal
// kernels (it caps their registers at 65536 / (128 * blocks)): 9 blocks = 56
// registers, 36 warps per SM, for a few bytes of spills in the closest-hit
// kernel (measured fastest against 7-8 blocks without spills and 10 blocks
// with 50+ bytes of spills).
#ifndef WF_TRACE_MIN_BLOCKS
#define WF_TRACE_MIN_BLOCKS 9
#endif
// The same for the 4-wide BLAS layouts, whose node step holds four child
// boxes and their sort keys at once: 8 blocks (64 registers) measured 1-3 %
// faster than 9 (56 registers, 40-72 bytes of spills) on both layouts.
#ifndef WF_TRACE_QB_MIN_BLOCKS
#define WF_TRACE_QB_MIN_BLOCKS 8
#endif
int sm_count();

// The traversal kernel: a persistent grid over count rays (read from
// count_ptr on the device when it is non-null), rays handed out from *fetch.
// total (optional) accumulates the number of rays of each launch.
template <bool ANY, bool COUNT, int LAY, class IO>
__global__ void __launch_bounds__(kTraceBlock, LAY ? WF_TRACE_QB_MIN_BLOCKS : WF_TRACE_MIN_BLOCKS) k_trace(SceneRefs S, IO io, const uint32_t* count_ptr, uint32_t count,
                                                  uint32_t* fetch, uint32_t* status, Counters* counters,
                                                  unsigned long long* total) {
    const uint32_t n = count_ptr ? *count_ptr : count;
    if (total && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(total, (unsigned long long)n);
    LocalCounters c = {0, 0, 0, 0};
    bool overflow = false;
    trace_persistent<ANY, COUNT, LAY>(S, io, n, fetch, c, overflow);
    if (overflow) atomicOr(status, ERRF_STACK);
    if (COUNT) flush_counters(c, counters);
}

// Resident blocks per SM for a kernel, queried once per instantiation.
template <class K>
inline unsigned persistent_grid(K kernel) {
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceBlock, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    return (unsigned)(sm_count() * per_sm);
}

}  // namespace wf
