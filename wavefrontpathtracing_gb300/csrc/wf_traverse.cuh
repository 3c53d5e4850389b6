// wf_traverse.cuh — software TLAS -> BLAS traversal (closest hit / any hit).
//
// Follows trace_ray_tlas / trace_ray_bvh_instance / trace_ray_bvh_local
// (accelstruct.hlsl:58-218) step for step: TLAS root box test, near-child-first
// descent with ties to the left, far child pushed only when it was hit, leaf
// triangles tested in index-list order with strict "t < ray.t" acceptance (the
// first triangle found wins an exact tie), instance rays transformed by
// world_to_local without renormalising.  The reference pushes whole node
// copies; this pushes the 8 bytes a popped node needs ({left_first,
// prim_count} or {left_right, instance_idx}), which visits the same nodes in
// the same order.  Each level keeps its own 64-entry stack, as the reference;
// an overflow abandons the ray (reported as a miss) and raises ERRF_STACK
// where the reference would write past its array.
#pragma once
#include "wf_device.cuh"

namespace wf {

struct Hit {
    uint32_t inst, prim;
    float t, u, v;
};

struct LocalCounters {
    uint32_t tlas_nodes, instances, blas_nodes, tris;
};

// Returns false when a stack overflowed (h then reports a miss).
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trace_ray(const SceneRefs& S, V3 o, V3 d, float tmax, bool no_cull, Hit& h,
                                          LocalCounters& cnt) {
    h.inst = kInvalid; h.prim = kInvalid; h.t = FLT_MAX; h.u = 0.0f; h.v = 0.0f;
    if (S.inst_count == 0) return true;
    const V3 inv = rcp(d);
    float t = tmax;
    float4 n0 = ldg4(S.tnodes), n1 = ldg4(S.tnodes + 1);
    if (COUNT) cnt.tlas_nodes++;
    if (slab(xyz(n0), xyz(n1), o, inv, t) == FLT_MAX) return true;
    uint32_t lr = __float_as_uint(n0.w), ii = __float_as_uint(n1.w);
    uint2 tstack[kStack];
    uint2 bstack[kStack];
    int tsp = 0;
    for (;;) {
        if (lr == 0u) {
            // instance leaf: trace_ray_bvh_instance
            const float4* ip = S.tinst + 4ull * ii;
            float4 c0 = ldg4(ip), c1 = ldg4(ip + 1), c2 = ldg4(ip + 2), c3 = ldg4(ip + 3);
            if (COUNT) cnt.instances++;
            const V3 lo = xform(o, 1.0f, c0, c1, c2, c3);
            const V3 ld = xform(d, 0.0f, c0, c1, c2, c3);
            const V3 linv = rcp(ld);
            const BlasRef B = S.blas[__float_as_uint(c0.w)];
            float lt = t;
            bool hit_here = false;
            float4 r0 = ldg4(B.nodes), r1 = ldg4(B.nodes + 1);
            if (COUNT) cnt.blas_nodes++;
            uint32_t first = __float_as_uint(r0.w), count = __float_as_uint(r1.w);
            int bsp = 0;
            for (;;) {
                if (count > 0u) {
                    for (uint32_t i = first; i < first + count; ++i) {
                        const float4* tp = B.tris + 3ull * i;
                        float4 a = ldg4(tp), b = ldg4(tp + 1), c = ldg4(tp + 2);
                        if (COUNT) cnt.tris++;
                        float bu, bv;
                        if (tri_hit(xyz(a), xyz(b), xyz(c), lo, ld, lt, bu, bv, no_cull)) {
                            h.prim = __float_as_uint(a.w);
                            h.u = bu; h.v = bv;
                            hit_here = true;
                            if (ANY) {
                                h.inst = ii;
                                h.t = lt;
                                return true;
                            }
                        }
                    }
                    if (bsp == 0) break;
                    uint2 e = bstack[--bsp];
                    first = e.x; count = e.y;
                    continue;
                }
                const float4* np = B.nodes + 2ull * first;
                float4 l0 = ldg4(np), l1 = ldg4(np + 1), q0 = ldg4(np + 2), q1 = ldg4(np + 3);
                if (COUNT) cnt.blas_nodes += 2;
                float dl = slab(xyz(l0), xyz(l1), lo, linv, lt);
                float dr = slab(xyz(q0), xyz(q1), lo, linv, lt);
                uint2 L = make_uint2(__float_as_uint(l0.w), __float_as_uint(l1.w));
                uint2 R = make_uint2(__float_as_uint(q0.w), __float_as_uint(q1.w));
                if (dl > dr) {
                    float td = dl; dl = dr; dr = td;
                    uint2 tn = L; L = R; R = tn;
                }
                if (dl == FLT_MAX) {
                    if (bsp == 0) break;
                    uint2 e = bstack[--bsp];
                    first = e.x; count = e.y;
                } else {
                    first = L.x; count = L.y;
                    if (dr != FLT_MAX) {
                        if (bsp == kStack) {
                            h.inst = kInvalid; h.prim = kInvalid; h.t = FLT_MAX; h.u = 0.0f; h.v = 0.0f;
                            return false;
                        }
                        bstack[bsp++] = R;
                    }
                }
            }
            t = lt;
            if (hit_here) { h.inst = ii; h.t = t; }
            if (tsp == 0) break;
            uint2 e = tstack[--tsp];
            lr = e.x; ii = e.y;
            continue;
        }
        const float4* ap = S.tnodes + 2ull * (lr >> 16);
        const float4* bp = S.tnodes + 2ull * (lr & 0xFFFFu);
        float4 a0 = ldg4(ap), a1 = ldg4(ap + 1), b0 = ldg4(bp), b1 = ldg4(bp + 1);
        if (COUNT) cnt.tlas_nodes += 2;
        float dl = slab(xyz(a0), xyz(a1), o, inv, t);
        float dr = slab(xyz(b0), xyz(b1), o, inv, t);
        uint2 L = make_uint2(__float_as_uint(a0.w), __float_as_uint(a1.w));
        uint2 R = make_uint2(__float_as_uint(b0.w), __float_as_uint(b1.w));
        if (dl > dr) {
            float td = dl; dl = dr; dr = td;
            uint2 tn = L; L = R; R = tn;
        }
        if (dl == FLT_MAX) {
            if (tsp == 0) break;
            uint2 e = tstack[--tsp];
            lr = e.x; ii = e.y;
        } else {
            lr = L.x; ii = L.y;
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

}  // namespace wf
