// wf_device.cuh — device-side layouts and exact-order float helpers.
//
// Every kernel is compiled with --fmad=false, -prec-div=true and
// -prec-sqrt=true, so a*b+c rounds twice, x/y and sqrtf are correctly
// rounded, and expressions evaluate in the order written.  The helpers below
// fix that order (dot = (ax*bx + ay*by) + az*bz, and so on); the CPU oracle
// performs the same operations, which is what makes hit ids, t values and
// per-path radiance bit-identical between the two.
#pragma once
#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

namespace wf {

// ---------------------------------------------------------------- layouts in HBM
//
// BLAS (one per mesh), traversal side:
//   nodes : 2 x float4 per node, the reference's 32-byte bvh_node_t verbatim
//           {min.xyz, left_first} {max.xyz, prim_count}; node 1 is unused so a
//           child pair (2k, 2k+1) is one 64-byte aligned line.
//   tris  : 3 x float4 per triangle in leaf order (position i of the index
//           list): {v0.xyz, original index} {e1 = v1-v0} {e2 = v2-v0}; e1 and
//           e2 are the exact differences Moeller-Trumbore forms first, so
//           storing them changes no result and removes the index indirection.
// TLAS:
//   tnodes: the reference's 32-byte tlas_node_t verbatim.
//   tinst : 4 x float4 per instance: world_to_local columns m[0..2], m[4..6],
//           m[8..10], m[12..14] (the only entries the transform reads), with
//           the mesh id in the first .w.
// Shading side, per mesh: stri = 6 x float4 per triangle in original order
//   {p0, u0} {p1, v0} {p2, u1} {n0, v1} {n1, u2} {n2, v2} (vertex uv in .w).
// Shading side, per instance: sinst = kInstRows (7) x float4
//   {l2w m[0..2], mesh} {m[4..6], bsdf} {m[8..10], ior} {m[12..14], roughness}
//   {base rgb, metallic} {emissive rgb (strength*factor), strength}
//   {texture ids: base colour, normal, metallic-roughness, emissive (0 = default)}
// Textures: RGBA float texels, row-major, row 0 at v = 0.

struct BlasRef {
    const float4* nodes;
    const float4* tris;
    uint32_t node_count, tri_count;   // read by checked builds only
    // the 4-wide layouts (wf_init_params.blas_layout = 1 / 2; csrc/wf_qbvh.cu):
    // 4 (quantized) or 8 (exact) float4 per node; root_count = the triangles of
    // a BLAS that is one leaf
    const float4* qnodes = nullptr;
    uint32_t qnode_count = 0, root_count = 0;
};

struct SceneRefs {
    const float4* tnodes;      // TLAS nodes
    const float4* tinst;       // TLAS instances
    const BlasRef* blas;       // indexed by mesh id
    uint32_t inst_count;
    uint32_t tnode_count, mesh_count;   // checked builds: bounds of the indices above
    uint32_t* status;                   // checked builds: where ERRF_BOUNDS is raised
    uint32_t qbvh = 0;                  // BLAS layout: 1 / 2 = the quantized / exact 4-wide nodes, tie rule
};

constexpr int kInstRows = 7;   // float4 rows per instance in the shading table

// Knuth's TwoSum: s = fl(a + b) and e with a + b = s + e exactly (IEEE
// arithmetic without contraction, as this library is compiled).
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
    const float s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
    return s;
}

struct LightTri {
    float4 p0;   // .w = area
    float4 e1;   // .w = running area sum (cdf)
    float4 e2;
    float4 n;    // unit geometric normal, .w = instance index (bits)
    float4 le;   // emitted radiance (strength * factor), .w = emissive texture id (bits)
    float4 uv01; // vertex uv {u0, v0, u1, v1}
    float4 uv2;  // {u2, v2, -, -}
};

struct TexRef {
    const float4* texels;   // nullptr: no texture
    uint32_t w, h;
};

struct Counters {
    unsigned long long tlas_node_loads, instance_loads, blas_node_loads, triangle_tests;
};

// Device error flags (bit set in the context's status word).
enum : uint32_t { ERRF_STACK = 1u, ERRF_CAPACITY = 2u, ERRF_TIMEOUT = 4u, ERRF_BOUNDS = 8u };

// Checked builds (-DWF_CHECKED=1, libwf_checked.so): every index a kernel
// takes from memory (a node's children, a leaf's triangles, an instance, a
// mesh, a hit's primitive, a texture, a path, a queue slot) is compared with
// the size of what it indexes before the access.  A bad index raises
// ERRF_BOUNDS in the status word (WF_ERR_BOUNDS from the next synchronising
// call) and the access is skipped: the ray reports a miss, the path ends,
// the write is dropped.  Normal builds compile the checks away.  It takes the
// place of compute-sanitizer, which this deployment cannot run: the GPU
// parity suite runs a second time against the checked library.
#ifndef WF_CHECKED
#define WF_CHECKED 0
#endif
__device__ __forceinline__ bool in_bounds(uint64_t i, uint64_t n, uint32_t* status) {
#if WF_CHECKED
    if (i < n) return true;
    if (status) atomicOr(status, ERRF_BOUNDS);
    return false;
#else
    (void)i; (void)n; (void)status;
    return true;
#endif
}

constexpr int kStack = 64;                 // per level, as the reference (accelstruct.hlsl:64,160)
constexpr float kEps = 1e-8f;              // SMALL_FLOAT (common.hlsl:8)
constexpr float kPi = 3.14159265f;         // PI (common.hlsl:20)
constexpr float kInvPi = 0.31830988f;      // INV_PI
constexpr float kInvTwoPi = 0.15915494f;   // INV_TWO_PI
constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// ---------------------------------------------------------------- vector helpers
struct V3 { float x, y, z; };

__host__ __device__ __forceinline__ V3 mk(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
__host__ __device__ __forceinline__ V3 xyz(float4 a) { return mk(a.x, a.y, a.z); }
__host__ __device__ __forceinline__ V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 sub(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 mul(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ V3 scl(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ V3 neg(V3 a) { return mk(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ V3 normalize(V3 v) { float s = 1.0f / sqrtf(dot(v, v)); return scl(v, s); }
__host__ __device__ __forceinline__ V3 rcp(V3 v) { return mk(1.0f / v.x, 1.0f / v.y, 1.0f / v.z); }

// HLSL mul(float4(v, w), M) with row-major packing (= glm M*v):
// out_j = ((v.x*m[j] + v.y*m[4+j]) + v.z*m[8+j]) + w*m[12+j]; the matrix is
// given as its four column-triples c0 = m[0..2], c1 = m[4..6], ...
__host__ __device__ __forceinline__ V3 xform(V3 v, float w, float4 c0, float4 c1, float4 c2, float4 c3) {
    return mk(v.x * c0.x + v.y * c1.x + v.z * c2.x + w * c3.x,
              v.x * c0.y + v.y * c1.y + v.z * c2.y + w * c3.y,
              v.x * c0.z + v.y * c1.z + v.z * c2.z + w * c3.z);
}

// ---------------------------------------------------------------- random numbers
// wang_hash / rand_float (common.hlsl:79-97).
__host__ __device__ __forceinline__ uint32_t wang_hash(uint32_t s) {
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}
__host__ __device__ __forceinline__ float rand_float(uint32_t& s) {
    s = wang_hash(s);
    return (float)s * 2.3283064365387e-10f;
}
// Per-path stream keyed by (pixel, sample, depth) instead of the reference's
// frame_seed + compacted queue index (shade.hlsl:80), so paths replay exactly.
__host__ __device__ __forceinline__ uint32_t path_seed(uint32_t frame_seed, uint32_t pixel, uint32_t sample,
                                                       uint32_t depth) {
    uint32_t s = frame_seed + pixel;
    s = wang_hash(s) ^ (sample * 0x9E3779B9u);
    s = wang_hash(s) ^ (depth * 0x85EBCA6Bu);
    return s;
}

// sin(phi), cos(phi): Cody-Waite reduction by pi/2 with a three-part
// constant (1.5703125 + 4.838268e-4 + 2.563344e-12; k times the first two
// parts is exact while |k| <= 4), k = rint(phi * 2/pi), x = phi - k*pi/2;
// truncated Taylor series in Horner form (sin to x^9, cos to x^10; truncation
// error < 2e-9 on [-pi/4, pi/4]), then a quarter-turn rotation by k mod 4.
// Absolute error against sin/cos of the same float phi < 1e-7 on [0, 2*pi].
__host__ __device__ __forceinline__ void sincos_rad(float phi, float& s_out, float& c_out) {
    float k = rintf(phi * 0.636619747f);
    float x = phi - k * 1.5703125f;
    x = x - k * 4.83826792e-4f;
    x = x - k * 2.56334415e-12f;
    float x2 = x * x;
    float sp = -1.98412698e-4f + x2 * 2.75573192e-6f;
    sp = 8.33333377e-3f + x2 * sp;
    sp = -1.66666672e-1f + x2 * sp;
    float sn = x + (x * x2) * sp;
    float cp = 2.48015876e-5f + x2 * -2.75573188e-7f;
    cp = -1.38888892e-3f + x2 * cp;
    cp = 4.16666679e-2f + x2 * cp;
    cp = -0.5f + x2 * cp;
    float cs = 1.0f + x2 * cp;
    int q = ((int)k) & 3;
    if (q == 0) { s_out = sn; c_out = cs; }
    else if (q == 1) { s_out = cs; c_out = -sn; }
    else if (q == 2) { s_out = -sn; c_out = -cs; }
    else { s_out = -cs; c_out = sn; }
}

// The hemisphere samplers' angle (sample.hlsl:29-54): phi = 2.0 * PI * r.y
// with PI = 3.14159265, i.e. the float 6.28318548 times r rounded to float,
// then sin(phi) and cos(phi).
__host__ __device__ __forceinline__ void sincos_2pi(float r, float& s_out, float& c_out) {
    sincos_rad(6.28318548f * r, s_out, c_out);
}

// ---------------------------------------------------------------- intersection
// intersect_ray_aabb (intersect.hlsl:53-76): fminf/fmaxf are IEEE
// minNum/maxNum, as HLSL min/max.
__device__ __forceinline__ float slab(V3 bmn, V3 bmx, V3 o, V3 inv, float t) {
    float tx1 = (bmn.x - o.x) * inv.x, tx2 = (bmx.x - o.x) * inv.x;
    float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
    float ty1 = (bmn.y - o.y) * inv.y, ty2 = (bmx.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(ty1, ty2));
    tmax = fminf(tmax, fmaxf(ty1, ty2));
    float tz1 = (bmn.z - o.z) * inv.z, tz2 = (bmx.z - o.z) * inv.z;
    tmin = fmaxf(tmin, fminf(tz1, tz2));
    tmax = fminf(tmax, fmaxf(tz1, tz2));
    return (tmax >= tmin && tmin < t && tmax > 0.0f) ? tmin : FLT_MAX;
}

// The slab test of the order-independent tie rule (closest-hit rays over the
// quantized layout): a box entered at exactly the current t is still visited,
// since it may hold an equal-t hit with a smaller (instance, primitive).
__device__ __forceinline__ float slab_le(V3 bmn, V3 bmx, V3 o, V3 inv, float t) {
    float tx1 = (bmn.x - o.x) * inv.x, tx2 = (bmx.x - o.x) * inv.x;
    float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
    float ty1 = (bmn.y - o.y) * inv.y, ty2 = (bmx.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(ty1, ty2));
    tmax = fminf(tmax, fmaxf(ty1, ty2));
    float tz1 = (bmn.z - o.z) * inv.z, tz2 = (bmx.z - o.z) * inv.z;
    tmin = fmaxf(tmin, fminf(tz1, tz2));
    tmax = fminf(tmax, fmaxf(tz1, tz2));
    return (tmax >= tmin && tmin <= t && tmax > 0.0f) ? tmin : FLT_MAX;
}

// intersect_ray_triangle (intersect.hlsl:7-51) on a pre-differenced triangle.
__device__ __forceinline__ bool tri_hit(V3 v0, V3 e1, V3 e2, V3 o, V3 d, float& t_io, float& bu, float& bv,
                                        bool no_cull) {
    V3 pvec = cross(d, e2);
    float det = dot(e1, pvec);
    if (no_cull ? (fabsf(det) < kEps) : (det < kEps)) return false;
    float inv_det = 1.0f / det;
    V3 tvec = sub(o, v0);
    float v = dot(tvec, pvec) * inv_det;
    if (v < 0.0f || v > 1.0f) return false;
    V3 qvec = cross(tvec, e1);
    float w = dot(d, qvec) * inv_det;
    if (w < 0.0f || v + w > 1.0f) return false;
    float t = dot(e2, qvec) * inv_det;
    if (t < 0.0f || t >= t_io) return false;
    t_io = t; bu = v; bv = w;
    return true;
}

// The same test under the tie rule: a hit at exactly t_io is taken when
// tie_wins (its (instance, primitive) is smaller than the current hit's).
__device__ __forceinline__ bool tri_hit_tie(V3 v0, V3 e1, V3 e2, V3 o, V3 d, float& t_io, float& bu, float& bv,
                                            bool no_cull, bool tie_wins) {
    V3 pvec = cross(d, e2);
    float det = dot(e1, pvec);
    if (no_cull ? (fabsf(det) < kEps) : (det < kEps)) return false;
    float inv_det = 1.0f / det;
    V3 tvec = sub(o, v0);
    float v = dot(tvec, pvec) * inv_det;
    if (v < 0.0f || v > 1.0f) return false;
    V3 qvec = cross(tvec, e1);
    float w = dot(d, qvec) * inv_det;
    if (w < 0.0f || v + w > 1.0f) return false;
    float t = dot(e2, qvec) * inv_det;
    if (t < 0.0f || t > t_io || (t == t_io && !tie_wins)) return false;
    t_io = t; bu = v; bv = w;
    return true;
}

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// ---------------------------------------------------------------- textures
// Texture slots of material_t and the values of the reference's default
// textures (renderer.cpp:244-272): base colour / emissive white, normal
// RGBA8 (127, 127, 255, 255), metallic-roughness RG8 (255, 255) read as
// (1, 1, 0, 1).
enum : uint32_t { TEX_BASE = 0, TEX_NORMAL = 1, TEX_METAL_ROUGH = 2, TEX_EMISSIVE = 3 };
__host__ __device__ __forceinline__ float4 tex_default(uint32_t slot) {
    if (slot == TEX_NORMAL) return make_float4(127.0f / 255.0f, 127.0f / 255.0f, 1.0f, 1.0f);
    if (slot == TEX_METAL_ROUGH) return make_float4(1.0f, 1.0f, 0.0f, 1.0f);
    return make_float4(1.0f, 1.0f, 1.0f, 1.0f);
}

// Wrap addressing of an integral float coordinate; out-of-range or
// non-finite coordinates read texel 0.
__host__ __device__ __forceinline__ uint32_t wrap_texel(float f, uint32_t n) {
    if (!(f > -16777216.0f && f < 16777216.0f)) return 0u;
    int m = ((int)f) % (int)n;
    if (m < 0) m += (int)n;
    return (uint32_t)m;
}

__host__ __device__ __forceinline__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }

// Sample(sampler_linear_wrap, uv) (material.hlsl:20-36) at the top level: texel
// centres at (i + 0.5) / w, wrap addressing, bilinear weights in FP32 (the
// hardware filter's weights have 8 fractional bits; these are exact).
__device__ __forceinline__ float4 tex_bilinear(const TexRef& t, float u, float v) {
    const float x = u * (float)t.w - 0.5f, y = v * (float)t.h - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float ax = x - x0, ay = y - y0;
    const uint32_t i0 = wrap_texel(x0, t.w), i1 = wrap_texel(x0 + 1.0f, t.w);
    const uint32_t j0 = wrap_texel(y0, t.h), j1 = wrap_texel(y0 + 1.0f, t.h);
    const float4 a = ldg4(t.texels + (size_t)j0 * t.w + i0), b = ldg4(t.texels + (size_t)j0 * t.w + i1);
    const float4 c = ldg4(t.texels + (size_t)j1 * t.w + i0), d = ldg4(t.texels + (size_t)j1 * t.w + i1);
    float4 r;
    r.x = lerpf(lerpf(a.x, b.x, ax), lerpf(c.x, d.x, ax), ay);
    r.y = lerpf(lerpf(a.y, b.y, ax), lerpf(c.y, d.y, ax), ay);
    r.z = lerpf(lerpf(a.z, b.z, ax), lerpf(c.z, d.z, ax), ay);
    r.w = lerpf(lerpf(a.w, b.w, ax), lerpf(c.w, d.w, ax), ay);
    return r;
}

// ---------------------------------------------------------------- inverse trigonometry
// Our own arctangent: on [0, 1], arguments above tan(pi/8) are reduced by
// atan z = pi/4 + atan((z - 1) / (z + 1)); on |z| <= tan(pi/8) the Taylor series
// z - z^3/3 + ... - z^15/15 + z^17/17 (truncation error < 3e-9) in Horner form.
__host__ __device__ __forceinline__ float atan_unit(float z) {
    float off = 0.0f;
    if (z > 0.41421357f) {
        z = (z - 1.0f) / (z + 1.0f);
        off = 0.78539819f;
    }
    const float t2 = z * z;
    float p = 0.05882353f;             // 1/17
    p = 0.06666667f - t2 * p;          // 1/15
    p = 0.07692308f - t2 * p;          // 1/13
    p = 0.09090909f - t2 * p;          // 1/11
    p = 0.11111111f - t2 * p;          // 1/9
    p = 0.14285715f - t2 * p;          // 1/7
    p = 0.2f - t2 * p;                 // 1/5
    p = 0.33333334f - t2 * p;          // 1/3
    p = 1.0f - t2 * p;
    return off + z * p;
}
// atan2 by octant: the smaller of |y|/|x|, |x|/|y| goes to atan_unit.
__host__ __device__ __forceinline__ float atan2_wf(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f) return 0.0f;
    float a = (ay <= ax) ? atan_unit(ay / ax) : 1.57079637f - atan_unit(ax / ay);
    if (x < 0.0f) a = 3.14159274f - a;
    return (y < 0.0f) ? -a : a;
}
__host__ __device__ __forceinline__ float asin_wf(float y) {
    return atan2_wf(y, sqrtf(fmaxf(0.0f, (1.0f - y) * (1.0f + y))));
}

// sample_hdr_env (shade.hlsl:36-40): direction_to_equirect_uv
// (sample.hlsl:4-11, INV_ATAN = (0.1591, 0.3183)) scaled to texels and
// truncated; a texel position outside the image reads zero, as an
// out-of-range Texture2D load does.
__device__ __forceinline__ V3 env_texel(const TexRef& e, V3 d) {
    const float u = atan2_wf(d.z, d.x) * 0.1591f + 0.5f;
    const float v = asin_wf(-d.y) * 0.3183f + 0.5f;
    const float fx = u * (float)e.w, fy = v * (float)e.h;
    if (!(fx >= 0.0f && fx < (float)e.w && fy >= 0.0f && fy < (float)e.h)) return mk(0.0f, 0.0f, 0.0f);
    return xyz(ldg4(e.texels + (size_t)(uint32_t)fy * e.w + (uint32_t)fx));
}

// int_to_color (common.hlsl:276-295).
__host__ __device__ __forceinline__ uint32_t murmur_mix(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
__host__ __device__ __forceinline__ V3 int_to_color(uint32_t v) {
    const uint32_t h = murmur_mix(v);
    const float k = 1.0f / 255.0f;
    return mk((float)(h & 255u) * k, (float)((h >> 8) & 255u) * k, (float)((h >> 16) & 255u) * k);
}

}  // namespace wf
