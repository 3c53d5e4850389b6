/*
 * hlsl_shim.h — the HLSL vocabulary of the reference's compute shaders
 * (source/renderer/shaders/), written as C++ so that the shader files
 * themselves compile on the host after the mechanical rewrite of
 * oracle/ref_hlsl/hlsl_to_cpp.py.
 *
 * TEST INFRASTRUCTURE ONLY: it exists to run the reference's own traversal,
 * intersection, sampling and shading text on the CPU and pin the oracle's
 * restatement (oracle/orc_impl.h) to it.  The product never includes it.
 *
 * What this header defines, and so what the comparison does NOT pin:
 *  - vector / matrix types with the shaders' layouts (float3 = 12 bytes,
 *    float4x4 = 16 floats in memory order, read row by row as DXC's
 *    row-major packing does, shaders/.. d3d12_backend.cpp:558);
 *  - the order of the sums inside the intrinsics: dot = (x*x' + y*y') + z*z',
 *    mul(v, M)[c] = ((v0*M[0][c] + v1*M[1][c]) + v2*M[2][c]) + v3*M[3][c],
 *    normalize(v) = v * (1 / sqrt(dot(v, v))), lerp(x, y, s) = x + s*(y - x);
 *  - sin / cos / atan2 / asin: the oracle's own implementations (orc_sincos,
 *    orc_atan2, orc_asin in liborc.so), sqrt = IEEE square root, min / max =
 *    IEEE minNum / maxNum (fminf / fmaxf);
 *  - Texture2D.Sample: the oracle's FP32 bilinear filter with wrap addressing
 *    (the hardware's 8-bit filter weights are not reproducible);
 *  - FP32 storage for RWTexture2D (the reference allocates RGBA16F energy and
 *    throughput textures, renderer.cpp:470-480);
 *  - D3D's rule that a read outside a buffer or texture returns 0.
 * Everything else — control flow, operand order of every expression,
 * constants, tie rules, stacks, the shade stage's enqueue — is the
 * reference's own text.
 *
 * No <math.h> / <cmath> is included: the shaders' unqualified sqrt, min, max,
 * abs, sin, ... must resolve to the overloads below and to nothing else.
 */
#pragma once
#include <stdint.h>
#include <type_traits>

extern "C" {
struct hlsl_shim_texture { const float* texels; uint32_t w, h; };
void orc_sincos(float phi, float* s, float* c);
float orc_atan2(float y, float x);
float orc_asin(float y);
void orc_tex_sample(const hlsl_shim_texture* t, float u, float v, float out[4]);
}

namespace hlsl_shim {

typedef uint32_t uint;
template <class T>
using if_num = typename std::enable_if<std::is_arithmetic<T>::value, int>::type;

// ------------------------------------------------------------------ vectors
struct float2 {
    float x, y;
    float2() : x(0.0f), y(0.0f) {}
    template <class S, if_num<S> = 0> float2(S s) : x(float(s)), y(float(s)) {}
    template <class A, class B, if_num<A> = 0, if_num<B> = 0> float2(A a, B b) : x(float(a)), y(float(b)) {}
};

struct float3 {
    float x, y, z;
    float3() : x(0.0f), y(0.0f), z(0.0f) {}
    template <class S, if_num<S> = 0> float3(S s) : x(float(s)), y(float(s)), z(float(s)) {}
    template <class A, class B, class C, if_num<A> = 0, if_num<B> = 0, if_num<C> = 0>
    float3(A a, B b, C c) : x(float(a)), y(float(b)), z(float(c)) {}
    template <class S, if_num<S> = 0> float3(float2 v, S s) : x(v.x), y(v.y), z(float(s)) {}
};

// Swizzles of a float4: read as a float3 / float2, assignable from one.
template <int A, int B, int C>
struct swizzle3 {
    float v[4];
    operator float3() const { return float3(v[A], v[B], v[C]); }
    swizzle3& operator=(const float3& s) { v[A] = s.x; v[B] = s.y; v[C] = s.z; return *this; }
};
template <int A, int B>
struct swizzle2 {
    float v[4];
    operator float2() const { return float2(v[A], v[B]); }
    swizzle2& operator=(const float2& s) { v[A] = s.x; v[B] = s.y; return *this; }
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        swizzle3<0, 1, 2> xyz;
        swizzle3<0, 1, 2> rgb;
        swizzle2<0, 1> xy;
    };
    float4() { x = y = z = w = 0.0f; }
    template <class S, if_num<S> = 0> float4(S s) { x = y = z = w = float(s); }
    template <class A, class B, class C, class D, if_num<A> = 0, if_num<B> = 0, if_num<C> = 0, if_num<D> = 0>
    float4(A a_, B b_, C c_, D d_) { x = float(a_); y = float(b_); z = float(c_); w = float(d_); }
    template <class S, if_num<S> = 0> float4(float3 v, S s) { x = v.x; y = v.y; z = v.z; w = float(s); }
    template <class S, class T, if_num<S> = 0, if_num<T> = 0> float4(float2 v, S s, T t) {
        x = v.x; y = v.y; z = float(s); w = float(t);
    }
};

struct uint2 {
    uint x, y;
    uint2() : x(0u), y(0u) {}
    template <class A, class B, if_num<A> = 0, if_num<B> = 0> uint2(A a, B b) : x(uint(a)), y(uint(b)) {}
    uint2(float2 f) : x(uint(f.x)), y(uint(f.y)) {}   // HLSL float -> uint conversion (truncation)
    operator float2() const { return float2(x, y); }
};
struct uint3 {
    uint x, y, z;
    uint3() : x(0u), y(0u), z(0u) {}
    template <class A, class B, class C, if_num<A> = 0, if_num<B> = 0, if_num<C> = 0>
    uint3(A a, B b, C c) : x(uint(a)), y(uint(b)), z(uint(c)) {}
};
struct uint4 { uint x, y, z, w; };

// float3x3(a, b, c) has rows a, b, c (HLSL); float4x4 holds 16 floats in
// memory order, row r = m[4r .. 4r+3] under row-major packing.
struct float3x3 {
    float3 r0, r1, r2;
    float3x3() {}
    float3x3(float3 a, float3 b, float3 c) : r0(a), r1(b), r2(c) {}
};
struct float4x4 { float m[16]; };

static_assert(sizeof(float2) == 8 && sizeof(float3) == 12 && sizeof(float4) == 16, "vector layout");
static_assert(sizeof(uint2) == 8 && sizeof(float4x4) == 64, "vector layout");

// -------------------------------------------------------------- arithmetic
#define HS_VEC2_OPS(op)                                                                                  \
    inline float2 operator op(float2 a, float2 b) { return float2(a.x op b.x, a.y op b.y); }             \
    inline float2 operator op(float2 a, float s) { return float2(a.x op s, a.y op s); }                  \
    inline float2 operator op(float s, float2 b) { return float2(s op b.x, s op b.y); }                  \
    inline float2& operator op##=(float2& a, float2 b) { a = a op b; return a; }                         \
    inline float2& operator op##=(float2& a, float s) { a = a op s; return a; }
#define HS_VEC3_OPS(op)                                                                                  \
    inline float3 operator op(float3 a, float3 b) { return float3(a.x op b.x, a.y op b.y, a.z op b.z); } \
    inline float3 operator op(float3 a, float s) { return float3(a.x op s, a.y op s, a.z op s); }        \
    inline float3 operator op(float s, float3 b) { return float3(s op b.x, s op b.y, s op b.z); }        \
    inline float3& operator op##=(float3& a, float3 b) { a = a op b; return a; }                         \
    inline float3& operator op##=(float3& a, float s) { a = a op s; return a; }
#define HS_VEC4_OPS(op)                                                                                  \
    inline float4 operator op(float4 a, float4 b) {                                                      \
        return float4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w);                                   \
    }                                                                                                    \
    inline float4 operator op(float4 a, float s) { return float4(a.x op s, a.y op s, a.z op s, a.w op s); } \
    inline float4 operator op(float s, float4 b) { return float4(s op b.x, s op b.y, s op b.z, s op b.w); }
HS_VEC2_OPS(+) HS_VEC2_OPS(-) HS_VEC2_OPS(*) HS_VEC2_OPS(/)
HS_VEC3_OPS(+) HS_VEC3_OPS(-) HS_VEC3_OPS(*) HS_VEC3_OPS(/)
HS_VEC4_OPS(+) HS_VEC4_OPS(-) HS_VEC4_OPS(*) HS_VEC4_OPS(/)
#undef HS_VEC2_OPS
#undef HS_VEC3_OPS
#undef HS_VEC4_OPS
inline float2 operator-(float2 a) { return float2(-a.x, -a.y); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }

// -------------------------------------------------------------- intrinsics
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float abs(float x) { return __builtin_fabsf(x); }
inline float3 abs(float3 v) { return float3(abs(v.x), abs(v.y), abs(v.z)); }
inline float min(float a, float b) { return __builtin_fminf(a, b); }
inline float max(float a, float b) { return __builtin_fmaxf(a, b); }
inline float3 min(float3 a, float3 b) { return float3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float3 max(float3 a, float3 b) { return float3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float3 clamp(float3 v, float lo, float hi) { return float3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)); }
inline float sin(float x) { float s, c; orc_sincos(x, &s, &c); return s; }
inline float cos(float x) { float s, c; orc_sincos(x, &s, &c); return c; }
inline float atan2(float y, float x) { return orc_atan2(y, x); }
inline float asin(float y) { return orc_asin(y); }
inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float3 pow(float3 v, float y) { return float3(pow(v.x, y), pow(v.y, y), pow(v.z, y)); }
inline float step(float y, float x) { return x >= y ? 1.0f : 0.0f; }
inline float3 step(float3 y, float3 x) { return float3(step(y.x, x.x), step(y.y, x.y), step(y.z, x.z)); }
inline float3 step(float3 y, float x) { return float3(step(y.x, x), step(y.y, x), step(y.z, x)); }
inline float lerp(float x, float y, float s) { return x + s * (y - x); }
inline float3 lerp(float3 x, float3 y, float s) { return x + s * (y - x); }
inline float3 lerp(float3 x, float3 y, float3 s) { return x + s * (y - x); }
inline bool any(float3 v) { return v.x != 0.0f || v.y != 0.0f || v.z != 0.0f; }
inline bool isinf(float x) { return __builtin_isinf(x); }
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float3 normalize(float3 v) { float s = 1.0f / sqrt(dot(v, v)); return v * s; }
inline float4 mul(float4 v, const float4x4& M) {
    const float* m = M.m;
    float o[4];
    for (int c = 0; c < 4; ++c) o[c] = v.x * m[c] + v.y * m[4 + c] + v.z * m[8 + c] + v.w * m[12 + c];
    return float4(o[0], o[1], o[2], o[3]);
}
inline float3 mul(float3 v, const float3x3& M) {
    return float3(v.x * M.r0.x + v.y * M.r1.x + v.z * M.r2.x, v.x * M.r0.y + v.y * M.r1.y + v.z * M.r2.y,
                  v.x * M.r0.z + v.y * M.r1.z + v.z * M.r2.z);
}
inline float asfloat(uint u) { float f; __builtin_memcpy(&f, &u, 4); return f; }
inline float asfloat(int i) { return asfloat(uint(i)); }
inline uint asuint(float f) { uint u; __builtin_memcpy(&u, &f, 4); return u; }
inline uint asuint(uint u) { return u; }
inline uint asuint(int i) { return uint(i); }

// --------------------------------------------------------------- resources
// One descriptor: bytes of a buffer, or RGBA float texels of a texture.
struct descriptor {
    uint8_t* data;
    uint32_t bytes;
    uint32_t width, height;
};
constexpr uint32_t kHeapSize = 8192;
inline descriptor g_heap[kHeapSize];

struct SamplerState {};

struct ByteAddressBuffer {
    const uint8_t* p = nullptr;
    uint32_t n = 0;
    static ByteAddressBuffer from(const descriptor& d) { ByteAddressBuffer b; b.p = d.data; b.n = d.bytes; return b; }
    template <class T>
    T Load(uint32_t off) const {
        T v{};
        if (p && (uint64_t)off + sizeof(T) <= n) __builtin_memcpy((void*)&v, p + off, sizeof(T));
        return v;
    }
};
struct RWByteAddressBuffer {
    uint8_t* p = nullptr;
    uint32_t n = 0;
    static RWByteAddressBuffer from(const descriptor& d) { RWByteAddressBuffer b; b.p = d.data; b.n = d.bytes; return b; }
    template <class T>
    T Load(uint32_t off) const {
        T v{};
        if (p && (uint64_t)off + sizeof(T) <= n) __builtin_memcpy((void*)&v, p + off, sizeof(T));
        return v;
    }
    template <class T>
    void Store(uint32_t off, const T& v) const {
        if (p && (uint64_t)off + sizeof(T) <= n) __builtin_memcpy(p + off, (const void*)&v, sizeof(T));
    }
    void InterlockedAdd(uint32_t off, uint32_t value, uint32_t& original) const {
        uint32_t cur = Load<uint32_t>(off);
        original = cur;
        Store<uint32_t>(off, cur + value);
    }
};
struct Texture2D {
    const float* t = nullptr;
    uint32_t w = 0, h = 0;
    static Texture2D from(const descriptor& d) {
        Texture2D x;
        if (d.width && d.height) { x.t = (const float*)d.data; x.w = d.width; x.h = d.height; }
        return x;
    }
    float4 Sample(SamplerState, float2 uv) const {
        if (!t) return float4();
        hlsl_shim_texture tx{t, w, h};
        float o[4];
        orc_tex_sample(&tx, uv.x, uv.y, o);
        return float4(o[0], o[1], o[2], o[3]);
    }
    float4 operator[](uint2 p) const {
        if (!t || p.x >= w || p.y >= h) return float4();
        const float* q = t + 4 * ((uint64_t)p.y * w + p.x);
        return float4(q[0], q[1], q[2], q[3]);
    }
};
struct RWTexture2D {
    float* t = nullptr;
    uint32_t w = 0, h = 0;
    static RWTexture2D from(const descriptor& d) {
        RWTexture2D x;
        if (d.width && d.height) { x.t = (float*)d.data; x.w = d.width; x.h = d.height; }
        return x;
    }
    float4& operator[](uint2 p) const {
        static thread_local float4 outside;   // writes outside the texture are dropped, reads give 0
        if (!t || p.x >= w || p.y >= h) { outside = float4(); return outside; }
        return *reinterpret_cast<float4*>(t + 4 * ((uint64_t)p.y * w + p.x));
    }
};

// ResourceDescriptorHeap[i] converts to whichever resource type the shader asks for.
struct heap_entry {
    uint32_t i;
    template <class T>
    operator T() const { return T::from(i < kHeapSize ? g_heap[i] : descriptor{nullptr, 0, 0, 0}); }
};
struct descriptor_heap {
    heap_entry operator[](uint32_t i) const { return heap_entry{i}; }
};
inline descriptor_heap ResourceDescriptorHeap;
inline uint32_t NonUniformResourceIndex(uint32_t i) { return i; }

template <class T>
using ConstantBuffer = T;

// The DXR ray description (HLSL built-in), used by raydesc2_to_raydesc.
struct RayDesc {
    float3 Origin;
    float TMin;
    float3 Direction;
    float TMax;
};

}  // namespace hlsl_shim

// shared.hlsl.h names glm's types under __cplusplus; here they are the shim's.
namespace glm {
using vec2 = hlsl_shim::float2;
using vec3 = hlsl_shim::float3;
using vec4 = hlsl_shim::float4;
using uvec2 = hlsl_shim::uint2;
using uvec3 = hlsl_shim::uint3;
using uvec4 = hlsl_shim::uint4;
using mat3 = hlsl_shim::float3x3;
using mat4 = hlsl_shim::float4x4;
}  // namespace glm
