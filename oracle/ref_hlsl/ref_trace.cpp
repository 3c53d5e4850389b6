/*
 * ref_trace.cpp — the reference's software ray query, compiled from its own
 * shader text: source/renderer/shaders/accelstruct.hlsl:6-218 (TLAS and BLAS
 * stack walks, instance transform), intersect.hlsl:7-76 (Moeller-Trumbore,
 * slab test) and common.hlsl (constants, RNG, hit records) with
 * RAYTRACING_MODE_SOFTWARE = 1, as the megakernel build compiles them
 * (renderer.cpp:368-376).
 *
 * TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into
 * oracle/_ref/libref_hlsl.so where the reference checkout exists; the tests
 * compare the oracle (oracle/orc_impl.h) with it.
 *
 * The one piece of glue that is not reference text: extend.hlsl hands a
 * RayDesc2 (origin, TMin, direction, TMax) to the hardware ray query, while
 * the software walk takes a ray_t (origin, direction, inv_dir, t).  The bridge
 * here sets inv_dir = 1.0f / direction (as make_ray does, common.hlsl:150)
 * and t = TMax, and keeps the origin; the software walk has no TMin (it
 * accepts 0 <= t, intersect.hlsl:43).  The oracle and the GPU library use
 * the same bridge.
 */
#include "hlsl_shim.h"

#define RAYTRACING_MODE_SOFTWARE 1
namespace ref_sw {
using namespace hlsl_shim;
#include "accelstruct.hlsl"
}  // namespace ref_sw

using namespace hlsl_shim;

static_assert(sizeof(ref_sw::RayDesc2) == 32 && sizeof(ref_sw::hit_result_t) == 20, "ABI layout");
static_assert(sizeof(ref_sw::bvh_node_t) == 32 && sizeof(ref_sw::bvh_instance_t) == 92, "ABI layout");
static_assert(sizeof(ref_sw::tlas_node_t) == 32 && sizeof(ref_sw::bvh_triangle_t) == 36, "ABI layout");

extern "C" {

/* Resource registration: one descriptor per heap slot (buffers: bytes;
 * textures: RGBA float texels).  The caller keeps the memory alive. */
int refh_set_buffer(uint32_t slot, void* data, uint32_t bytes) {
    if (slot >= kHeapSize) return -1;
    g_heap[slot] = descriptor{(uint8_t*)data, bytes, 0u, 0u};
    return 0;
}
int refh_set_texture(uint32_t slot, float* texels, uint32_t w, uint32_t h) {
    if (slot >= kHeapSize) return -1;
    g_heap[slot] = descriptor{(uint8_t*)texels, 16u * w * h, w, h};
    return 0;
}
void refh_clear_heap(void) {
    for (uint32_t i = 0; i < kHeapSize; ++i) g_heap[i] = descriptor{nullptr, 0u, 0u, 0u};
}

/* extend (extend.hlsl:25-40) with the software query: for each ray,
 * hit = make_hit_result(); trace_ray_tlas(tlas, ray, hit).  The TLAS blob is
 * the buffer in `tlas_slot`; each instance's BLAS is the buffer in the slot
 * named by its bvh_index (accelstruct.hlsl:143). */
int refh_trace(uint32_t tlas_slot, const void* rays, uint32_t n, void* hits) {
    if (tlas_slot >= kHeapSize) return -1;
    const ByteAddressBuffer tlas = ByteAddressBuffer::from(g_heap[tlas_slot]);
    for (uint32_t i = 0; i < n; ++i) {
        ref_sw::RayDesc2 rd;
        __builtin_memcpy((void*)&rd, (const uint8_t*)rays + 32ull * i, 32);
        ref_sw::ray_t ray{};
        ray.Origin = rd.Origin;
        ray.Direction = rd.Direction;
        ray.inv_dir = 1.0f / rd.Direction;
        ray.t = rd.TMax;
        ref_sw::hit_result_t hit = ref_sw::make_hit_result();
        ref_sw::trace_ray_tlas(tlas, ray, hit);
        __builtin_memcpy((uint8_t*)hits + 20ull * i, (const void*)&hit, 20);
    }
    return 0;
}

/* intersect_ray_triangle (intersect.hlsl:7-51) on its own: t_inout is the
 * ray's t on entry and the hit's t on a hit. */
int refh_intersect_triangle(const float v0[3], const float v1[3], const float v2[3], const float org[3],
                            const float dir[3], float* t_inout, float bary[2]) {
    ref_sw::ray_t ray{};
    ray.Origin = float3(org[0], org[1], org[2]);
    ray.Direction = float3(dir[0], dir[1], dir[2]);
    ray.inv_dir = 1.0f / ray.Direction;
    ray.t = *t_inout;
    float2 b(bary[0], bary[1]);
    bool hit = ref_sw::intersect_ray_triangle(float3(v0[0], v0[1], v0[2]), float3(v1[0], v1[1], v1[2]),
                                              float3(v2[0], v2[1], v2[2]), ray, b);
    *t_inout = ray.t;
    bary[0] = b.x;
    bary[1] = b.y;
    return hit ? 1 : 0;
}

/* intersect_ray_aabb (intersect.hlsl:53-76). */
float refh_intersect_aabb(const float bmin[3], const float bmax[3], const float org[3], const float inv_dir[3],
                          float t) {
    ref_sw::ray_t ray{};
    ray.Origin = float3(org[0], org[1], org[2]);
    ray.inv_dir = float3(inv_dir[0], inv_dir[1], inv_dir[2]);
    ray.t = t;
    return ref_sw::intersect_ray_aabb(float3(bmin[0], bmin[1], bmin[2]), float3(bmax[0], bmax[1], bmax[2]), ray);
}

/* wang_hash / rand_float (common.hlsl:79-97). */
uint32_t refh_wang_hash(uint32_t seed) { return ref_sw::wang_hash(seed); }
float refh_rand_float(uint32_t* seed) {
    uint32_t s = *seed;
    float r = ref_sw::rand_float(s);
    *seed = s;
    return r;
}

}  // extern "C"
