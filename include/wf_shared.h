/*
 * wf_shared.h — data layouts that cross the drop-in boundary.
 *
 * Every struct here has the byte layout of its counterpart in the reference's
 * CPU/GPU shared header (source/renderer/shaders/shared.hlsl.h:34-161), which
 * the reference compiles as C++ with glm types (float3 = glm::vec3, 12 bytes,
 * 4-byte aligned; float4x4 = glm::mat4, column-major, 64 bytes).  A caller that
 * already fills those structs can pass the same bytes to this library.
 *
 * Matrix convention: 16 floats, glm column-major (m[4*col + row]).  The
 * reference's HLSL packs matrices row-major, so its mul(float4(v,w), M) is the
 * glm product M * v; every kernel here evaluates it as
 * ((v.x*m[0+j] + v.y*m[4+j]) + v.z*m[8+j]) + w*m[12+j] without fused
 * multiply-add, which is the operation order the CPU oracle also uses.
 */
#ifndef WF_SHARED_H
#define WF_SHARED_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* RENDER_VIEW_MODE (shared.hlsl.h:17-32). */
enum wf_render_view_mode {
    RENDER_VIEW_MODE_NONE = 0,
    RENDER_VIEW_MODE_GEOMETRY_INSTANCE,
    RENDER_VIEW_MODE_GEOMETRY_PRIMITIVE,
    RENDER_VIEW_MODE_GEOMETRY_BARYCENTRICS,
    RENDER_VIEW_MODE_GEOMETRY_NORMAL,
    RENDER_VIEW_MODE_GEOMETRY_UV,
    RENDER_VIEW_MODE_MATERIAL_BASE_COLOR,
    RENDER_VIEW_MODE_MATERIAL_NORMAL,
    RENDER_VIEW_MODE_MATERIAL_METALLIC_ROUGHNESS,
    RENDER_VIEW_MODE_MATERIAL_EMISSIVE,
    RENDER_VIEW_MODE_WORLD_NORMAL,
    RENDER_VIEW_MODE_RENDER_TARGET_DEPTH,
    RENDER_VIEW_MODE_COUNT
};

/* render_settings_t (shared.hlsl.h:34-44), 28 bytes. */
typedef struct render_settings_t {
    uint32_t use_wavefront_pathtracing; /* 1 = wavefront stages, 0 = megakernel */
    uint32_t use_software_rt;           /* ignored: traversal is always software */
    uint32_t render_view_mode;          /* enum wf_render_view_mode */
    uint32_t max_bounces;               /* depth loop runs d = 0..max_bounces */
    uint32_t cosine_weighted_diffuse;   /* 1 = cosine, 0 = uniform hemisphere */
    uint32_t accumulate;                /* running average across wf_render calls */
    float    hdr_env_strength;
} render_settings_t;

/* view_t (shared.hlsl.h:46-56), 272 bytes. */
typedef struct view_t {
    float world_to_view[16];
    float view_to_world[16];
    float view_to_clip[16];
    float clip_to_view[16];
    float render_dim[2];
    float near_plane;
    float far_plane;
} view_t;

/* vertex_t (shared.hlsl.h:58-64), 48 bytes. */
typedef struct vertex_t {
    float position[3];
    float normal[3];
    float tangent[4];
    float uv[2];
} vertex_t;

/* triangle_t (shared.hlsl.h:66-71), 144 bytes. */
typedef struct triangle_t {
    vertex_t v0, v1, v2;
} triangle_t;

/* material_t (shared.hlsl.h:73-85), 52 bytes. */
typedef struct material_t {
    float    base_color_factor[3];
    float    metallic_factor;
    float    roughness_factor;
    float    emissive_factor[3];
    float    emissive_strength;
    uint32_t base_color_index;
    uint32_t normal_index;
    uint32_t metallic_roughness_index;
    uint32_t emissive_index;
} material_t;

/* instance_data_t (shared.hlsl.h:87-94), 184 bytes. */
typedef struct instance_data_t {
    float      local_to_world[16];
    float      world_to_local[16];
    material_t material;
    uint32_t   triangle_buffer_idx;
} instance_data_t;

/* bvh_header_t (shared.hlsl.h:99-104), 12 bytes. */
typedef struct bvh_header_t {
    uint32_t nodes_offset;
    uint32_t triangles_offset;
    uint32_t indices_offset;
} bvh_header_t;

/* bvh_node_t (shared.hlsl.h:106-112), 32 bytes.  prim_count > 0 marks a leaf
 * whose triangles are index-list entries [left_first, left_first+prim_count);
 * otherwise the children are nodes left_first and left_first+1. */
typedef struct bvh_node_t {
    float    aabb_min[3];
    uint32_t left_first;
    float    aabb_max[3];
    uint32_t prim_count;
} bvh_node_t;

/* bvh_triangle_t (shared.hlsl.h:114-119), 36 bytes. */
typedef struct bvh_triangle_t {
    float p0[3], p1[3], p2[3];
} bvh_triangle_t;

/* bvh_instance_t (shared.hlsl.h:121-127), 92 bytes. */
typedef struct bvh_instance_t {
    float    world_to_local[16];
    float    aabb_min[3];
    float    aabb_max[3];
    uint32_t bvh_index;
} bvh_instance_t;

/* tlas_header_t (shared.hlsl.h:129-133), 8 bytes. */
typedef struct tlas_header_t {
    uint32_t nodes_offset;
    uint32_t instances_offset;
} tlas_header_t;

/* tlas_node_t (shared.hlsl.h:135-142), 32 bytes.  left_right == 0 marks a
 * leaf; otherwise the children are (left_right >> 16) and (left_right & 0xFFFF). */
typedef struct tlas_node_t {
    float    aabb_min[3];
    uint32_t left_right;
    float    aabb_max[3];
    uint32_t instance_idx;
} tlas_node_t;

/* hit_result_t (shared.hlsl.h:144-150), 20 bytes.  0xFFFFFFFF ids = miss. */
typedef struct hit_result_t {
    uint32_t instance_idx;
    uint32_t primitive_idx;
    float    t;
    float    bary[2];
} hit_result_t;

/* RayDesc2 (shared.hlsl.h:155-161), 32 bytes. */
typedef struct RayDesc2 {
    float Origin[3];
    float TMin;
    float Direction[3];
    float TMax;
} RayDesc2;

#define WF_INVALID_INDEX 0xFFFFFFFFu

#if defined(__cplusplus) && __cplusplus >= 201103L
static_assert(sizeof(render_settings_t) == 28, "render_settings_t layout");
static_assert(sizeof(view_t) == 272, "view_t layout");
static_assert(sizeof(vertex_t) == 48, "vertex_t layout");
static_assert(sizeof(triangle_t) == 144, "triangle_t layout");
static_assert(sizeof(material_t) == 52, "material_t layout");
static_assert(sizeof(instance_data_t) == 184, "instance_data_t layout");
static_assert(sizeof(bvh_header_t) == 12, "bvh_header_t layout");
static_assert(sizeof(bvh_node_t) == 32, "bvh_node_t layout");
static_assert(sizeof(bvh_triangle_t) == 36, "bvh_triangle_t layout");
static_assert(sizeof(bvh_instance_t) == 92, "bvh_instance_t layout");
static_assert(sizeof(tlas_header_t) == 8, "tlas_header_t layout");
static_assert(sizeof(tlas_node_t) == 32, "tlas_node_t layout");
static_assert(sizeof(hit_result_t) == 20, "hit_result_t layout");
static_assert(sizeof(RayDesc2) == 32, "RayDesc2 layout");
#endif

#ifdef __cplusplus
}
#endif

#endif /* WF_SHARED_H */
