"""numpy dtypes and ctypes structs with the byte layouts of include/wf_shared.h.

These are the reference's CPU/GPU shared structs
(source/renderer/shaders/shared.hlsl.h:34-161); arrays of them are passed to the
C ABI as plain pointers.
"""
import ctypes

import numpy as np

f4, u4 = "<f4", "<u4"

vertex_dtype = np.dtype([("position", f4, 3), ("normal", f4, 3), ("tangent", f4, 4), ("uv", f4, 2)])
triangle_dtype = np.dtype([("v0", vertex_dtype), ("v1", vertex_dtype), ("v2", vertex_dtype)])
material_dtype = np.dtype([
    ("base_color_factor", f4, 3), ("metallic_factor", f4), ("roughness_factor", f4),
    ("emissive_factor", f4, 3), ("emissive_strength", f4),
    ("base_color_index", u4), ("normal_index", u4), ("metallic_roughness_index", u4), ("emissive_index", u4),
])
material_ext_dtype = np.dtype([("base", material_dtype), ("bsdf", u4), ("ior", f4)])
ray_dtype = np.dtype([("origin", f4, 3), ("tmin", f4), ("dir", f4, 3), ("tmax", f4)])
hit_dtype = np.dtype([("instance", u4), ("primitive", u4), ("t", f4), ("bary", f4, 2)])
bvh_instance_dtype = np.dtype([("world_to_local", f4, 16), ("aabb_min", f4, 3), ("aabb_max", f4, 3),
                               ("bvh_index", u4)])
bvh_node_dtype = np.dtype([("aabb_min", f4, 3), ("left_first", u4), ("aabb_max", f4, 3), ("prim_count", u4)])
tlas_node_dtype = np.dtype([("aabb_min", f4, 3), ("left_right", u4), ("aabb_max", f4, 3), ("instance_idx", u4)])

for _dt, _size in ((vertex_dtype, 48), (triangle_dtype, 144), (material_dtype, 52), (ray_dtype, 32),
                   (hit_dtype, 20), (bvh_instance_dtype, 92), (bvh_node_dtype, 32), (tlas_node_dtype, 32),
                   (material_ext_dtype, 60)):
    assert _dt.itemsize == _size, (_dt, _dt.itemsize, _size)

INVALID = 0xFFFFFFFF
BSDF_LAMBERT, BSDF_METAL, BSDF_DIELECTRIC = 0, 1, 2
# RENDER_VIEW_MODE (shared.hlsl.h:17-32)
(RENDER_VIEW_MODE_NONE, RENDER_VIEW_MODE_GEOMETRY_INSTANCE, RENDER_VIEW_MODE_GEOMETRY_PRIMITIVE,
 RENDER_VIEW_MODE_GEOMETRY_BARYCENTRICS, RENDER_VIEW_MODE_GEOMETRY_NORMAL, RENDER_VIEW_MODE_GEOMETRY_UV,
 RENDER_VIEW_MODE_MATERIAL_BASE_COLOR, RENDER_VIEW_MODE_MATERIAL_NORMAL, RENDER_VIEW_MODE_MATERIAL_METALLIC_ROUGHNESS,
 RENDER_VIEW_MODE_MATERIAL_EMISSIVE, RENDER_VIEW_MODE_WORLD_NORMAL, RENDER_VIEW_MODE_RENDER_TARGET_DEPTH) = range(12)
TRACE_ANY_HIT, TRACE_NO_CULL, TRACE_COUNT_TRAFFIC, TRACE_REORDER = 1, 2, 4, 8


class RenderSettings(ctypes.Structure):
    """render_settings_t (shared.hlsl.h:34-44)."""
    _fields_ = [("use_wavefront_pathtracing", ctypes.c_uint32), ("use_software_rt", ctypes.c_uint32),
                ("render_view_mode", ctypes.c_uint32), ("max_bounces", ctypes.c_uint32),
                ("cosine_weighted_diffuse", ctypes.c_uint32), ("accumulate", ctypes.c_uint32),
                ("hdr_env_strength", ctypes.c_float)]


class View(ctypes.Structure):
    """view_t (shared.hlsl.h:46-56); matrices are glm column-major."""
    _fields_ = [("world_to_view", ctypes.c_float * 16), ("view_to_world", ctypes.c_float * 16),
                ("view_to_clip", ctypes.c_float * 16), ("clip_to_view", ctypes.c_float * 16),
                ("render_dim", ctypes.c_float * 2), ("near_plane", ctypes.c_float),
                ("far_plane", ctypes.c_float)]


class InitParams(ctypes.Structure):
    _fields_ = [("render_width", ctypes.c_uint32), ("render_height", ctypes.c_uint32),
                ("backbuffer_count", ctypes.c_uint32), ("vsync", ctypes.c_uint32),
                ("device", ctypes.c_int32), ("wave_capacity", ctypes.c_uint32),
                ("tlas_metric", ctypes.c_uint32), ("blas_layout", ctypes.c_uint32),
                ("instance_bounds", ctypes.c_uint32)]


class BvhOptions(ctypes.Structure):
    _fields_ = [("interval_count", ctypes.c_uint32), ("subdivide_single_prim", ctypes.c_uint32),
                ("max_leaf_prims", ctypes.c_uint32)]


class Env(ctypes.Structure):
    _fields_ = [("color", ctypes.c_float * 3), ("texture", ctypes.c_uint32)]


TEXTURE_RGBA8, TEXTURE_RGBA8_SRGB, TEXTURE_RG8, TEXTURE_RGBA32F = 0, 1, 2, 3
(TEXTURE_BC1, TEXTURE_BC1_SRGB, TEXTURE_BC2, TEXTURE_BC2_SRGB, TEXTURE_BC3, TEXTURE_BC3_SRGB, TEXTURE_BC4,
 TEXTURE_BC5, TEXTURE_BC7, TEXTURE_BC7_SRGB) = range(4, 14)
SCHEDULE_SEPARATE, SCHEDULE_FUSED, SCHEDULE_SERIAL = 0, 1, 2


class RenderOptions(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint32), ("nee", ctypes.c_uint32), ("rr_start_depth", ctypes.c_uint32),
                ("wave_paths", ctypes.c_uint32), ("profile", ctypes.c_uint32),
                ("count_traffic", ctypes.c_uint32), ("trace_schedule", ctypes.c_uint32),
                ("tail_paths", ctypes.c_uint32), ("fused_from_depth", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("ms_total", ctypes.c_double), ("ms_generate", ctypes.c_double), ("ms_extend", ctypes.c_double),
                ("ms_shade", ctypes.c_double), ("ms_connect", ctypes.c_double), ("ms_post", ctypes.c_double),
                ("ms_tlas_build", ctypes.c_double),
                ("launches", ctypes.c_uint64), ("launches_extend", ctypes.c_uint64),
                ("launches_connect", ctypes.c_uint64), ("rays_extend", ctypes.c_uint64),
                ("rays_connect", ctypes.c_uint64), ("paths", ctypes.c_uint64),
                ("tlas_node_loads", ctypes.c_uint64), ("instance_loads", ctypes.c_uint64),
                ("blas_node_loads", ctypes.c_uint64), ("triangle_tests", ctypes.c_uint64),
                ("shadow_tlas_node_loads", ctypes.c_uint64), ("shadow_instance_loads", ctypes.c_uint64),
                ("shadow_blas_node_loads", ctypes.c_uint64), ("shadow_triangle_tests", ctypes.c_uint64),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("extend_rays_depth", ctypes.c_uint64 * 16), ("shadow_rays_depth", ctypes.c_uint64 * 16),
                ("ms_tail", ctypes.c_double), ("tail_depth", ctypes.c_uint64),
                ("ms_extend_depth", ctypes.c_double * 16), ("ms_connect_depth", ctypes.c_double * 16),
                ("extend_fetch_depth", (ctypes.c_uint64 * 4) * 16), ("shadow_fetch_depth", (ctypes.c_uint64 * 4) * 16)]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_}
        for k in ("extend_rays_depth", "shadow_rays_depth", "ms_extend_depth", "ms_connect_depth"):
            d[k] = list(getattr(self, k))
        for k in ("extend_fetch_depth", "shadow_fetch_depth"):
            d[k] = [list(row) for row in getattr(self, k)]
        return d


class BatchConfig(ctypes.Structure):
    _fields_ = [("capacity", ctypes.c_uint32), ("regen_threshold", ctypes.c_float), ("block", ctypes.c_uint32),
                ("use_graph", ctypes.c_uint32), ("max_iterations", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 3)]

    def as_dict(self):
        return {"capacity": self.capacity, "regen_threshold": round(self.regen_threshold, 6), "block": self.block,
                "use_graph": self.use_graph, "max_iterations": self.max_iterations}


class BatchStats(ctypes.Structure):
    _fields_ = [("ms_total", ctypes.c_double), ("paths", ctypes.c_uint64), ("rays_extend", ctypes.c_uint64),
                ("rays_connect", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("iterations", ctypes.c_uint32), ("graph_launches", ctypes.c_uint32), ("scenes", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32 * 3)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


assert ctypes.sizeof(RenderSettings) == 28 and ctypes.sizeof(View) == 272
assert ctypes.sizeof(BatchConfig) == 32 and ctypes.sizeof(BatchStats) == 64
assert ctypes.sizeof(Stats) == 1736   # wf_stats


def ptr(a):
    """ctypes void pointer to a contiguous numpy array (None for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return ctypes.c_void_p(a.ctypes.data)


def mat_f32(m):
    """4x4 numpy matrix (row-major math convention, M @ v) -> 16 floats, glm column-major."""
    m = np.asarray(m, dtype=np.float32)
    return np.ascontiguousarray(m.T).reshape(16)
