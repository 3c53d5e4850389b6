"""Runs the reference's own shader text on the CPU: oracle/_ref/libref_hlsl.so,
built by oracle/build_ref.sh from source/renderer/shaders/ (accelstruct.hlsl,
intersect.hlsl, common.hlsl, sample.hlsl, material.hlsl, brdf.hlsl,
wavefront/shade.hlsl) rewritten by oracle/ref_hlsl/hlsl_to_cpp.py and compiled
with oracle/ref_hlsl/hlsl_shim.h.  Test infrastructure only: the tests compare
the oracle with it.

Resources live in the shim's descriptor heap, one slot each: a BLAS blob in
the slot its bvh_index names (the mesh number), the TLAS blob, the
instance_data_t array, each mesh's triangle_t buffer, the environment, the
reference's default textures (renderer.cpp:244-272) and the scene's textures.
"""
import ctypes
import os

import numpy as np

from wavefrontpathtracing_gb300.abi import RenderSettings, hit_dtype, material_dtype, ptr, ray_dtype

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_hlsl.so")

SLOT_TLAS, SLOT_INSTANCES, SLOT_ENV = 7000, 7001, 7002
SLOT_WHITE, SLOT_NORMAL, SLOT_METAL_ROUGH = 7003, 7004, 7005
SLOT_TRIANGLES, SLOT_TEXTURES = 7100, 7600

instance_data_dtype = np.dtype([("local_to_world", "<f4", 16), ("world_to_local", "<f4", 16),
                                ("material", material_dtype), ("triangle_buffer_idx", "<u4")])
assert instance_data_dtype.itemsize == 184


class _Frame(ctypes.Structure):
    _fields_ = [("view", ctypes.c_void_p), ("settings", ctypes.c_void_p), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("frame_seed", ctypes.c_uint32), ("sample", ctypes.c_uint32),
                ("tlas_slot", ctypes.c_uint32), ("instances_slot", ctypes.c_uint32), ("env_slot", ctypes.c_uint32),
                ("env_width", ctypes.c_uint32), ("env_height", ctypes.c_uint32)]


_lib = None


def available():
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        from oracle import oracle as orc
        orc.lib()   # liborc.so: the shim's sin / cos / atan2 / asin / texture filter
        L = ctypes.CDLL(LIB)
        vp, u32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float
        L.refh_set_buffer.argtypes = [u32, vp, u32]
        L.refh_set_texture.argtypes = [u32, vp, u32, u32]
        L.refh_trace.argtypes = [u32, vp, u32, vp]
        L.refh_intersect_triangle.argtypes = [vp, vp, vp, vp, vp, ctypes.POINTER(f32), vp]
        L.refh_intersect_aabb.argtypes = [vp, vp, vp, vp, f32]
        L.refh_intersect_aabb.restype = f32
        L.refh_wang_hash.argtypes = [u32]
        L.refh_wang_hash.restype = u32
        L.refh_rand_float.argtypes = [ctypes.POINTER(u32)]
        L.refh_rand_float.restype = f32
        L.refh_primary_ray.argtypes = [vp, u32, u32, vp]
        L.refh_hemisphere_sample.argtypes = [vp, f32, f32, ctypes.c_int, vp]
        L.refh_int_to_color.argtypes = [u32, vp]
        L.refh_equirect_uv.argtypes = [vp, vp]
        L.refh_render.argtypes = [ctypes.POINTER(_Frame), vp, vp]
        _lib = L
    return _lib


class RefScene:
    """The reference's view of an oracle.Scene: its BLAS / TLAS blobs and an
    instance_data_t array built from its instances."""

    def __init__(self, scene, env_color=(0.0, 0.0, 0.0)):
        self.scene = scene
        self._keep = []
        L = lib()
        L.refh_clear_heap()
        for m, blob in enumerate(scene._blas):
            assert m < SLOT_TLAS
            L.refh_set_buffer(m, blob.ctypes.data, blob.nbytes)
        L.refh_set_buffer(SLOT_TLAS, scene._tlas.ctypes.data, scene._tlas.nbytes)
        for m, tris in enumerate(scene._tris):
            L.refh_set_buffer(SLOT_TRIANGLES + m, tris.ctypes.data, tris.nbytes)
        inst = np.zeros(len(scene._inst), dtype=instance_data_dtype)
        for k, src in enumerate(scene._inst):
            inst[k]["local_to_world"] = src["local_to_world"]
            inst[k]["world_to_local"] = src["world_to_local"]
            mat = src["material"].copy()
            for field, default in (("base_color_index", SLOT_WHITE), ("normal_index", SLOT_NORMAL),
                                   ("metallic_roughness_index", SLOT_METAL_ROUGH), ("emissive_index", SLOT_WHITE)):
                mat[field] = default if mat[field] == 0 else SLOT_TEXTURES + mat[field]
            inst[k]["material"] = mat
            inst[k]["triangle_buffer_idx"] = SLOT_TRIANGLES + src["mesh"]
        self.instances = inst
        L.refh_set_buffer(SLOT_INSTANCES, inst.ctypes.data, inst.nbytes)
        # the reference's default textures: white sRGB base colour / emission,
        # normal (127, 127, 255, 255) / 255, metallic-roughness RG8 (255, 255)
        self._white = np.ones((1, 1, 4), np.float32)
        self._normal = np.array([[[np.float32(127.0) / np.float32(255.0)] * 2 + [1.0, 1.0]]], np.float32)
        self._mr = np.array([[[1.0, 1.0, 0.0, 1.0]]], np.float32)
        for slot, t in ((SLOT_WHITE, self._white), (SLOT_NORMAL, self._normal), (SLOT_METAL_ROUGH, self._mr)):
            L.refh_set_texture(slot, t.ctypes.data, 1, 1)
        for i, t in enumerate(scene._textures):
            L.refh_set_texture(SLOT_TEXTURES + 1 + i, t.ctypes.data, t.shape[1], t.shape[0])
        if scene.c.env_texture:
            env = scene._textures[scene.c.env_texture - 1]
        else:
            env = np.array([[[env_color[0], env_color[1], env_color[2], 1.0]]], np.float32)
        self._env = np.ascontiguousarray(env, np.float32)
        L.refh_set_texture(SLOT_ENV, self._env.ctypes.data, self._env.shape[1], self._env.shape[0])

    def trace(self, rays):
        rays = np.ascontiguousarray(rays, dtype=ray_dtype)
        hits = np.zeros(len(rays), dtype=hit_dtype)
        assert lib().refh_trace(SLOT_TLAS, ptr(rays), len(rays), ptr(hits)) == 0
        return hits

    def render_sample(self, view, width, height, sample, max_bounces=4, frame_seed=1, cosine=1, env_strength=1.0,
                      view_mode=0):
        """One frame of the reference's wavefront loop in which every path is
        sample `sample` of its pixel; returns (energy RGBA h x w x 4, the nine
        ray counts)."""
        s = RenderSettings()
        s.use_wavefront_pathtracing, s.use_software_rt, s.render_view_mode = 1, 0, view_mode
        s.max_bounces, s.cosine_weighted_diffuse, s.accumulate, s.hdr_env_strength = max_bounces, cosine, 1, \
            env_strength
        f = _Frame(ctypes.cast(ctypes.pointer(view), ctypes.c_void_p), ctypes.cast(ctypes.pointer(s), ctypes.c_void_p),
                   width, height, frame_seed, sample, SLOT_TLAS, SLOT_INSTANCES, SLOT_ENV, self._env.shape[1],
                   self._env.shape[0])
        energy = np.zeros((height, width, 4), np.float32)
        counts = np.zeros(9, np.uint32)
        assert lib().refh_render(ctypes.byref(f), ptr(energy), ptr(counts)) == 0
        return energy, counts


def primary_rays(view, width, height):
    L = lib()
    out = np.zeros(width * height, dtype=ray_dtype)
    one = np.zeros(1, dtype=ray_dtype)
    for y in range(height):
        for x in range(width):
            L.refh_primary_ray(ctypes.byref(view), x, y, ptr(one))
            out[y * width + x] = one[0]
    return out


def intersect_triangle(v0, v1, v2, o, d, t=3.4e38):
    arr = [np.asarray(x, dtype=np.float32) for x in (v0, v1, v2, o, d)]
    tt = ctypes.c_float(t)
    bary = np.zeros(2, dtype=np.float32)
    hit = lib().refh_intersect_triangle(*[ptr(a) for a in arr], ctypes.byref(tt), ptr(bary))
    return hit, tt.value, bary


def intersect_aabb(bmin, bmax, o, inv, t):
    arr = [np.asarray(x, dtype=np.float32) for x in (bmin, bmax, o, inv)]
    return lib().refh_intersect_aabb(*[ptr(a) for a in arr], t)


def hemisphere_sample(n, r0, r1, cosine):
    out = np.zeros(3, np.float32)
    lib().refh_hemisphere_sample(ptr(np.asarray(n, np.float32)), r0, r1, int(cosine), ptr(out))
    return out
