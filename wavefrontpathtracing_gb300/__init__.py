"""GB300 wavefront path tracer: Python binding of the C ABI (include/wf.h).

The compute path is libwf.so (hand-written CUDA for sm_103a plus the C++ host
orchestration).  This module only loads it with ctypes and mirrors the
reference renderer's front end (source/renderer/renderer.h:13-55):

    r = Renderer(width, height)
    mesh = r.create_render_mesh(vertices, indices)      # create_render_mesh
    r.begin_scene(view)                                  # begin_scene
    r.submit_render_mesh(mesh, transform, material)      # submit_render_mesh
    r.end_scene()                                        # TLAS build
    r.render(settings, spp=16)                           # render
    img = r.read_image()

There is no CPU fallback: if libwf.so is missing or no CUDA device exists the
calls raise WFError.
"""
import ctypes
import os
import weakref

import numpy as np

from . import abi
from .abi import (BatchConfig, BatchStats, BvhOptions, Env, InitParams, RenderOptions, RenderSettings, Stats, View,
                  bvh_instance_dtype,
                  hit_dtype, material_dtype, material_ext_dtype, ptr, ray_dtype, triangle_dtype, vertex_dtype)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libwf.so")
# WF_LIBRARY names another build of the library (the bounds-checked
# _lib/libwf_checked.so); it must exist, nothing falls back to another build.
LIB_ENV = "WF_LIBRARY"

STATUS = {0: "WF_OK", -1: "WF_ERR_INVALID", -2: "WF_ERR_OOM", -3: "WF_ERR_CAPACITY", -4: "WF_ERR_TIMEOUT",
          -5: "WF_ERR_STACK", -6: "WF_ERR_CUDA", -7: "WF_ERR_STATE", -8: "WF_ERR_BOUNDS"}

# Every entry point declared in include/wf.h, with its ctypes signature.
_vp, _u32, _u64, _i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
_pu64, _pu32 = ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32)
SIGNATURES = {
    "wf_create": [_vp, ctypes.POINTER(_vp)],
    "wf_destroy": [_vp],
    "wf_status_string": [ctypes.c_int],
    "wf_last_error": [],
    "wf_abi_version": [],
    "wf_checked_build": [],
    "wf_set_device_memory_limit": [_u64],
    "wf_get_device_memory_usage": [_pu64],
    "wf_get_stream": [_vp, ctypes.POINTER(_vp)],
    "wf_synchronize": [_vp],
    "wf_mesh_create": [_vp, _vp, _u32, _vp, _u32, _vp, _pu32],
    "wf_mesh_create_prebuilt": [_vp, _vp, _u32, _vp, _u64, _pu32],
    "wf_mesh_get_blas": [_vp, _u32, _vp, _pu64],
    "wf_scene_begin": [_vp, _vp, _vp],
    "wf_instance_submit": [_vp, _u32, _vp, _vp],
    "wf_instance_submit_ex": [_vp, _u32, _vp, _vp],
    "wf_instance_submit_many": [_vp, _u32, _vp, _vp, _vp],
    "wf_scene_end": [_vp],
    "wf_scene_get_instances": [_vp, _vp, _u32, _pu32],
    "wf_scene_get_tlas": [_vp, _vp, _pu64],
    "wf_render": [_vp, _vp, _vp, _u32],
    "wf_read_image": [_vp, _vp, _u64],
    "wf_read_image_async": [_vp, _vp, _u64],
    "wf_read_image_ldr": [_vp, _vp, _u64],
    "wf_get_stats": [_vp, _vp],
    "wf_trace": [_vp, _vp, _u32, _vp, _u32],
    "wf_trace_device": [_vp, _vp, _u32, _vp, _u32],
    "wf_bvh_build": [_vp, _vp, _u32, _vp, _vp, _pu64],
    "wf_tlas_build": [_vp, _vp, _u32, _vp, _pu64],
    "wf_tlas_build_noalloc": [_vp, _u32, _vp, _u32, _vp],
    "wf_bvh_quantize": [_vp, _u64, _vp, _pu64, _pu32],
    "wf_bvh_widen": [_vp, _u64, _vp, _pu64, _pu32],
    "wf_image_decode": [_vp, _u64, _pu32, _pu32, _pu32, _vp, _pu64],
    "wf_texture_read": [_vp, _u32, _vp, _u64],
    "wf_scene_triangle_count": [_vp, _pu64],
    "wf_scene_set_albedo": [_vp, _vp, _u64],
    "wf_scene_set_emission": [_vp, _u32, ctypes.c_float],
    "wf_adjoint": [_vp, _vp, _vp, _u32, _vp, _vp, _vp],
    "wf_texture_create": [_vp, _u32, _u32, _u32, _vp, _pu32],
    "wf_save_accumulator": [_vp, ctypes.c_char_p],
    "wf_load_accumulator": [_vp, ctypes.c_char_p, _pu32, _pu32],
    "wf_batch_create": [_vp, ctypes.POINTER(_vp)],
    "wf_batch_destroy": [_vp],
    "wf_batch_scene_begin": [_vp, _u32, _u32, _u32, _vp, _vp, _pu32],
    "wf_batch_instance_submit": [_vp, _u32, _vp, _vp],
    "wf_batch_scene_end": [_vp],
    "wf_batch_set_config": [_vp, _vp],
    "wf_batch_get_config": [_vp, _vp],
    "wf_batch_render": [_vp, _vp, _vp, _u32],
    "wf_batch_autotune": [_vp, _vp, _vp, _u32, _vp],
    "wf_batch_read_image": [_vp, _u32, _vp, _u64],
    "wf_batch_get_stats": [_vp, _vp],
}
_RESTYPES = {"wf_status_string": ctypes.c_char_p, "wf_last_error": ctypes.c_char_p}


class WFError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


_lib = None


def load(path=None):
    """Loads libwf.so (building it first when only the sources are present)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get(LIB_ENV) or LIB_PATH
    if not os.path.exists(path):
        if path != LIB_PATH:
            raise FileNotFoundError(f"{LIB_ENV}={path}: no such library")
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _RESTYPES.get(name, ctypes.c_int)
    _lib = L
    return L


def check(rc):
    if rc != 0:
        msg = load().wf_last_error()
        raise WFError(rc, msg.decode() if msg else "")
    return rc


def _f16(m):
    a = np.ascontiguousarray(m, dtype=np.float32)
    if a.shape == (4, 4):
        a = abi.mat_f32(a)
    assert a.shape == (16,)
    return a


def decode_image(data):
    """A .jpg / .png / .hdr / .dds file's contents decoded by wf_image_decode
    (host only): (texels or BC blocks as a uint8 / float32 array, width,
    height, wf_texture_format)."""
    L = load()
    buf = np.frombuffer(bytes(data), dtype=np.uint8)
    w, h, f = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    n = ctypes.c_uint64(0)
    check(L.wf_image_decode(ptr(buf), buf.nbytes, ctypes.byref(w), ctypes.byref(h), ctypes.byref(f), None,
                            ctypes.byref(n)))
    out = np.zeros(max(1, n.value), np.uint8)
    check(L.wf_image_decode(ptr(buf), buf.nbytes, ctypes.byref(w), ctypes.byref(h), ctypes.byref(f), ptr(out),
                            ctypes.byref(n)))
    out = out[:n.value]
    if f.value == abi.TEXTURE_RGBA32F:
        out = out.view(np.float32).reshape(h.value, w.value, 4)
    elif f.value in (abi.TEXTURE_RGBA8, abi.TEXTURE_RGBA8_SRGB):
        out = out.reshape(h.value, w.value, 4)
    elif f.value == abi.TEXTURE_RG8:
        out = out.reshape(h.value, w.value, 2)
    return out, w.value, h.value, f.value


def bvh_quantize(blob):
    """The quantized 4-wide nodes of a BLAS blob (wf_bvh_quantize; host only):
    (uint32 array of 16 words per node, root leaf triangle count)."""
    L = load()
    blob = np.ascontiguousarray(blob, dtype=np.uint8)
    n = ctypes.c_uint64(0)
    rc_root = ctypes.c_uint32(0)
    check(L.wf_bvh_quantize(ptr(blob), blob.nbytes, None, ctypes.byref(n), ctypes.byref(rc_root)))
    out = np.zeros(max(1, n.value // 4), dtype=np.uint32)
    check(L.wf_bvh_quantize(ptr(blob), blob.nbytes, ptr(out), ctypes.byref(n), ctypes.byref(rc_root)))
    return out[:n.value // 4], rc_root.value


def bvh_widen(blob):
    """The exact 4-wide nodes of a BLAS blob (wf_bvh_widen; host only):
    (uint32 array of 32 words per node, root leaf triangle count)."""
    L = load()
    blob = np.ascontiguousarray(blob, dtype=np.uint8)
    n = ctypes.c_uint64(0)
    rc_root = ctypes.c_uint32(0)
    check(L.wf_bvh_widen(ptr(blob), blob.nbytes, None, ctypes.byref(n), ctypes.byref(rc_root)))
    out = np.zeros(max(1, n.value // 4), dtype=np.uint32)
    check(L.wf_bvh_widen(ptr(blob), blob.nbytes, ptr(out), ctypes.byref(n), ctypes.byref(rc_root)))
    return out[:n.value // 4], rc_root.value


class Renderer:
    """One wf_ctx: a CUDA device, its stream and all device memory."""

    def __init__(self, width, height, device=0, wave_capacity=0, tlas_metric=0, blas_layout=0, instance_bounds=0):
        """blas_layout 1 / 2: the traversal reads the quantized / exact 4-wide
        BLAS nodes (with the order-independent tie rule for closest hits).
        instance_bounds 1: instance world boxes from the BLAS frontier boxes
        (tighter TLAS leaves) instead of the transformed root box."""
        L = load()
        p = InitParams(width, height, 1, 0, device, wave_capacity, tlas_metric, blas_layout, instance_bounds)
        h = ctypes.c_void_p()
        check(L.wf_create(ctypes.byref(p), ctypes.byref(h)))
        self.h, self.L, self.width, self.height = h, L, width, height
        self._batches = weakref.WeakSet()
        self._tex_sizes = {}

    def close(self):
        if getattr(self, "h", None):
            for b in list(self._batches):   # a batch must not outlive its context
                b.close()
            self.L.wf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- meshes
    def create_render_mesh(self, vertices, indices, interval_count=8, subdivide_single_prim=False,
                           max_leaf_prims=0):
        v = np.ascontiguousarray(vertices, dtype=vertex_dtype)
        i = np.ascontiguousarray(indices, dtype=np.uint32)
        o = BvhOptions(interval_count, int(subdivide_single_prim), max_leaf_prims)
        out = ctypes.c_uint32()
        check(self.L.wf_mesh_create(self.h, ptr(v), len(v), ptr(i), len(i), ctypes.byref(o), ctypes.byref(out)))
        return out.value

    def create_mesh_from_triangles(self, tris, **opts):
        """De-indexed triangle_t input: vertices = the 3n corners, indices = 0..3n-1."""
        tris = np.ascontiguousarray(tris, dtype=triangle_dtype)
        verts = tris.view(vertex_dtype).reshape(-1)
        return self.create_render_mesh(verts, np.arange(len(verts), dtype=np.uint32), **opts)

    def create_mesh_prebuilt(self, tris, blob):
        tris = np.ascontiguousarray(tris, dtype=triangle_dtype)
        blob = np.ascontiguousarray(blob, dtype=np.uint8)
        out = ctypes.c_uint32()
        check(self.L.wf_mesh_create_prebuilt(self.h, ptr(tris), len(tris), ptr(blob), blob.nbytes,
                                             ctypes.byref(out)))
        return out.value

    def mesh_blas(self, mesh):
        n = ctypes.c_uint64(0)
        self.L.wf_mesh_get_blas(self.h, mesh, None, ctypes.byref(n))
        out = np.zeros(n.value, dtype=np.uint8)
        check(self.L.wf_mesh_get_blas(self.h, mesh, ptr(out), ctypes.byref(n)))
        return out

    # ---- textures
    def create_texture(self, texels, fmt=None):
        """texels: h x w x 4 uint8 (RGBA8, or RGBA8_SRGB with fmt), h x w x 2
        uint8 (RG8) or h x w x 4 float32 (RGBA32F).  Returns the texture id."""
        texels = np.ascontiguousarray(texels)
        h, w = texels.shape[0], texels.shape[1]
        if fmt is None:
            if texels.dtype == np.float32:
                fmt = abi.TEXTURE_RGBA32F
            elif texels.shape[2] == 2:
                fmt = abi.TEXTURE_RG8
            else:
                fmt = abi.TEXTURE_RGBA8
        out = ctypes.c_uint32()
        check(self.L.wf_texture_create(self.h, w, h, fmt, ptr(texels), ctypes.byref(out)))
        self._tex_sizes[out.value] = (w, h)
        return out.value

    def read_texture(self, texture):
        """A texture's RGBA float texels (h x w x 4) as the sampler reads them."""
        w, h = self._texture_size(texture)
        out = np.zeros((h, w, 4), np.float32)
        check(self.L.wf_texture_read(self.h, texture, ptr(out), out.size))
        return out

    def _texture_size(self, texture):
        return self._tex_sizes[texture]

    def create_texture_raw(self, data, width, height, fmt):
        """Texels or BC blocks in a wf_texture_format (as wf_image_decode
        returns them).  Returns the texture id."""
        data = np.ascontiguousarray(data)
        out = ctypes.c_uint32()
        check(self.L.wf_texture_create(self.h, width, height, fmt, ptr(data), ctypes.byref(out)))
        self._tex_sizes[out.value] = (width, height)
        return out.value

    def load_texture_file(self, path, srgb=False):
        """A texture from an image file, as the reference's asset loader takes
        it (asset_loader.cpp:56-206), decoded by wf_image_decode: .png / .jpg /
        .jpeg (RGBA8, or RGBA8_SRGB when srgb), .hdr (RGBA32F), .dds (its
        format, the sRGB variant of RGBA8 / BC1-BC3 / BC7 when srgb, dds.h:125-147)."""
        ext = os.path.splitext(path)[1].lower()
        data = open(path, "rb").read()
        if ext not in (".png", ".jpg", ".jpeg", ".hdr", ".dds"):
            raise ValueError(f"unsupported texture file type: {path}")
        raw, w, h, fmt = decode_image(data)
        if srgb:
            fmt = {abi.TEXTURE_RGBA8: abi.TEXTURE_RGBA8_SRGB, abi.TEXTURE_BC1: abi.TEXTURE_BC1_SRGB,
                   abi.TEXTURE_BC2: abi.TEXTURE_BC2_SRGB, abi.TEXTURE_BC3: abi.TEXTURE_BC3_SRGB,
                   abi.TEXTURE_BC7: abi.TEXTURE_BC7_SRGB}.get(fmt, fmt)
        return self.create_texture_raw(raw, w, h, fmt)

    # ---- scene
    def begin_scene(self, view, env=None, env_texture=0):
        e = None
        if env is not None or env_texture:
            e = Env()
            e.color[:] = list(env) if env is not None else [1.0, 1.0, 1.0]
            e.texture = env_texture
        check(self.L.wf_scene_begin(self.h, ctypes.byref(view), ctypes.byref(e) if e is not None else None))

    def submit_render_mesh(self, mesh, transform, material=None):
        """material: material_ext_dtype record (bsdf + ior) or material_dtype record (Lambert)."""
        m = _f16(transform)
        if material is None:
            material = np.zeros(1, dtype=material_ext_dtype)[0]
            material["base"]["base_color_factor"] = (0.8, 0.8, 0.8)
        if material.dtype == material_dtype:
            rec = np.array([material], dtype=material_dtype)
            check(self.L.wf_instance_submit(self.h, mesh, ptr(m), ptr(rec)))
        else:
            rec = np.array([material], dtype=material_ext_dtype)
            check(self.L.wf_instance_submit_ex(self.h, mesh, ptr(m), ptr(rec)))

    def submit_render_meshes(self, meshes, transforms, materials):
        """Many instances in one call: meshes (n,), transforms (n, 4, 4) or (n, 16)
        glm column-major, materials (n,) material_ext_dtype records."""
        meshes = np.ascontiguousarray(meshes, dtype=np.uint32)
        t = np.asarray(transforms, dtype=np.float32)
        if t.ndim == 3:
            t = np.ascontiguousarray(np.transpose(t, (0, 2, 1))).reshape(len(t), 16)   # column-major
        t = np.ascontiguousarray(t, dtype=np.float32)
        mats = np.ascontiguousarray(materials, dtype=material_ext_dtype)
        assert len(meshes) == len(t) == len(mats)
        check(self.L.wf_instance_submit_many(self.h, len(meshes), ptr(meshes), ptr(t), ptr(mats)))

    def end_scene(self):
        check(self.L.wf_scene_end(self.h))

    def scene_instances(self):
        n = ctypes.c_uint32(0)
        self.L.wf_scene_get_instances(self.h, None, 0, ctypes.byref(n))
        out = np.zeros(n.value, dtype=bvh_instance_dtype)
        check(self.L.wf_scene_get_instances(self.h, ptr(out), n.value, ctypes.byref(n)))
        return out

    def scene_tlas(self):
        n = ctypes.c_uint64(0)
        self.L.wf_scene_get_tlas(self.h, None, ctypes.byref(n))
        out = np.zeros(n.value, dtype=np.uint8)
        check(self.L.wf_scene_get_tlas(self.h, ptr(out), ctypes.byref(n)))
        return out

    # ---- rendering
    def render(self, max_bounces=3, spp=1, frame_seed=1, nee=0, rr_start_depth=0xFFFFFFFF, accumulate=True,
               cosine=1, env_strength=1.0, wave_paths=0, profile=False, count_traffic=False, view_mode=0,
               megakernel=False, fused_connect=False, tail_paths=0, serial_connect=False, fused_from_depth=0):
        """megakernel: whole paths per thread (use_wavefront_pathtracing = 0), the A/B comparator.
        fused_connect: the shadow rays of depth d in one launch with the extension rays of depth d + 1
        (instead of their own launch on a second stream).
        serial_connect: the shadow rays' launches on the main stream after shade (no
        overlap; per-kernel timings).
        fused_from_depth: with the separate schedule, from this depth on each extension
        launch also traces the previous depth's shadow rays (0 = never).
        tail_paths: queue size below which a wave's remaining bounces run per path in one launch
        (0 = never)."""
        s = RenderSettings(0 if megakernel else 1, 1, view_mode, max_bounces, cosine, int(accumulate), env_strength)
        o = RenderOptions(spp, nee, rr_start_depth, wave_paths, int(profile), int(count_traffic),
                          abi.SCHEDULE_FUSED if fused_connect else
                          abi.SCHEDULE_SERIAL if serial_connect else abi.SCHEDULE_SEPARATE, tail_paths,
                          fused_from_depth)
        check(self.L.wf_render(self.h, ctypes.byref(s), ctypes.byref(o), frame_seed))

    # ---- differentiable rendering
    def scene_triangle_count(self):
        n = ctypes.c_uint64()
        check(self.L.wf_scene_triangle_count(self.h, ctypes.byref(n)))
        return n.value

    def set_albedo(self, rgb):
        """Per scene triangle albedo, shape (triangle_count, 3); None restores the materials."""
        if rgb is None:
            check(self.L.wf_scene_set_albedo(self.h, None, 0))
            return
        a = np.ascontiguousarray(rgb, dtype=np.float32).reshape(-1)
        check(self.L.wf_scene_set_albedo(self.h, ptr(a), len(a) // 3))

    def set_emission(self, instance, strength):
        check(self.L.wf_scene_set_emission(self.h, instance, strength))

    def adjoint(self, dloss_dimage, max_bounces=6, spp=1, frame_seed=1, cosine=1, env_strength=1.0, wave_paths=0,
                profile=False, nee=0, rr_start_depth=0xFFFFFFFF):
        """Returns (d_albedo (triangles x 3), d_emission (instances,))."""
        s = RenderSettings(1, 1, 0, max_bounces, cosine, 0, env_strength)
        o = RenderOptions(spp, nee, rr_start_depth, wave_paths, int(profile), 0)
        d = np.ascontiguousarray(dloss_dimage, dtype=np.float32).reshape(-1)
        assert len(d) == 3 * self.width * self.height
        ga = np.zeros(3 * self.scene_triangle_count(), dtype=np.float32)
        ge = np.zeros(len(self.scene_instances()), dtype=np.float32)
        check(self.L.wf_adjoint(self.h, ctypes.byref(s), ctypes.byref(o), frame_seed, ptr(d), ptr(ga), ptr(ge)))
        return ga.reshape(-1, 3), ge

    def save_accumulator(self, path):
        check(self.L.wf_save_accumulator(self.h, os.fsencode(path)))

    def load_accumulator(self, path):
        """Returns (samples accumulated, frame seed of the last render)."""
        n, seed = ctypes.c_uint32(), ctypes.c_uint32()
        check(self.L.wf_load_accumulator(self.h, os.fsencode(path), ctypes.byref(n), ctypes.byref(seed)))
        return n.value, seed.value

    def read_image(self):
        out = np.zeros((self.height, self.width, 4), dtype=np.float32)
        check(self.L.wf_read_image(self.h, ptr(out), out.size))
        return out

    def read_image_async(self, out):
        """Starts copying the image into out ((height, width, 4) float32, best
        page-locked) and returns; out is complete after synchronize()."""
        assert out.dtype == np.float32 and out.flags["C_CONTIGUOUS"] and out.size >= self.width * self.height * 4
        check(self.L.wf_read_image_async(self.h, ptr(out), out.size))

    def read_image_ldr(self):
        out = np.zeros((self.height, self.width, 4), dtype=np.uint8)
        check(self.L.wf_read_image_ldr(self.h, ptr(out), out.size))
        return out

    def stats(self):
        s = Stats()
        check(self.L.wf_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def synchronize(self):
        check(self.L.wf_synchronize(self.h))

    def stream(self):
        p = ctypes.c_void_p()
        check(self.L.wf_get_stream(self.h, ctypes.byref(p)))
        return p.value

    # ---- queries and builders
    def trace(self, rays, any_hit=False, no_cull=False, reorder=False):
        """reorder: trace the rays in the order of their origins' Morton codes (WF_TRACE_REORDER)."""
        rays = np.ascontiguousarray(rays, dtype=ray_dtype)
        hits = np.zeros(len(rays), dtype=hit_dtype)
        flags = (abi.TRACE_ANY_HIT if any_hit else 0) | (abi.TRACE_NO_CULL if no_cull else 0) | \
            (abi.TRACE_REORDER if reorder else 0)
        check(self.L.wf_trace(self.h, ptr(rays), len(rays), ptr(hits), flags))
        return hits

    def trace_device(self, d_rays, n, d_hits, any_hit=False, no_cull=False, count_traffic=False, reorder=False):
        flags = (abi.TRACE_ANY_HIT if any_hit else 0) | (abi.TRACE_NO_CULL if no_cull else 0) | \
            (abi.TRACE_COUNT_TRAFFIC if count_traffic else 0) | (abi.TRACE_REORDER if reorder else 0)
        check(self.L.wf_trace_device(self.h, ctypes.c_void_p(d_rays), n, ctypes.c_void_p(d_hits), flags))

    def bvh_build(self, tris, interval_count=8, subdivide_single_prim=False, max_leaf_prims=0):
        tris = np.ascontiguousarray(tris, dtype=triangle_dtype)
        o = BvhOptions(interval_count, int(subdivide_single_prim), max_leaf_prims)
        # WF_BVH_BLOB_MAX: 2n nodes of 32 bytes at most, 40 bytes per triangle
        out = np.empty(12 + 104 * len(tris), dtype=np.uint8)
        n = ctypes.c_uint64(out.nbytes)
        check(self.L.wf_bvh_build(self.h, ptr(tris), len(tris), ctypes.byref(o), ptr(out), ctypes.byref(n)))
        return out[:n.value]   # pages past the blob were never touched

    def tlas_build(self, instances):
        inst = np.ascontiguousarray(instances, dtype=bvh_instance_dtype)
        n = ctypes.c_uint64(0)
        self.L.wf_tlas_build(self.h, ptr(inst), len(inst), None, ctypes.byref(n))
        out = np.zeros(n.value, dtype=np.uint8)
        check(self.L.wf_tlas_build(self.h, ptr(inst), len(inst), ptr(out), ctypes.byref(n)))
        return out


class Batch:
    """Many scenes of one Renderer's meshes rendered together (wf_batch_*).

    Each scene has its own camera, resolution, spp and instances; a scene's
    image equals Renderer.render's image of the same scene (accumulate off)."""

    def __init__(self, renderer):
        self.r = renderer
        self.L = renderer.L
        h = ctypes.c_void_p()
        check(self.L.wf_batch_create(renderer.h, ctypes.byref(h)))
        self.h = h
        self.sizes = []
        renderer._batches.add(self)

    def close(self):
        if self.h:
            self.L.wf_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def begin_scene(self, width, height, spp, view, env=None, env_texture=0):
        e = None
        if env is not None or env_texture:
            e = Env()
            e.color[:] = list(env) if env is not None else [1.0, 1.0, 1.0]
            e.texture = env_texture
        idx = ctypes.c_uint32(0)
        check(self.L.wf_batch_scene_begin(self.h, width, height, spp, ctypes.byref(view),
                                          ctypes.byref(e) if e is not None else None, ctypes.byref(idx)))
        self.sizes.append((width, height))
        return idx.value

    def submit(self, mesh, transform, material=None):
        m = _f16(transform)
        if material is None:
            material = np.zeros(1, dtype=material_ext_dtype)[0]
            material["base"]["base_color_factor"] = (0.8, 0.8, 0.8)
        if material.dtype == material_dtype:
            ext = np.zeros(1, dtype=material_ext_dtype)
            ext[0]["base"] = material
            ext[0]["ior"] = 1.5
            rec = ext
        else:
            rec = np.array([material], dtype=material_ext_dtype)
        check(self.L.wf_batch_instance_submit(self.h, mesh, ptr(m), ptr(rec)))

    def end_scene(self):
        check(self.L.wf_batch_scene_end(self.h))

    def config(self):
        c = BatchConfig()
        check(self.L.wf_batch_get_config(self.h, ctypes.byref(c)))
        return c.as_dict()

    def set_config(self, capacity=0, regen_threshold=0.0, block=0, use_graph=1, max_iterations=0):
        c = BatchConfig(capacity, regen_threshold, block, use_graph, max_iterations)
        check(self.L.wf_batch_set_config(self.h, ctypes.byref(c)))

    @staticmethod
    def _settings(max_bounces, nee, rr_start_depth, cosine, env_strength):
        s = RenderSettings(1, 1, 0, max_bounces, cosine, 0, env_strength)
        o = RenderOptions(0, nee, rr_start_depth, 0, 0, 0)
        return s, o

    def render(self, max_bounces=3, frame_seed=1, nee=0, rr_start_depth=0xFFFFFFFF, cosine=1, env_strength=1.0):
        s, o = self._settings(max_bounces, nee, rr_start_depth, cosine, env_strength)
        check(self.L.wf_batch_render(self.h, ctypes.byref(s), ctypes.byref(o), frame_seed))

    def autotune(self, max_bounces=3, frame_seed=1, nee=0, rr_start_depth=0xFFFFFFFF, cosine=1, env_strength=1.0):
        s, o = self._settings(max_bounces, nee, rr_start_depth, cosine, env_strength)
        c = BatchConfig()
        check(self.L.wf_batch_autotune(self.h, ctypes.byref(s), ctypes.byref(o), frame_seed, ctypes.byref(c)))
        return c.as_dict()

    def read_image(self, scene):
        w, h = self.sizes[scene]
        out = np.zeros((h, w, 4), dtype=np.float32)
        check(self.L.wf_batch_read_image(self.h, scene, ptr(out), out.size))
        return out

    def stats(self):
        s = BatchStats()
        check(self.L.wf_batch_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()


__all__ = ["Renderer", "Batch", "WFError", "load", "check", "abi", "SIGNATURES", "View", "LIB_PATH"]
