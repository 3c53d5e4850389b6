"""ctypes wrapper of the CPU oracle (oracle/_build/liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, bench.py's CPU-baseline leg and
__graft_entry__.smoke() as the checker.  The product (the GPU library) never
imports it.  The optional reference library oracle/_ref/libref_bvh.so (the
reference's own builders, built by oracle/build_ref.sh where the reference
checkout exists) pins the builder restatement.
"""
import ctypes
import os
import subprocess

import numpy as np

from wavefrontpathtracing_gb300.abi import (INVALID, bvh_instance_dtype, hit_dtype, material_dtype, ptr, ray_dtype,
                                            triangle_dtype, View)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_bvh.so")

instance_dtype = np.dtype([("local_to_world", "<f4", 16), ("world_to_local", "<f4", 16),
                           ("material", material_dtype), ("mesh", "<u4"), ("bsdf", "<u4"), ("ior", "<f4")])
assert instance_dtype.itemsize == 192

ANY_HIT, NO_CULL, TIE_RULE = 1, 2, 4


class _Mesh(ctypes.Structure):
    _fields_ = [("tris", ctypes.c_void_p), ("tri_count", ctypes.c_uint32), ("blas", ctypes.c_void_p)]


class _Texture(ctypes.Structure):
    _fields_ = [("texels", ctypes.c_void_p), ("w", ctypes.c_uint32), ("h", ctypes.c_uint32)]


class _Scene(ctypes.Structure):
    _fields_ = [("meshes", ctypes.POINTER(_Mesh)), ("mesh_count", ctypes.c_uint32), ("tlas", ctypes.c_void_p),
                ("inst", ctypes.c_void_p), ("inst_count", ctypes.c_uint32), ("tri_albedo", ctypes.c_void_p),
                ("inst_tri_offset", ctypes.c_void_p), ("textures", ctypes.POINTER(_Texture)),
                ("texture_count", ctypes.c_uint32), ("env_texture", ctypes.c_uint32)]


class Counters(ctypes.Structure):
    _fields_ = [("tlas_node_loads", ctypes.c_uint64), ("instance_loads", ctypes.c_uint64),
                ("blas_node_loads", ctypes.c_uint64), ("triangle_tests", ctypes.c_uint64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class RenderParams(ctypes.Structure):
    _fields_ = [("max_bounces", ctypes.c_uint32), ("cosine_weighted_diffuse", ctypes.c_uint32),
                ("hdr_env_strength", ctypes.c_float), ("env_color", ctypes.c_float * 3),
                ("spp", ctypes.c_uint32), ("sample_offset", ctypes.c_uint32), ("nee", ctypes.c_uint32),
                ("rr_start_depth", ctypes.c_uint32), ("frame_seed", ctypes.c_uint32),
                ("pixel_begin", ctypes.c_uint32), ("pixel_end", ctypes.c_uint32), ("view_mode", ctypes.c_uint32),
                ("tie_rule", ctypes.c_uint32)]


class RenderStats(ctypes.Structure):
    _fields_ = [("extend_rays", ctypes.c_uint64 * 16), ("shadow_rays", ctypes.c_uint64 * 16),
                ("stack_overflows", ctypes.c_uint64), ("extend_traffic", Counters), ("shadow_traffic", Counters)]


_lib = None
_ref = None


def build():
    """Compiles liborc.so with the oracle's Makefile (gcc -O2 -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        L.orc_bvh_build.argtypes = [vp, u32, u32, u32, u32, ctypes.POINTER(ctypes.c_void_p),
                                    ctypes.POINTER(ctypes.c_uint64)]
        L.orc_tlas_build.argtypes = [vp, u32, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64)]
        L.orc_tlas_build_metric.argtypes = [vp, u32, u32, ctypes.POINTER(ctypes.c_void_p),
                                            ctypes.POINTER(ctypes.c_uint64)]
        L.orc_free.argtypes = [vp]
        L.orc_trace.argtypes = [ctypes.POINTER(_Scene), vp, u32, vp, u32, ctypes.POINTER(Counters), i32]
        L.orc_trace.restype = u32
        L.orc_trace_f64.argtypes = [ctypes.POINTER(_Scene), vp, u32, vp, u32, i32]
        L.orc_trace_f64.restype = u32
        L.orc_render.argtypes = [ctypes.POINTER(_Scene), ctypes.POINTER(View), ctypes.POINTER(RenderParams), vp,
                                 ctypes.POINTER(RenderStats), i32]
        L.orc_render_f64.argtypes = [ctypes.POINTER(_Scene), ctypes.POINTER(View), ctypes.POINTER(RenderParams),
                                     vp, i32]
        L.orc_adjoint_f64.argtypes = [ctypes.POINTER(_Scene), ctypes.POINTER(View), ctypes.POINTER(RenderParams), vp,
                                      vp, vp]
        L.orc_adjoint_f32.argtypes = L.orc_adjoint_f64.argtypes
        L.orc_wang_hash.argtypes = [u32]
        L.orc_wang_hash.restype = u32
        L.orc_rand_float.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
        L.orc_rand_float.restype = ctypes.c_float
        L.orc_path_seed.argtypes = [u32, u32, u32, u32]
        L.orc_path_seed.restype = u32
        L.orc_sincos_2pi.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
        L.orc_sincos.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
        L.orc_hemisphere_sample.argtypes = [vp, ctypes.c_float, ctypes.c_float, i32, vp]
        dbl = ctypes.c_double
        L.orc_sample_bsdf_batch.argtypes = [i32, u32, vp, dbl, dbl, vp, vp, vp, u32, i32, vp, vp, vp, vp]
        L.orc_eval_bsdf_batch.argtypes = [u32, vp, dbl, vp, vp, vp, u32, i32, vp, vp, vp]
        L.orc_intersect_triangle.argtypes = [vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_float), vp, i32]
        L.orc_intersect_aabb.argtypes = [vp, vp, vp, vp, ctypes.c_float]
        L.orc_intersect_aabb.restype = ctypes.c_float
        L.orc_primary_ray.argtypes = [ctypes.POINTER(View), u32, u32, vp]
        L.orc_atan2.argtypes = [ctypes.c_float, ctypes.c_float]
        L.orc_atan2.restype = ctypes.c_float
        L.orc_asin.argtypes = [ctypes.c_float]
        L.orc_asin.restype = ctypes.c_float
        L.orc_int_to_color.argtypes = [u32, vp]
        L.orc_tex_sample.argtypes = [ctypes.POINTER(_Texture), ctypes.c_float, ctypes.c_float, vp]
        L.orc_env_texel.argtypes = [ctypes.POINTER(_Texture), vp, vp]
        L.orc_decode_bc.argtypes = [u32, vp, u32, u32, vp]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own builders, or None where they were not compiled."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = ctypes.CDLL(REF_PATH)
        vp, u32 = ctypes.c_void_p, ctypes.c_uint32
        R.ref_bvh_build.argtypes = [vp, u32, u32, u32, vp, ctypes.POINTER(ctypes.c_uint64)]
        R.ref_tlas_build.argtypes = [vp, u32, vp, ctypes.POINTER(ctypes.c_uint64)]
        _ref = R
    return _ref


def _blob(fn, *args):
    p = ctypes.c_void_p()
    n = ctypes.c_uint64()
    rc = fn(*args, ctypes.byref(p), ctypes.byref(n))
    if rc != 0:
        raise ValueError(f"oracle builder failed ({rc})")
    out = np.frombuffer(ctypes.string_at(p, n.value), dtype=np.uint8).copy()
    lib().orc_free(p)
    return out


def bvh_build(tris, interval_count=8, subdivide_single_prim=False, max_leaf_prims=0):
    tris = np.ascontiguousarray(tris, dtype=triangle_dtype)
    return _blob(lib().orc_bvh_build, ptr(tris), len(tris), interval_count, int(subdivide_single_prim),
                 max_leaf_prims)


def tlas_build(instances, metric=0):
    instances = np.ascontiguousarray(instances, dtype=bvh_instance_dtype)
    return _blob(lib().orc_tlas_build_metric, ptr(instances), len(instances), metric)


def ref_bvh_build(tris, interval_count=8, subdivide_single_prim=False):
    R = ref_lib()
    tris = np.ascontiguousarray(tris, dtype=triangle_dtype)
    n = ctypes.c_uint64(0)
    R.ref_bvh_build(ptr(tris), len(tris), interval_count, int(subdivide_single_prim), None, ctypes.byref(n))
    out = np.zeros(n.value, dtype=np.uint8)
    rc = R.ref_bvh_build(ptr(tris), len(tris), interval_count, int(subdivide_single_prim), ptr(out),
                         ctypes.byref(n))
    assert rc == 0
    return out


def ref_tlas_build(instances):
    R = ref_lib()
    instances = np.ascontiguousarray(instances, dtype=bvh_instance_dtype)
    n = ctypes.c_uint64(0)
    R.ref_tlas_build(ptr(instances), len(instances), None, ctypes.byref(n))
    out = np.zeros(n.value, dtype=np.uint8)
    rc = R.ref_tlas_build(ptr(instances), len(instances), ptr(out), ctypes.byref(n))
    assert rc == 0
    return out


class Scene:
    """An oracle scene: meshes (triangles + BLAS blobs), a TLAS blob and the
    per-instance shading data.  Keeps every array alive for the C side."""

    def __init__(self, meshes, tlas, instances):
        # meshes: list of (triangles ndarray[triangle_dtype], blas blob uint8)
        self._tris = [np.ascontiguousarray(t, dtype=triangle_dtype) for t, _ in meshes]
        self._blas = [np.ascontiguousarray(b, dtype=np.uint8) for _, b in meshes]
        self._tlas = np.ascontiguousarray(tlas, dtype=np.uint8)
        self._inst = np.ascontiguousarray(instances, dtype=instance_dtype)
        arr = (_Mesh * max(1, len(meshes)))()
        for i, (t, b) in enumerate(zip(self._tris, self._blas)):
            arr[i].tris = t.ctypes.data
            arr[i].tri_count = len(t)
            arr[i].blas = b.ctypes.data
        self._meshes = arr
        self.c = _Scene(arr, len(meshes), self._tlas.ctypes.data, self._inst.ctypes.data if len(self._inst) else None,
                        len(self._inst), None, None, None, 0, 0)
        self._textures = []
        self._albedo = None
        counts = [len(self._tris[m]) for m in self._inst["mesh"]]
        self.inst_tri_offset = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32) if counts else \
            np.zeros(0, np.uint32)
        self.triangle_count = int(sum(counts))

    def set_albedo(self, rgb):
        """Per scene triangle albedo (triangle_count x 3), or None for the materials."""
        if rgb is None:
            self._albedo = None
            self.c.tri_albedo = None
            self.c.inst_tri_offset = None
            return
        self._albedo = np.ascontiguousarray(rgb, dtype=np.float64).reshape(-1)
        assert len(self._albedo) == 3 * self.triangle_count
        self.c.tri_albedo = self._albedo.ctypes.data
        self.c.inst_tri_offset = self.inst_tri_offset.ctypes.data

    def set_textures(self, textures, env_texture=0):
        """textures: list of RGBA float32 arrays (h x w x 4), ids 1..n in list
        order; env_texture: 0 = the constant env colour, else a texture id."""
        self._textures = [np.ascontiguousarray(t, dtype=np.float32) for t in textures]
        arr = (_Texture * max(1, len(self._textures)))()
        for i, t in enumerate(self._textures):
            arr[i].texels = t.ctypes.data
            arr[i].h, arr[i].w = t.shape[0], t.shape[1]
        self._tex_arr = arr
        self.c.textures = arr
        self.c.texture_count = len(self._textures)
        self.c.env_texture = env_texture

    def set_emission(self, instance, strength):
        self._inst[instance]["material"]["emissive_strength"] = strength

    def adjoint(self, view, width, height, dloss_dimage, max_bounces=6, spp=1, frame_seed=1, cosine=1,
                env_color=(0.0, 0.0, 0.0), env_strength=1.0, nee=0, rr_start_depth=0xFFFFFFFF, f64=True):
        """d(loss)/d(albedo) per scene triangle and d(loss)/d(strength) per
        instance; f64=False traces the paths in single precision (the GPU's
        paths), the gradient still summed in double."""
        p = RenderParams()
        p.max_bounces, p.cosine_weighted_diffuse, p.hdr_env_strength = max_bounces, cosine, env_strength
        p.env_color[:] = env_color
        p.spp, p.sample_offset, p.nee, p.rr_start_depth, p.frame_seed = spp, 0, nee, rr_start_depth, frame_seed
        d = np.ascontiguousarray(dloss_dimage, dtype=np.float64).reshape(-1)
        assert len(d) == 3 * width * height
        ga = np.zeros(3 * self.triangle_count, dtype=np.float64)
        ge = np.zeros(len(self._inst), dtype=np.float64)
        fn = lib().orc_adjoint_f64 if f64 else lib().orc_adjoint_f32
        rc = fn(ctypes.byref(self.c), ctypes.byref(view), ctypes.byref(p), ptr(d), ptr(ga), ptr(ge))
        if rc != 0:
            raise ValueError("oracle adjoint failed")
        return ga.reshape(-1, 3), ge

    def trace(self, rays, flags=0, threads=1, f64=False):
        rays = np.ascontiguousarray(rays, dtype=ray_dtype)
        hits = np.zeros(len(rays), dtype=hit_dtype)
        cnt = Counters()
        if f64:
            ovf = lib().orc_trace_f64(ctypes.byref(self.c), ptr(rays), len(rays), ptr(hits), flags, threads)
        else:
            ovf = lib().orc_trace(ctypes.byref(self.c), ptr(rays), len(rays), ptr(hits), flags, ctypes.byref(cnt),
                                  threads)
        return hits, cnt.as_dict(), int(ovf)

    def render(self, view, width, height, max_bounces=4, spp=1, frame_seed=1, nee=0, rr_start_depth=0xFFFFFFFF,
               env_color=(0.0, 0.0, 0.0), env_strength=1.0, cosine=1, sample_offset=0, threads=1, f64=False,
               pixel_range=None, accum=None, view_mode=0, tie_rule=False):
        p = RenderParams()
        p.view_mode = view_mode
        p.tie_rule = int(tie_rule)
        p.max_bounces, p.cosine_weighted_diffuse, p.hdr_env_strength = max_bounces, cosine, env_strength
        p.env_color[:] = env_color
        p.spp, p.sample_offset, p.nee, p.rr_start_depth, p.frame_seed = spp, sample_offset, nee, rr_start_depth, \
            frame_seed
        if pixel_range:
            p.pixel_begin, p.pixel_end = pixel_range
        if accum is None:
            accum = np.zeros((height, width, 4), dtype=np.float64 if f64 else np.float32)
        st = RenderStats()
        if f64:
            rc = lib().orc_render_f64(ctypes.byref(self.c), ctypes.byref(view), ctypes.byref(p), ptr(accum), threads)
        else:
            rc = lib().orc_render(ctypes.byref(self.c), ctypes.byref(view), ctypes.byref(p), ptr(accum),
                                  ctypes.byref(st), threads)
        if rc != 0:
            raise ValueError("oracle render failed")
        stats = {"extend_rays": list(st.extend_rays), "shadow_rays": list(st.shadow_rays),
                 "stack_overflows": st.stack_overflows, "extend_traffic": st.extend_traffic.as_dict(),
                 "shadow_traffic": st.shadow_traffic.as_dict()}
        return accum, stats


def texture_struct(texels):
    """A _Texture over an RGBA float32 array (h x w x 4); keep texels alive."""
    t = _Texture()
    t.texels = texels.ctypes.data
    t.h, t.w = texels.shape[0], texels.shape[1]
    return t


def tex_sample(texels, u, v):
    texels = np.ascontiguousarray(texels, dtype=np.float32)
    out = np.zeros(4, np.float32)
    lib().orc_tex_sample(ctypes.byref(texture_struct(texels)), u, v, ptr(out))
    return out


def env_texel(texels, d):
    texels = np.ascontiguousarray(texels, dtype=np.float32)
    dd = np.asarray(d, dtype=np.float32)
    out = np.zeros(3, np.float32)
    lib().orc_env_texel(ctypes.byref(texture_struct(texels)), ptr(dd), ptr(out))
    return out


def sample_bsdf(bsdf, base, alpha, ior, n, rd, r, cosine=1, f64=True):
    """The shade stage's scattering step for m random pairs r (m x 2) at one
    surface: returns (L m x 3, weight m x 3, pdf m, flags m: 1 delta, 2 valid,
    4 crosses the dielectric)."""
    L_ = lib()
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    r = d(r).reshape(-1, 2)
    m = len(r)
    Lo, w, pdf, fl = np.zeros((m, 3)), np.zeros((m, 3)), np.zeros(m), np.zeros(m, np.int32)
    L_.orc_sample_bsdf_batch(int(f64), bsdf, ptr(d(base)), float(alpha), float(ior), ptr(d(n)), ptr(d(rd)), ptr(r), m,
                             int(cosine), ptr(Lo), ptr(w), ptr(pdf), ptr(fl))
    return Lo, w, pdf, fl


def eval_bsdf(bsdf, base, alpha, n, v, wl, cosine=1):
    """BSDF value and sampling pdf toward directions wl (m x 3): (f m x 3, pdf m, ok m)."""
    L_ = lib()
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    wl = d(wl).reshape(-1, 3)
    m = len(wl)
    f, pdf, ok = np.zeros((m, 3)), np.zeros(m), np.zeros(m, np.int32)
    L_.orc_eval_bsdf_batch(bsdf, ptr(d(base)), float(alpha), ptr(d(n)), ptr(d(v)), ptr(wl), m, int(cosine), ptr(f),
                           ptr(pdf), ptr(ok))
    return f, pdf, ok


def decode_bc(fmt, blocks, w, h):
    """BC1-BC5 / BC7 blocks -> h x w x 4 uint8 (the checker of the GPU block decoder)."""
    out = np.zeros((h, w, 4), np.uint8)
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8)
    if lib().orc_decode_bc(fmt, ptr(blocks), w, h, ptr(out)) != 0:
        raise ValueError("oracle: unknown block format")
    return out


def hemisphere_sample(n, r1, r2, cosine):
    out = np.zeros(3, np.float32)
    lib().orc_hemisphere_sample(ptr(np.asarray(n, np.float32)), r1, r2, int(cosine), ptr(out))
    return out


def int_to_color(v):
    out = np.zeros(3, np.float32)
    lib().orc_int_to_color(v, ptr(out))
    return out


def primary_rays(view, width, height):
    """All primary rays of an image, row-major (orc_primary_ray per pixel)."""
    L = lib()
    out = np.zeros(width * height, dtype=ray_dtype)
    one = np.zeros(1, dtype=ray_dtype)
    for y in range(height):
        for x in range(width):
            L.orc_primary_ray(ctypes.byref(view), x, y, ptr(one))
            out[y * width + x] = one[0]
    return out


def miss_hit():
    h = np.zeros(1, dtype=hit_dtype)
    h["instance"] = INVALID
    h["primitive"] = INVALID
    return h
