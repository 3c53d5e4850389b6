"""CPU: the oracle against the reference's own shader text.

oracle/_ref/libref_hlsl.so is the reference's traversal, intersection,
sampling and shade-stage HLSL (source/renderer/shaders/) compiled as C++ by
oracle/build_ref.sh (rewrite: oracle/ref_hlsl/hlsl_to_cpp.py; vocabulary:
oracle/ref_hlsl/hlsl_shim.h).  These tests pin the oracle's restatement
(oracle/orc_impl.h) to it bit for bit; the GPU tests pin the CUDA library to
the oracle bit for bit, so the library follows the reference's text.

Shared by both sides, and so not pinned by these tests: the sin / cos /
atan2 / asin / texture-filter implementations and the sums' order inside
dot / mul (hlsl_shim.h lists them), and the keyed per-path seeds.
"""
import numpy as np
import pytest

from tests import ref_hlsl
from tests.helpers import oracle_scene_from_desc, single_instance_scene
from wavefrontpathtracing_gb300 import scenes

pytestmark = pytest.mark.skipif(not ref_hlsl.available(),
                                reason="oracle/_ref/libref_hlsl.so not built (needs the reference checkout)")


def same_hits(a, b):
    """Instance, primitive, t and barycentrics equal bit for bit."""
    return (np.array_equal(a["instance"], b["instance"]) and np.array_equal(a["primitive"], b["primitive"])
            and np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
            and np.array_equal(a["bary"].view(np.uint32), b["bary"].view(np.uint32)))


def random_rays(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, dtype=scenes.ray_dtype)
    r["origin"] = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r["dir"] = d
    r["tmin"] = 1e-8
    r["tmax"] = np.finfo(np.float32).max
    return r


# ---------------------------------------------------------------- scalar helpers

def test_rng_equals_reference_text(orc):
    L, R = orc.lib(), ref_hlsl.lib()
    seeds = np.random.default_rng(1).integers(0, 2 ** 32, 20000, dtype=np.uint64)
    for s in list(seeds) + [0, 61, 0xFFFFFFFF, 0xC977E154]:
        assert L.orc_wang_hash(int(s)) == R.refh_wang_hash(int(s))
    import ctypes
    a, b = ctypes.c_uint32(12345), ctypes.c_uint32(12345)
    for _ in range(5000):
        x, y = L.orc_rand_float(ctypes.byref(a)), R.refh_rand_float(ctypes.byref(b))
        assert np.float32(x).view(np.uint32) == np.float32(y).view(np.uint32) and a.value == b.value


def test_triangle_intersection_equals_reference_text(orc):
    from tests.test_oracle_kat import _tri
    rng = np.random.default_rng(2)
    cases = []
    for _ in range(20000):
        v = rng.normal(size=(3, 3))
        o = rng.normal(size=3) * 2
        target = v[0] + rng.uniform(-0.2, 1.2) * (v[1] - v[0]) + rng.uniform(-0.2, 1.2) * (v[2] - v[0])
        d = target - o
        cases.append((v[0], v[1], v[2], o, d / np.linalg.norm(d)))
    # edges, vertices, grazing and degenerate triangles, back faces, det near 1e-8
    cases += [((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.5, 0.5, 1.0), (0, 0, -1)),
              ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.0, 0.0, 1.0), (0, 0, -1)),
              ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.25, 0.25, -1.0), (0, 0, 1)),
              ((0, 0, 0), (1, 0, 0), (2, 0, 0), (0.5, 0.0, 1.0), (0, 0, -1)),
              ((0, 0, 0), (1e-4, 0, 0), (0, 1e-4, 0), (0.0, 0.0, 1.0), (0, 0, -1)),
              ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0.25, 0.25, 0.0), (1, 0, 0))]
    for v0, v1, v2, o, d in cases:
        for t in (3.4e38, 1.0):
            h1, t1, b1 = _tri(orc, v0, v1, v2, o, d, t=t)
            h2, t2, b2 = ref_hlsl.intersect_triangle(v0, v1, v2, o, d, t=t)
            assert h1 == h2
            assert np.float32(t1).view(np.uint32) == np.float32(t2).view(np.uint32)
            assert np.array_equal(b1.view(np.uint32), b2.view(np.uint32))


def test_slab_test_equals_reference_text(orc):
    import ctypes
    from wavefrontpathtracing_gb300.abi import ptr
    rng = np.random.default_rng(3)
    L = orc.lib()
    inf = np.float32(np.inf)
    for i in range(20000):
        lo = rng.uniform(-1, 1, 3).astype(np.float32)
        hi = (lo + rng.uniform(0, 1, 3)).astype(np.float32)
        o = rng.uniform(-2, 2, 3).astype(np.float32)
        d = rng.normal(size=3).astype(np.float32)
        if i % 7 == 0:
            d[i % 3] = 0.0               # axis-parallel: inv_dir = +-inf, 0 * inf = NaN in the slab
        if i % 11 == 0:
            o[i % 3] = lo[i % 3]         # origin on a slab plane
        with np.errstate(divide="ignore"):
            inv = (np.float32(1.0) / d).astype(np.float32)
        for t in (np.float32(3.4e38), np.float32(0.5), inf):
            a = L.orc_intersect_aabb(ptr(lo), ptr(hi), ptr(o), ptr(inv), ctypes.c_float(t))
            b = ref_hlsl.intersect_aabb(lo, hi, o, inv, float(t))
            assert np.float32(a).view(np.uint32) == np.float32(b).view(np.uint32)


def test_primary_rays_equal_reference_text(orc):
    desc = scenes.box_scene(width=96, height=64)
    a = orc.primary_rays(desc.view, 96, 64)
    b = ref_hlsl.primary_rays(desc.view, 96, 64)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_hemisphere_samples_equal_reference_text(orc):
    rng = np.random.default_rng(4)
    normals = rng.normal(size=(3000, 3))
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    normals = np.concatenate([normals, np.eye(3), -np.eye(3)]).astype(np.float32)
    rs = list(zip(rng.random(len(normals), dtype=np.float32), rng.random(len(normals), dtype=np.float32)))
    rs[:8] = [(0.0, 0.0), (1.0, 0.0), (0.5, 0.25), (0.5, 0.5), (0.5, 0.75), (0.25, 1.0), (0.999, 0.125), (1e-7, 0.375)]
    for n, (r1, r2) in zip(normals, rs):
        for cosine in (1, 0):
            a = orc.hemisphere_sample(n, float(r1), float(r2), cosine)
            b = ref_hlsl.hemisphere_sample(n, float(r1), float(r2), cosine)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (n, r1, r2, cosine, a, b)


def test_int_to_color_equals_reference_text(orc):
    from wavefrontpathtracing_gb300.abi import ptr
    for v in [0, 1, 2, 255, 12345, 0xFFFFFFFF]:
        out = np.zeros(3, np.float32)
        ref_hlsl.lib().refh_int_to_color(v, ptr(out))
        assert np.array_equal(orc.int_to_color(v).view(np.uint32), out.view(np.uint32))


# ------------------------------------------------------------------- traversal

def test_box_scene_hits_equal_reference_text(orc):
    desc = scenes.box_scene(width=128, height=128)
    sc = oracle_scene_from_desc(orc, desc)
    rs = ref_hlsl.RefScene(sc)
    rays = np.concatenate([orc.primary_rays(desc.view, 128, 128), random_rays(20000, 0.02, 0.98, 5)])
    want, _, ovf = sc.trace(rays)
    assert ovf == 0
    got = rs.trace(rays)
    assert same_hits(want, got)
    assert (got["instance"] != 0xFFFFFFFF).mean() > 0.9


def test_soup_hits_equal_reference_text(orc):
    # the micro-benchmark's distributions at 200k triangles: centroids uniform
    # in the unit cube, log-normal edges; pinhole and uniform-sphere rays
    soup = scenes.triangle_soup(200_000, seed=7)
    sc = single_instance_scene(orc, [soup], interval_count=16, max_leaf=4)
    rs = ref_hlsl.RefScene(sc)
    for kind in ("coherent", "incoherent"):
        rays = scenes.soup_rays(128, seed=7, kind=kind)
        want, _, ovf = sc.trace(rays, threads=8)
        assert ovf == 0
        got = rs.trace(rays)
        assert same_hits(want, got), kind


def test_instanced_scene_hits_equal_reference_text(orc):
    desc = scenes.instanced_scene(width=160, height=90, instances=96, freqs=(6, 9, 12, 15), spp=1)
    sc = oracle_scene_from_desc(orc, desc)
    rs = ref_hlsl.RefScene(sc)
    rays = np.concatenate([orc.primary_rays(desc.view, 160, 90), random_rays(20000, 0.0, 100.0, 6)])
    want, _, ovf = sc.trace(rays, threads=8)
    assert ovf == 0
    got = rs.trace(rays)
    assert same_hits(want, got)
    assert len(np.unique(got["instance"])) > 40


# ------------------------------------------------------------------ shading

def _box(orc, w=64, h=64, subdivision=5):
    desc = scenes.box_scene(width=w, height=h, subdivision=subdivision)
    return desc, oracle_scene_from_desc(orc, desc)


@pytest.mark.parametrize("cosine", [1, 0])
def test_lambert_paths_equal_reference_text(orc, cosine):
    """Every path's radiance and every depth's queue size of the box scene
    (64 x 64, depth 4) equal the reference's wavefront loop bit for bit."""
    desc, sc = _box(orc)
    env = (0.25, 0.5, 0.75)
    rs = ref_hlsl.RefScene(sc, env_color=env)
    for sample in range(2):
        energy, counts = rs.render_sample(desc.view, 64, 64, sample, max_bounces=4, frame_seed=7, cosine=cosine,
                                          env_strength=1.5)
        acc, st = sc.render(desc.view, 64, 64, max_bounces=4, spp=1, sample_offset=sample, frame_seed=7,
                            env_color=env, env_strength=1.5, cosine=cosine, threads=8)
        assert np.array_equal(energy[..., :3].view(np.uint32), acc[..., :3].view(np.uint32))
        assert list(counts[:5]) == st["extend_rays"][:5]
        assert (energy[..., :3] > 0).mean() > 0.05   # paths that reached the light or the environment


def test_textured_materials_and_environment_equal_reference_text(orc):
    desc, sc = _box(orc, 48, 40, subdivision=3)
    rng = np.random.default_rng(8)
    tex = [rng.random((16, 8, 4), dtype=np.float32), rng.random((5, 7, 4), dtype=np.float32),
           rng.random((32, 64, 4), dtype=np.float32)]
    sc.set_textures(tex, env_texture=3)
    sc._inst[0]["material"]["base_color_index"] = 1
    sc._inst[1]["material"]["base_color_index"] = 2
    sc._inst[1]["material"]["metallic_roughness_index"] = 1
    # camera rays that miss the box read the environment texture
    rs = ref_hlsl.RefScene(sc)
    energy, counts = rs.render_sample(desc.view, 48, 40, 0, max_bounces=3, frame_seed=3)
    acc, st = sc.render(desc.view, 48, 40, max_bounces=3, spp=1, frame_seed=3, threads=8)
    assert np.array_equal(energy[..., :3].view(np.uint32), acc[..., :3].view(np.uint32))
    assert list(counts[:4]) == st["extend_rays"][:4]


@pytest.mark.parametrize("mode", [1, 2, 3, 4, 5, 6, 7, 8, 9, 11])
def test_view_modes_equal_reference_text(orc, mode):
    # the debug views of shade.hlsl:140-153 (world normal, mode 10, is left
    # out: on a miss the reference normalises a zero vector read from
    # outside the instance buffer, NaN, where the oracle writes 0)
    desc, sc = _box(orc, 48, 40, subdivision=3)
    rs = ref_hlsl.RefScene(sc)
    energy, counts = rs.render_sample(desc.view, 48, 40, 0, max_bounces=3, frame_seed=3, view_mode=mode)
    acc, _ = sc.render(desc.view, 48, 40, max_bounces=3, spp=1, frame_seed=3, threads=8, view_mode=mode)
    assert np.array_equal(energy[..., :3], acc[..., :3])   # values (the reference may write -0 where 0 + -0 = 0)
    assert counts[1] == 0
