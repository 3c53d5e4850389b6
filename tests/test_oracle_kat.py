"""CPU: known answers for the oracle's scalar helpers (RNG, sin/cos,
intersection edge cases) and basic traversal/render sanity."""
import ctypes
import math

import numpy as np
import pytest

from wavefrontpathtracing_gb300.abi import ptr


def wang_ref(s):
    # common.hlsl:79-88 written out in Python integers
    s = ((s ^ 61) ^ (s >> 16)) & 0xFFFFFFFF
    s = (s * 9) & 0xFFFFFFFF
    s = s ^ (s >> 4)
    s = (s * 0x27D4EB2D) & 0xFFFFFFFF
    s = s ^ (s >> 15)
    return s


def test_wang_hash_known_answers(orc):
    L = orc.lib()
    for s in [0, 1, 61, 0xC977E154, 0xFFFFFFFF, 123456789]:
        assert L.orc_wang_hash(s) == wang_ref(s)


def test_rand_float_range_and_rounding(orc):
    L = orc.lib()
    seed = ctypes.c_uint32(1)
    vals = [L.orc_rand_float(ctypes.byref(seed)) for _ in range(10000)]
    assert min(vals) >= 0.0 and max(vals) <= 1.0
    # float(0xFFFFFFFF) * 2.3283064365387e-10f rounds to exactly 1.0f
    assert np.float32(np.float32(4294967295.0) * np.float32(2.3283064365387e-10)) == np.float32(1.0)


def test_sincos_2pi_accuracy(orc):
    # the samplers' angle is phi = float(2.0 * PI) * r rounded to float
    # (sample.hlsl:31-32, 47-48); sin / cos of that phi to < 1.2e-7, and so
    # within the rounding of phi of the exact sin(2 pi r)
    L = orc.lib()
    s, c = ctypes.c_float(), ctypes.c_float()
    worst_phi = worst_exact = 0.0
    rs = np.concatenate([np.linspace(0.0, 1.0, 4097, dtype=np.float32),
                         np.random.default_rng(5).random(4096, dtype=np.float32)])
    for r in rs:
        L.orc_sincos_2pi(float(r), ctypes.byref(s), ctypes.byref(c))
        phi = float(np.float32(np.float32(6.28318548) * r))
        worst_phi = max(worst_phi, abs(s.value - math.sin(phi)), abs(c.value - math.cos(phi)))
        a = 2.0 * math.pi * float(r)
        worst_exact = max(worst_exact, abs(s.value - math.sin(a)), abs(c.value - math.cos(a)))
    assert worst_phi < 1.2e-7
    assert worst_exact < 6e-7


def _tri(orc, v0, v1, v2, o, d, t=3.4e38, no_cull=0):
    arr = [np.asarray(x, dtype=np.float32) for x in (v0, v1, v2, o, d)]
    tt = ctypes.c_float(t)
    bary = np.zeros(2, dtype=np.float32)
    hit = orc.lib().orc_intersect_triangle(*[ptr(a) for a in arr], ctypes.byref(tt), ptr(bary), no_cull)
    return hit, tt.value, bary


def test_triangle_front_back_and_ties(orc):
    v0, v1, v2 = (0, 0, 0), (1, 0, 0), (0, 1, 0)   # (v1-v0)x(v2-v0) = +z: front side is +z
    hit, t, bary = _tri(orc, v0, v1, v2, (0.25, 0.25, 1.0), (0, 0, -1))
    assert hit and t == np.float32(1.0) and np.allclose(bary, [0.25, 0.25])
    hit, _, _ = _tri(orc, v0, v1, v2, (0.25, 0.25, -1.0), (0, 0, 1))
    assert not hit                                          # back face culled (det < 1e-8)
    hit, _, _ = _tri(orc, v0, v1, v2, (0.25, 0.25, -1.0), (0, 0, 1), no_cull=1)
    assert hit
    hit, _, _ = _tri(orc, v0, v1, v2, (0.25, 0.25, 1.0), (0, 0, -1), t=1.0)
    assert not hit                                          # t >= ray.t is rejected: first found wins ties
    hit, _, _ = _tri(orc, v0, v1, v2, (0.25, 0.25, 1.0), (1, 0, 0))
    assert not hit                                          # parallel ray: det = 0
    hit, t, bary = _tri(orc, v0, v1, v2, (0.0, 0.0, 1.0), (0, 0, -1))
    assert hit and bary[0] == 0 and bary[1] == 0            # vertex hit: v = w = 0 accepted


def test_aabb_slab_edge_cases(orc):
    L = orc.lib()
    bmin = np.zeros(3, np.float32)
    bmax = np.ones(3, np.float32)

    def slab(o, d, t=3.4e38):
        d = np.asarray(d, np.float32)
        with np.errstate(divide="ignore"):
            inv = (np.float32(1.0) / d).astype(np.float32)
        return L.orc_intersect_aabb(ptr(bmin), ptr(bmax), ptr(np.asarray(o, np.float32)), ptr(inv), t)

    big = np.float32(3.4028235e38)
    assert slab((-1, 0.5, 0.5), (1, 0, 0)) == np.float32(1.0)
    assert slab((0.5, 0.5, 0.5), (1, 0, 0)) == np.float32(-0.5)   # origin inside: negative tmin
    assert slab((2, 0.5, 0.5), (1, 0, 0)) == big                  # box behind the ray
    assert slab((-1, 0.5, 0.5), (1, 0, 0), t=0.5) == big          # beyond ray.t
    # axis-parallel ray in the plane of a face: (0 - 0) * inf = NaN, and
    # minNum/maxNum then keep the other slab value (+inf), so tmin = +inf: a miss
    assert slab((-1, 0.0, 0.5), (1, 0, 0)) == big
    # strictly inside the slab of the parallel axis: hit
    assert slab((-1, 1e-3, 0.5), (1, 0, 0)) == np.float32(1.0)


def test_primary_ray_points_forward(orc):
    from wavefrontpathtracing_gb300 import scenes
    view = scenes.make_view((0.0, 0.0, -5.0), (0.0, 0.0, 0.0), 60.0, 65, 33)
    rays = orc.primary_rays(view, 65, 33)
    centre = rays[16 * 65 + 32]
    assert np.allclose(centre["origin"], (0, 0, -5), atol=1e-5)
    assert np.allclose(centre["dir"], (0, 0, 1), atol=1e-3)
    assert rays[0]["dir"][1] > 0 and rays[0]["dir"][0] < 0           # row 0 is the top, x grows right
    assert np.allclose(np.linalg.norm(rays["dir"], axis=1), 1.0, atol=1e-5)


def test_trace_single_instance_against_brute_force(orc):
    """Closest hits through the BVH equal a brute-force minimum over all triangles
    (ties excepted), for a small random soup."""
    from wavefrontpathtracing_gb300 import scenes
    from tests.helpers import single_instance_scene
    tris = scenes.triangle_soup(400, seed=3, mu=-2.5)
    sc = single_instance_scene(orc, [tris])
    rays = scenes.soup_rays(24, kind="incoherent")
    hits, cnt, ovf = sc.trace(rays)
    assert ovf == 0 and cnt["triangle_tests"] > 0
    bt = np.full(len(rays), np.inf)
    for i in range(len(tris)):
        for j in range(len(rays)):
            ok, t, _ = _tri(orc, tris["v0"]["position"][i], tris["v1"]["position"][i], tris["v2"]["position"][i],
                            rays["origin"][j], rays["dir"][j])
            if ok and t < bt[j]:
                bt[j] = t
    got = np.where(hits["instance"] == 0xFFFFFFFF, np.inf, hits["t"])
    assert np.array_equal(np.isinf(got), np.isinf(bt))
    fin = np.isfinite(bt)
    assert np.array_equal(got[fin].astype(np.float32), bt[fin].astype(np.float32))


def test_render_f32_and_f64_agree_on_box(orc):
    from wavefrontpathtracing_gb300 import scenes
    from tests.helpers import oracle_scene_from_desc
    desc = scenes.box_scene(width=24, height=24, subdivision=2)
    sc = oracle_scene_from_desc(orc, desc)
    a32, st = sc.render(desc.view, 24, 24, max_bounces=4, spp=8, frame_seed=7)
    a64, _ = sc.render(desc.view, 24, 24, max_bounces=4, spp=8, frame_seed=7, f64=True)
    assert st["extend_rays"][0] == 24 * 24 * 8 and st["stack_overflows"] == 0
    img32 = a32[..., :3] / a32[..., 3:]
    img64 = a64[..., :3] / a64[..., 3:]
    assert img32.mean() > 0.01
    # the same random numbers drive both; rare paths diverge at triangle edges
    assert np.sqrt(np.mean((img32 - img64) ** 2)) < 2e-2


def test_own_atan2_and_asin_are_accurate(orc):
    """The FP32 arctangent both sides evaluate (Taylor series after reduction
    by tan(pi/8)) against numpy's correctly rounded double results."""
    L = orc.lib()
    rng = np.random.default_rng(5)
    y = rng.normal(size=4000).astype(np.float32)
    x = rng.normal(size=4000).astype(np.float32)
    y[:8] = [0, 0, 1, -1, 0, 0, 1e-30, -1e-30]
    x[:8] = [1, -1, 0, 0, 0, -0.0, 1e-30, -1e-30]
    got = np.array([L.orc_atan2(float(a), float(b)) for a, b in zip(y, x)])
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    want[4:6] = 0.0   # atan2(0, +-0): defined as 0 here
    assert np.abs(got - want).max() < 6e-7
    s = np.concatenate([rng.uniform(-1, 1, 2000), [-1.0, 1.0, 0.0, 0.5]]).astype(np.float32)
    got = np.array([L.orc_asin(float(v)) for v in s])
    assert np.abs(got - np.arcsin(s.astype(np.float64))).max() < 1e-6


def test_int_to_color_known_answers(orc):
    def murmur(h):
        h ^= h >> 16
        h = (h * 0x85EBCA6B) & 0xFFFFFFFF
        h ^= h >> 13
        h = (h * 0xC2B2AE35) & 0xFFFFFFFF
        h ^= h >> 16
        return h
    for v in (0, 1, 7, 123456, 0xFFFFFFFF):
        h = murmur(v)
        want = np.array([h & 255, (h >> 8) & 255, (h >> 16) & 255], np.float32) * np.float32(1.0 / 255.0)
        assert np.array_equal(orc.int_to_color(v), want)


def test_bilinear_wrap_sampling(orc):
    rng = np.random.default_rng(3)
    tex = rng.uniform(0, 1, (5, 7, 4)).astype(np.float32)
    h, w = tex.shape[:2]
    for u, v in [(0.0, 0.0), (0.5, 0.5), (1.3, -0.2), (-2.71, 3.14), (0.07, 0.93)]:
        x, y = u * w - 0.5, v * h - 0.5
        x0, y0 = np.floor(x), np.floor(y)
        ax, ay = x - x0, y - y0
        i0, i1 = int(x0) % w, int(x0 + 1) % w
        j0, j1 = int(y0) % h, int(y0 + 1) % h
        t = tex.astype(np.float64)
        want = (1 - ay) * ((1 - ax) * t[j0, i0] + ax * t[j0, i1]) + ay * ((1 - ax) * t[j1, i0] + ax * t[j1, i1])
        np.testing.assert_allclose(orc.tex_sample(tex, u, v), want, atol=2e-6)
    # a 1x1 texture returns its texel exactly
    one = np.array([[[0.3, 0.6, 0.9, 1.0]]], np.float32)
    assert np.array_equal(orc.tex_sample(one, 0.37, -5.2), one[0, 0])


def test_equirect_environment_lookup(orc):
    rng = np.random.default_rng(8)
    env = rng.uniform(0, 1, (8, 16, 4)).astype(np.float32)
    d = rng.normal(size=(500, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    agree = 0
    for v in d.astype(np.float32):
        u = np.arctan2(float(v[2]), float(v[0])) * 0.1591 + 0.5
        w = np.arcsin(-float(v[1])) * 0.3183 + 0.5
        want = env[int(w * 8), int(u * 16), :3]
        agree += np.array_equal(orc.env_texel(env, v), want)
    assert agree >= 495   # texel boundaries may round either way in float


def test_tangent_plane_cosine_sample_ends_the_path(orc):
    """Box scene at 512x512 (depth 6, per-triangle albedo 0.5, emitter strength
    10, frame seed 5): sample 54 of pixel (494, 400) draws a cosine-weighted
    direction in the tangent plane at its second hit.  The reference's
    weight NoL * brdf * (1 / pdf) is 0 * inf = NaN there (shade.hlsl:123-135);
    the oracle (and the GPU kernels) end the path instead, so the pixel stays
    finite and FP32 agrees with FP64."""
    from wavefrontpathtracing_gb300 import scenes
    from tests.helpers import oracle_scene_from_desc
    desc = scenes.box_scene(width=512, height=512, max_bounces=6)
    sc = oracle_scene_from_desc(orc, desc)
    sc.set_albedo(np.full((sc.triangle_count, 3), 0.5))
    sc.set_emission(2, 10.0)
    p = 400 * 512 + 494
    kw = dict(max_bounces=6, spp=1, sample_offset=54, frame_seed=5, pixel_range=(p, p + 1))
    a32, st = sc.render(desc.view, 512, 512, **kw)
    a64, _ = sc.render(desc.view, 512, 512, f64=True, **kw)
    v32, v64 = a32.reshape(-1, 4)[p], a64.reshape(-1, 4)[p]
    assert st["extend_rays"][:2] == [1, 1] and sum(st["extend_rays"]) == 2   # no third segment
    assert np.isfinite(v32).all() and v32[3] == 1
    assert np.allclose(v32, v64, rtol=1e-5, atol=0)
