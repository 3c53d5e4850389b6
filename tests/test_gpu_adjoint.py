"""GPU: the path-replay adjoint (wf_adjoint) for per-triangle albedo and the
emitter strength, through the torch.autograd.Function harness, with BSDF
sampling only, with next-event estimation, and with next-event estimation
and Russian roulette, checked against

(a) the oracle's replay of the same single-precision paths (orc_adjoint_f32:
    the GPU's paths, summed in double) to float-atomic rounding, and its
    double-precision replay to within the paths that single and double
    precision trace differently (a triangle edge or a grazing shadow ray);
(b) with BSDF sampling only, FP64 central finite differences of the oracle's
    image loss (h = 1e-3) on 32 random parameters.  With next-event
    estimation the double-precision replay itself equals finite differences
    (tests/test_oracle_adjoint.py, 1e-6); with roulette a perturbed albedo
    flips fixed-seed decisions, which the replay's constant survival
    probabilities leave out by design."""
import numpy as np
import pytest

from wavefrontpathtracing_gb300 import Renderer, scenes
from tests.helpers import load_scene_into, oracle_scene_from_renderer

pytestmark = pytest.mark.gpu

W = H = 48
SETTINGS = dict(max_bounces=6, spp=16, frame_seed=3)
LIGHT = 2   # the emissive ceiling quad is the box scene's third instance


@pytest.fixture(scope="module")
def setup(orc):
    desc = scenes.box_scene(width=W, height=H, subdivision=2, max_bounces=6)
    o = desc.bvh_options
    blobs = [orc.bvh_build(t, o["interval_count"], False, o["max_leaf_prims"]) for t in desc.meshes]
    r = Renderer(W, H)
    ids = load_scene_into(r, desc, prebuilt_blobs=blobs)
    sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
    n = r.scene_triangle_count()
    assert n == sc.triangle_count == 24 + 320 + 2
    rng = np.random.default_rng(2)
    truth = rng.uniform(0.1, 0.9, (n, 3)).astype(np.float32)
    r.set_albedo(truth)
    r.render(accumulate=False, **SETTINGS)
    target = r.read_image()[..., :3].astype(np.float64)
    yield desc, r, sc, n, target
    r.close()


def oracle_loss(sc, desc, albedo, strength, target, st=SETTINGS):
    sc.set_albedo(albedo)
    sc.set_emission(LIGHT, strength)
    acc, _ = sc.render(desc.view, W, H, max_bounces=st["max_bounces"], spp=st["spp"], frame_seed=st["frame_seed"],
                       nee=st.get("nee", 0), rr_start_depth=st.get("rr_start_depth", 0xFFFFFFFF), f64=True, threads=8)
    img = acc[..., :3] / acc[..., 3:]
    return float(np.sum((img - target) ** 2)), img


@pytest.mark.parametrize("extra", [{}, {"nee": 1}, {"nee": 1, "rr_start_depth": 2}], ids=["bsdf", "nee", "nee_rr"])
def test_adjoint_matches_cpu_reference_and_finite_differences(orc, setup, extra):
    torch = pytest.importorskip("torch")
    from tests.gradcheck_harness import RenderImage
    desc, r, sc, n, target = setup
    st = dict(SETTINGS, **extra)
    albedo = torch.full((n, 3), 0.5, dtype=torch.float64, requires_grad=True)
    strength = torch.tensor(10.0, dtype=torch.float64, requires_grad=True)
    img = RenderImage.apply(albedo, strength, r, LIGHT, st)
    loss = ((img - torch.from_numpy(target)) ** 2).sum()
    loss.backward()
    g_alb = albedo.grad.numpy()
    g_em = float(strength.grad)
    assert np.abs(g_alb).max() > 0 and g_em != 0

    # (a) the oracle's replay of the same FP32 paths: float atomics only
    base = np.full((n, 3), 0.5)
    sc.set_albedo(base)
    sc.set_emission(LIGHT, 10.0)
    r32, r32e = sc.adjoint(desc.view, W, H, 2.0 * (img.detach().numpy() - target), f64=False, **st)
    s32 = np.abs(r32).max()
    assert np.linalg.norm(g_alb - r32) <= 1e-5 * np.linalg.norm(r32)
    err32 = np.abs(g_alb - r32) / (np.abs(r32) + 1e-3 * s32)
    assert err32.max() <= 1e-4, err32.max()
    assert abs(g_em - r32e[LIGHT]) <= 1e-4 * abs(r32e[LIGHT])
    # ... and its FP64 replay: relative L2 error and, with BSDF sampling only,
    # a per-entry bound (the few paths that take a different triangle in FP64
    # near an edge move single entries, hence the 99.5 % quantile; shadow
    # rays add such paths at every vertex)
    l0, img64 = oracle_loss(sc, desc, base, 10.0, target, st)
    assert abs(float(loss.detach()) - l0) <= 1e-3 * max(1.0, l0)
    ref_a, ref_e = sc.adjoint(desc.view, W, H, 2.0 * (img64 - target), **st)
    scale = np.abs(ref_a).max()
    rel = np.linalg.norm(g_alb - ref_a) / np.linalg.norm(ref_a)
    assert rel <= 2e-3, rel
    assert abs(g_em - ref_e[LIGHT]) <= 2e-3 * abs(ref_e[LIGHT])
    if extra:
        return
    err = np.abs(g_alb - ref_a) / (np.abs(ref_a) + 1e-3 * scale)
    assert np.quantile(err, 0.995) <= 1e-2, np.quantile(err, 0.995)
    # (b) FP64 central finite differences on 32 random parameters
    h = 1e-3
    rng = np.random.default_rng(7)
    picks = rng.choice(3 * n, size=31, replace=False)
    for k in picks:
        t, c = divmod(int(k), 3)
        ap, am = base.copy(), base.copy()
        ap[t, c] += h
        am[t, c] -= h
        fd = (oracle_loss(sc, desc, ap, 10.0, target, st)[0] - oracle_loss(sc, desc, am, 10.0, target, st)[0]) / (2 * h)
        assert abs(g_alb[t, c] - fd) <= 1e-2 * max(abs(fd), 0.01 * scale), (t, c, g_alb[t, c], fd)
    sp, sm = float(np.float32(10.0 + h)), float(np.float32(10.0 - h))   # strengths are stored as float32
    fd = (oracle_loss(sc, desc, base, sp, target, st)[0] - oracle_loss(sc, desc, base, sm, target, st)[0]) / (sp - sm)
    assert abs(g_em - fd) <= 2e-3 * abs(fd), (g_em, fd)


def test_adjoint_rejects_debug_views_and_the_megakernel(setup):
    from wavefrontpathtracing_gb300.abi import RenderOptions, RenderSettings
    import ctypes
    desc, r, sc, n, target = setup
    d = np.zeros(3 * W * H, np.float32)
    ga = np.zeros(3 * n, np.float32)
    ge = np.zeros(3, np.float32)
    o = RenderOptions(4, 1, 2, 0, 0, 0)
    for s in (RenderSettings(1, 1, 1, 6, 1, 0, 1.0), RenderSettings(0, 1, 0, 6, 1, 0, 1.0)):
        rc = r.L.wf_adjoint(r.h, ctypes.byref(s), ctypes.byref(o), 3, d.ctypes.data, ga.ctypes.data, ge.ctypes.data)
        assert rc == -1


def test_adjoint_full_size_against_fp64_finite_differences(orc):
    """The differentiable configuration at full size: box scene (20,506
    triangles) at 512 x 512, 64 spp, depth 6; per-triangle albedo at 0.5 and
    emitter strength 10; L2 loss to a target rendered with seed-2 albedo
    U[0.1, 0.9].  The GPU adjoint against FP64 central finite differences
    (h = 1e-3) of the oracle's loss on 8 random albedo parameters (2 on the
    walls, 6 among the sphere's triangles that receive light) and the
    emitter strength.  About 19 FP64 renders of 16.8M paths: minutes of host
    time."""
    import os
    torch = pytest.importorskip("torch")
    from tests.gradcheck_harness import RenderImage
    Wf = Hf = 512
    st = dict(max_bounces=6, spp=64, frame_seed=3)
    desc = scenes.box_scene(width=Wf, height=Hf, subdivision=5, max_bounces=6)
    o = desc.bvh_options
    blobs = [orc.bvh_build(t, o["interval_count"], False, o["max_leaf_prims"]) for t in desc.meshes]
    threads = os.cpu_count() or 8
    with Renderer(Wf, Hf) as r:
        ids = load_scene_into(r, desc, prebuilt_blobs=blobs)
        sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
        n = r.scene_triangle_count()
        assert n == sc.triangle_count == 20506
        truth = np.random.default_rng(2).uniform(0.1, 0.9, (n, 3)).astype(np.float32)
        r.set_albedo(truth)
        r.render(accumulate=False, **st)
        target = r.read_image()[..., :3].astype(np.float64)
        albedo = torch.full((n, 3), 0.5, dtype=torch.float64, requires_grad=True)
        strength = torch.tensor(10.0, dtype=torch.float64, requires_grad=True)
        img = RenderImage.apply(albedo, strength, r, LIGHT, st)
        loss = ((img - torch.from_numpy(target)) ** 2).sum()
        loss.backward()
    g_alb = albedo.grad.numpy()
    g_em = float(strength.grad)
    scale = np.abs(g_alb).max()

    def loss64(alb, s):
        sc.set_albedo(alb)
        sc.set_emission(LIGHT, s)
        acc, _ = sc.render(desc.view, Wf, Hf, max_bounces=6, spp=64, frame_seed=3, f64=True, threads=threads)
        return float(np.sum((acc[..., :3] / acc[..., 3:] - target) ** 2))

    base = np.full((n, 3), 0.5)
    rng = np.random.default_rng(11)
    walls = [(int(t), int(c)) for t, c in zip(rng.choice(24, 2, replace=False), rng.integers(0, 3, 2))]
    lit = np.nonzero(np.abs(g_alb[24:24 + 20480]).max(axis=1) > 1e-3 * scale)[0] + 24
    sphere = [(int(t), int(rng.integers(0, 3))) for t in rng.choice(lit, 6, replace=False)]
    h = 1e-3
    for t, c in walls + sphere:
        ap, am = base.copy(), base.copy()
        ap[t, c] += h
        am[t, c] -= h
        fd = (loss64(ap, 10.0) - loss64(am, 10.0)) / (2 * h)
        assert abs(g_alb[t, c] - fd) <= 1e-2 * max(abs(fd), 0.01 * scale), (t, c, g_alb[t, c], fd)
    sp, sm = float(np.float32(10.0 + h)), float(np.float32(10.0 - h))
    fd = (loss64(base, sp) - loss64(base, sm)) / (sp - sm)
    assert abs(g_em - fd) <= 2e-3 * abs(fd), (g_em, fd)
