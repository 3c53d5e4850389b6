"""GPU parity: the CUDA traversal (extend / connect kernels behind wf_trace)
and the GPU TLAS builder against the CPU oracle, bit for bit.

Hit ids are compared exactly; t and barycentrics are compared as float bits
(the kernels and the oracle perform the same float operations, so equality
is exact, well inside the 1e-6 relative bound on t)."""
import os

import numpy as np
import pytest

from wavefrontpathtracing_gb300 import Renderer, scenes
from wavefrontpathtracing_gb300.abi import bvh_instance_dtype, ray_dtype
from tests.helpers import load_scene_into, oracle_scene_from_renderer, single_instance_scene

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "builders.npz")


def assert_hits_equal(got, want, what=""):
    for f in ("instance", "primitive"):
        bad = np.nonzero(got[f] != want[f])[0]
        assert bad.size == 0, f"{what}: {f} differs at {bad[:8]} ({bad.size} rays)"
    gt = got.view(np.uint32).reshape(-1, 5)
    wt = want.view(np.uint32).reshape(-1, 5)
    bad = np.nonzero((gt[:, 2:] != wt[:, 2:]).any(axis=1))[0]
    assert bad.size == 0, f"{what}: t/bary bits differ at {bad[:8]} ({bad.size} rays)"


def random_rays(n, lo, hi, seed, tmax=None):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, dtype=ray_dtype)
    r["origin"] = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    r["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r["origin"] += np.float32(0)
    r["dir"] += np.float32(0)
    r["tmin"] = 1e-8
    r["tmax"] = np.finfo(np.float32).max if tmax is None else rng.uniform(0, tmax, n)
    return r


@pytest.fixture(scope="module")
def box(orc):
    desc = scenes.box_scene(width=128, height=128)
    o = desc.bvh_options
    blobs = [orc.bvh_build(t, o["interval_count"], False, o["max_leaf_prims"]) for t in desc.meshes]
    r = Renderer(128, 128)
    ids = load_scene_into(r, desc, prebuilt_blobs=blobs)
    sc, bi = oracle_scene_from_renderer(orc, desc, r, ids)
    yield desc, r, sc, bi
    r.close()


def test_gpu_tlas_matches_oracle(orc, box):
    desc, r, sc, bi = box
    assert np.array_equal(r.scene_tlas(), orc.tlas_build(bi))


def test_primary_rays_closest_hit(orc, box):
    desc, r, sc, _ = box
    rays = orc.primary_rays(desc.view, 128, 128)
    want, _, ovf = sc.trace(rays, threads=8)
    got = r.trace(rays)
    assert ovf == 0
    assert (want["instance"] != 0xFFFFFFFF).mean() > 0.5
    assert_hits_equal(got, want, "primary")


@pytest.mark.parametrize("no_cull", [False, True])
def test_incoherent_closest_hit(orc, box, no_cull):
    desc, r, sc, _ = box
    rays = random_rays(50000, 0.02, 0.98, seed=5)
    want, _, _ = sc.trace(rays, flags=2 if no_cull else 0, threads=8)
    got = r.trace(rays, no_cull=no_cull)
    assert_hits_equal(got, want, f"incoherent no_cull={no_cull}")


def test_any_hit_with_random_tmax(orc, box):
    desc, r, sc, _ = box
    rays = random_rays(50000, 0.02, 0.98, seed=6, tmax=1.0)
    want, _, _ = sc.trace(rays, flags=1, threads=8)
    got = r.trace(rays, any_hit=True)
    assert_hits_equal(got, want, "any-hit")


def test_empty_and_single_ray_batches(orc, box):
    desc, r, sc, _ = box
    assert len(r.trace(np.zeros(0, dtype=ray_dtype))) == 0
    rays = random_rays(1, 0.4, 0.6, seed=1)
    want, _, _ = sc.trace(rays)
    assert_hits_equal(r.trace(rays), want, "single")


def test_instanced_transforms(orc):
    """Rotated, scaled and translated instances of two meshes (non-identity world_to_local)."""
    desc = scenes.instanced_scene(width=64, height=48, instances=40, freqs=(6, 9), spp=1, max_bounces=3)
    o = desc.bvh_options
    blobs = [orc.bvh_build(t, o["interval_count"], False, o["max_leaf_prims"]) for t in desc.meshes]
    with Renderer(64, 48) as r:
        ids = load_scene_into(r, desc, prebuilt_blobs=blobs)
        sc, bi = oracle_scene_from_renderer(orc, desc, r, ids)
        assert np.array_equal(r.scene_tlas(), orc.tlas_build(bi))
        rays = orc.primary_rays(desc.view, 64, 48)
        rays = np.concatenate([rays, random_rays(40000, 0.0, 100.0, seed=9)])
        want, _, _ = sc.trace(rays, threads=8)
        assert (want["instance"] != 0xFFFFFFFF).sum() > 1000
        assert_hits_equal(r.trace(rays), want, "instanced")
        want, _, _ = sc.trace(rays, flags=1, threads=8)
        assert_hits_equal(r.trace(rays, any_hit=True), want, "instanced any-hit")


def test_triangle_soup_microbench_small(orc):
    """The traversal micro-benchmark's distributions at a size the oracle
    finishes in seconds: 200k soup triangles, coherent + incoherent rays."""
    tris = scenes.triangle_soup(200_000, seed=7)
    sc = single_instance_scene(orc, [tris])
    with Renderer(16, 16) as r:
        blob = orc.bvh_build(tris, 16, False, 4)
        m = r.create_mesh_prebuilt(tris, blob)
        r.begin_scene(scenes.make_view((0.5, 0.5, -0.5), (0.5, 0.5, 0.5), 90, 16, 16))
        r.submit_render_mesh(m, np.eye(4))
        r.end_scene()
        for kind in ("coherent", "incoherent"):
            rays = scenes.soup_rays(256, kind=kind)
            want, _, _ = sc.trace(rays, threads=8)
            assert_hits_equal(r.trace(rays), want, kind)
            rays["tmax"] = np.random.default_rng(3).uniform(0, 1, len(rays)).astype(np.float32)
            want, _, _ = sc.trace(rays, flags=1, threads=8)
            got = r.trace(rays, any_hit=True)
            assert_hits_equal(got, want, kind + " any-hit")
            hit = (got["instance"] != 0xFFFFFFFF).mean()
            assert 0.05 < hit < 0.99, (kind, hit)   # tmax ends both before and after the first triangle


def test_tlas_builder_goldens_and_large(orc):
    g = np.load(GOLDEN)
    with Renderer(8, 8) as r:
        for k in [k for k in g.files if k.startswith("tlas/")]:
            inst = g["inst/" + k.split("/")[1]].view(bvh_instance_dtype)
            assert np.array_equal(r.tlas_build(inst), g[k]), k
        rng = np.random.default_rng(4)
        for n in (1000, 1025, 9000):          # beyond the reference's 256; 9000 uses the global-memory list
            inst = np.zeros(n, dtype=bvh_instance_dtype)
            c = rng.random((n, 3)) * 100
            inst["aabb_min"] = (c - rng.random((n, 3))).astype(np.float32)
            inst["aabb_max"] = (c + rng.random((n, 3))).astype(np.float32)
            assert np.array_equal(r.tlas_build(inst), orc.tlas_build(inst)), n


def test_trace_device_pointers(orc, box):
    torch = pytest.importorskip("torch")
    desc, r, sc, _ = box
    rays = random_rays(4096, 0.02, 0.98, seed=12)
    want, _, _ = sc.trace(rays)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(rays) * 20, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    r.trace_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr())
    r.synchronize()
    got = d_hits.cpu().numpy().view(want.dtype)
    assert_hits_equal(got, want, "device pointers")


@pytest.mark.parametrize("metric", [2, 3])
@pytest.mark.parametrize("n", [1, 2, 3, 17, 1025, 2048, 2049, 9000, 32768])
def test_tlas_ploc_matches_oracle(orc, n, metric):
    """tlas_metric 2 / 3: the single-block GPU clustering build and the
    top-down SAH sweep equal the oracle's restatements node for node (same
    orders, neighbour windows or sweeps, tie rules and node numbering), with
    their working sets in shared memory (up to 2,048 instances) and in global
    scratch (2,049 on)."""
    rng = np.random.default_rng(100 + n)
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    c = rng.random((n, 3)) * 100
    inst["aabb_min"] = (c - rng.random((n, 3))).astype(np.float32)
    inst["aabb_max"] = (c + rng.random((n, 3))).astype(np.float32)
    if n > 5:
        inst[4] = inst[3]
        inst["aabb_min"][5] = inst["aabb_max"][5] = inst["aabb_min"][2]   # a degenerate box
    with Renderer(8, 8, tlas_metric=metric) as r:
        assert np.array_equal(r.tlas_build(inst), orc.tlas_build(inst, metric=metric)), n


@pytest.mark.parametrize("metric", [2, 3])
def test_tlas_builds_with_signed_zeros_and_flat_boxes(orc, metric):
    """Boxes touching the origin with -0 and +0 bounds, flat (zero-extent)
    boxes and repeated centres: the GPU builds equal the oracle's bit for bit
    (the sweep's unions order -0 below +0, so their bits cannot depend on how
    a warp groups them)."""
    rng = np.random.default_rng(31)
    n = 96
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    lo = rng.uniform(-2.0, 2.0, (n, 3)).astype(np.float32)
    hi = (lo + rng.uniform(0.0, 1.0, (n, 3))).astype(np.float32)
    lo[:24] = np.float32(-0.0)
    hi[:12] = np.abs(hi[:12]) + np.float32(0.5)   # from -0 to a positive corner
    hi[12:24] = np.float32(0.0)            # flat at the origin, min -0, max +0
    hi[24:36] = lo[24:36]                  # flat boxes
    lo[36:48] = lo[48:60]                  # repeated boxes
    hi[36:48] = hi[48:60]
    inst["aabb_min"], inst["aabb_max"] = lo, hi
    with Renderer(8, 8, tlas_metric=metric) as r:
        assert np.array_equal(r.tlas_build(inst), orc.tlas_build(inst, metric=metric))


def test_tlas_sweep_all_centres_equal(orc):
    """The sweep over 300 identical boxes: every split ties, the tree is a
    300-deep chain (300 levels of the build), equal to the oracle's."""
    n = 300
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    inst["aabb_min"] = -1.0
    inst["aabb_max"] = 1.0
    with Renderer(8, 8, tlas_metric=3) as r:
        assert np.array_equal(r.tlas_build(inst), orc.tlas_build(inst, metric=3))


@pytest.mark.parametrize("metric", [2, 3])
def test_render_with_ploc_tlas_bit_exact(orc, metric):
    desc = scenes.instanced_scene(width=64, height=36, instances=200, freqs=(6, 9), spp=1, max_bounces=5)
    with Renderer(desc.width, desc.height, tlas_metric=metric) as r:
        ids = load_scene_into(r, desc)
        sc, bi = oracle_scene_from_renderer(orc, desc, r, ids)
        assert np.array_equal(r.scene_tlas(), orc.tlas_build(bi, metric=metric))
        r.render(max_bounces=5, spp=2, frame_seed=8, nee=1, rr_start_depth=3, accumulate=False)
        got = r.read_image()
    acc, _ = sc.render(desc.view, desc.width, desc.height, max_bounces=5, spp=2, frame_seed=8, nee=1,
                       rr_start_depth=3, env_color=desc.settings["env"], threads=8)
    want = np.zeros_like(acc)
    want[..., :3] = acc[..., :3] / acc[..., 3:]
    want[..., 3] = acc[..., 3]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_reordered_rays_give_the_same_hits(orc):
    """WF_TRACE_REORDER: the rays are traced in the order of their origins'
    Morton codes (a stable radix sort inside the call); every hit still lands
    at its own ray and equals the oracle's, for ray counts around the sort's
    tile size and for origins all in one cell (camera rays)."""
    tris = scenes.triangle_soup(200_000, seed=7)
    sc = single_instance_scene(orc, [tris])
    with Renderer(16, 16) as r:
        blob = orc.bvh_build(tris, 16, False, 4)
        m = r.create_mesh_prebuilt(tris, blob)
        r.begin_scene(scenes.make_view((0.5, 0.5, -0.5), (0.5, 0.5, 0.5), 90, 16, 16))
        r.submit_render_mesh(m, np.eye(4))
        r.end_scene()
        for kind in ("coherent", "incoherent"):
            rays = scenes.soup_rays(256, kind=kind)
            want, _, _ = sc.trace(rays, threads=8)
            assert_hits_equal(r.trace(rays, reorder=True), want, kind + " reordered")
            rays["tmax"] = np.random.default_rng(3).uniform(0, 1, len(rays)).astype(np.float32)
            want, _, _ = sc.trace(rays, flags=1, threads=8)
            assert_hits_equal(r.trace(rays, any_hit=True, reorder=True), want, kind + " any-hit reordered")
        rays = scenes.soup_rays(256, kind="incoherent")
        for n in (1, 3, 2047, 2048, 2049, 6000):
            sub = rays[:n].copy()
            assert_hits_equal(r.trace(sub, reorder=True), r.trace(sub), f"{n} rays")
