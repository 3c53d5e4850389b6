"""GPU parity at the full sizes of the benchmark workloads, where the oracle
cannot redo the whole workload in seconds.  Each test checks what does not
depend on size: the oracle on a sampled subset of the same rays or pixels
(bit for bit), and equalities between two GPU paths over every ray or pixel.

* traversal micro-benchmark: 8M soup triangles (centroids U[0,1]^3,
  log-normal edges mu=-5 sigma=0.5, seed 7), 16.8M coherent and 16.8M
  incoherent rays;
* instanced frame: 1920x1080, 16 spp, depth 8, RR from 3, NEE, 1,024
  instances of 8 displaced icospheres + one area light;
* batched form: 64 scenes of 1k..2M triangles, 109M camera paths;
* differentiable form: box scene at 512x512, 64 spp, depth 6."""
import os

import numpy as np
import pytest

from wavefrontpathtracing_gb300 import Batch, Renderer, scenes
from tests.helpers import load_scene_into, oracle_scene_from_renderer
from tests.test_gpu_render import assert_images_equal
from tests.test_gpu_trace import assert_hits_equal

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
THREADS = os.cpu_count() or 1


def test_soup_8m_blas_and_16m_ray_sets(orc):
    """The GPU BLAS of 8M triangles equals the oracle's restatement of the
    reference builder byte for byte (832 MB blob); 20,000 sampled rays of each
    16.8M-ray set hit exactly what the oracle's traversal hits over that blob,
    closest and any hit; over every ray, the origin-ordered traversal gives
    the same hits, and an any-hit ray reports a hit exactly when the
    closest-hit query with the same tmax does, which in turn equals the
    unbounded closest hit when that lies before tmax."""
    tris = scenes.triangle_soup(8_000_000, seed=7)
    with Renderer(16, 16) as r:
        m = r.create_mesh_from_triangles(tris, interval_count=16, max_leaf_prims=4)
        blob = r.mesh_blas(m)
        want = orc.bvh_build(tris, 16, False, 4)
        assert len(blob) == len(want) == 832_000_012
        assert np.array_equal(blob, want)
        del want
        r.begin_scene(scenes.make_view((0.5, 0.5, -0.5), (0.5, 0.5, 0.5), 90.0, 16, 16))
        r.submit_render_mesh(m, np.eye(4))
        r.end_scene()
        bi = r.scene_instances()
        oi = np.zeros(1, dtype=orc.instance_dtype)
        oi["local_to_world"] = np.eye(4, dtype=np.float32).reshape(16)
        oi["world_to_local"] = bi[0]["world_to_local"]
        sc = orc.Scene([(tris, blob)], r.scene_tlas(), oi)
        rng = np.random.default_rng(17)
        for kind in ("coherent", "incoherent"):
            rays = scenes.soup_rays(4096, seed=7, kind=kind)
            n = len(rays)
            assert n == 4096 * 4096
            pick = np.sort(rng.choice(n, 20_000, replace=False))
            closest = r.trace(rays)
            hit = closest["instance"] != MISS
            assert 0.3 < hit.mean(), (kind, hit.mean())
            want, _, ovf = sc.trace(rays[pick], threads=THREADS)
            assert ovf == 0
            assert_hits_equal(closest[pick], want, kind + " closest (sampled)")
            assert_hits_equal(r.trace(rays, reorder=True), closest, kind + " reordered (all rays)")

            rays["tmax"] = np.random.default_rng(9).uniform(0, 1, n).astype(np.float32)
            anyh = r.trace(rays, any_hit=True)
            want, _, _ = sc.trace(rays[pick], flags=1, threads=THREADS)
            assert_hits_equal(anyh[pick], want, kind + " any hit (sampled)")
            bounded = r.trace(rays)
            a_hit = anyh["instance"] != MISS
            b_hit = bounded["instance"] != MISS
            assert np.array_equal(a_hit, b_hit), f"{kind}: {(a_hit != b_hit).sum()} rays disagree"
            before = hit & (closest["t"] < rays["tmax"])
            assert np.array_equal(b_hit, before)
            assert_hits_equal(bounded[before], closest[before], kind + " bounded closest (all rays)")
            assert 0.05 < a_hit.mean() < 0.99, (kind, a_hit.mean())


def test_instanced_1080p_frame(orc):
    """The benchmark frame (SAH-sweep TLAS over tight instance boxes, as the
    bench runs it): the oracle renders six bands of 2,048 pixels of
    the same frame from the GPU's own BLAS, instances and TLAS, and those
    pixels must equal the GPU image bit for bit; over the whole frame the
    megakernel and the fused trace schedule give the same image and the same
    rays per depth as the default schedule."""
    desc = scenes.instanced_scene()
    w, h = desc.width, desc.height
    assert (w, h, len(desc.instances)) == (1920, 1080, 1025)
    st = desc.settings
    kw = dict(max_bounces=8, spp=16, frame_seed=5, nee=1, rr_start_depth=3, accumulate=False)
    assert (st["spp"], st["max_bounces"], st["rr_start_depth"], st["nee"]) == (16, 8, 3, 1)
    with Renderer(w, h, tlas_metric=3, instance_bounds=1) as r:
        ids = load_scene_into(r, desc)
        sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
        r.render(**kw)
        img = r.read_image()
        sw = r.stats()
        r.render(megakernel=True, **kw)
        mega = r.read_image()
        sm = r.stats()
        r.render(fused_connect=True, **kw)
        fused = r.read_image()
        sf = r.stats()
    assert np.isfinite(img).all()
    assert (img[..., 3] == 16).all()
    assert img[..., :3].mean() > 0.0
    assert sw["rays_connect"] > 0 and sw["rays_extend"] > w * h * 16
    # (the megakernel counts rays in total only, not per depth)
    for other, so, what, keys in ((mega, sm, "megakernel", ("rays_extend", "rays_connect")),
                                  (fused, sf, "fused schedule", ("rays_extend", "rays_connect", "extend_rays_depth",
                                                                 "shadow_rays_depth"))):
        assert_images_equal(other, img)
        for k in keys:
            assert np.array_equal(np.asarray(so[k]), np.asarray(sw[k])), (what, k)

    npix = w * h
    acc = np.zeros((h, w, 4), dtype=np.float32)
    bands = [(p0, p0 + 2048) for p0 in np.linspace(0, npix - 2048, 6).astype(int)]
    for b in bands:
        sc.render(desc.view, w, h, max_bounces=8, spp=16, frame_seed=5, nee=1, rr_start_depth=3,
                  env_color=st["env"], threads=THREADS, pixel_range=b, accum=acc)
    flat_img = img.reshape(-1, 4)
    flat_acc = acc.reshape(-1, 4)
    idx = np.concatenate([np.arange(*b) for b in bands])
    want = np.empty((len(idx), 4), np.float32)
    want[:, :3] = flat_acc[idx, :3] / flat_acc[idx, 3:]
    want[:, 3] = flat_acc[idx, 3]
    assert (want[:, 3] == 16).all()
    bad = np.nonzero((flat_img[idx].view(np.uint32) != want.view(np.uint32)).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} of {len(idx)} sampled pixels differ, first at pixel {idx[bad[:5]]}"
    assert want[:, :3].max() > 0.0


def test_batched_64_scenes():
    """The batched configuration: 64 scenes (109M camera paths) in one
    CUDA-graph launch through a pool of 2^22 paths (so camera paths are
    admitted many times over), and every scene's image equals the plain
    single-scene wavefront render of that scene bit for bit."""
    meshes, descs = scenes.batch_scenes(count=64)
    paths = sum(d.paths for d in descs)
    assert paths > 100_000_000
    kw = dict(max_bounces=6, nee=1, rr_start_depth=3)
    with Renderer(8, 8) as r:
        ids = [r.create_mesh_from_triangles(t, interval_count=16, max_leaf_prims=4) for t in meshes]
        b = Batch(r)
        for d in descs:
            b.begin_scene(d.width, d.height, d.spp, d.view, d.env)
            for mesh, l2w, mat in d.instances:
                b.submit(ids[mesh], l2w, mat)
            b.end_scene()
        b.set_config(capacity=1 << 22, regen_threshold=0.9, block=256)
        b.render(frame_seed=11, **kw)
        bst = b.stats()
        got = [b.read_image(k) for k in range(len(descs))]
        b.close()
    assert bst["paths"] == paths and bst["scenes"] == 64 and bst["graph_launches"] == 1
    rays = 0
    for side in sorted({d.width for d in descs}):
        with Renderer(side, side) as r:
            mid = {}
            for k, d in enumerate(descs):
                if d.width != side:
                    continue
                for mesh, _, _ in d.instances:
                    if mesh not in mid:
                        mid[mesh] = r.create_mesh_from_triangles(meshes[mesh], interval_count=16, max_leaf_prims=4)
                r.begin_scene(d.view, d.env)
                for mesh, l2w, mat in d.instances:
                    r.submit_render_mesh(mid[mesh], l2w, mat)
                r.end_scene()
                r.render(spp=d.spp, frame_seed=11, accumulate=False, **kw)
                rays += r.stats()["rays_extend"] + r.stats()["rays_connect"]
                assert_images_equal(got[k], r.read_image())
    assert rays == bst["rays_extend"] + bst["rays_connect"]


def test_adjoint_512_64spp_homogeneity():
    """The differentiable configuration at full size.  Every path's
    contribution is the emitter strength s times the product of the albedos
    at its Lambert vertices, with directions that do not depend on either, so
    for a linear image functional <g, I>: s * d<g, I>/ds = <g, I>, and the
    albedo gradient summed against the albedos equals d<g, I(lambda *
    albedo)>/dlambda at lambda = 1 (a central difference of two GPU renders of
    the same paths).  Checked for positive weights g (no cancellation: tight
    relative bounds) and for the gradient of the L2 loss to the seed-2 target
    (bounded by the magnitude of its terms)."""
    w = h = 512
    spp, depth, seed, light, s = 64, 6, 5, 2, 10.0
    desc = scenes.box_scene(width=w, height=h, max_bounces=depth)
    rkw = dict(max_bounces=depth, spp=spp, frame_seed=seed, accumulate=False)
    with Renderer(w, h) as r:
        load_scene_into(r, desc)
        n = r.scene_triangle_count()
        assert n == 20_506
        r.set_albedo(np.random.default_rng(2).uniform(0.1, 0.9, (n, 3)).astype(np.float32))
        r.render(**rkw)
        target = r.read_image()[..., :3].astype(np.float64)

        def image(albedo):
            r.set_albedo(np.full((n, 3), albedo, np.float32))
            r.render(**rkw)
            return r.read_image()[..., :3].astype(np.float64)

        r.set_emission(light, s)
        eps = 1e-2
        img_p, img_m = image(0.5 * (1 + eps)), image(0.5 * (1 - eps))
        img = image(0.5)
        assert np.isfinite(img).all() and np.isfinite(target).all() and img.mean() > 0.0
        g_pos = np.random.default_rng(4).uniform(0.5, 1.5, img.shape)
        g_l2 = 2.0 * (img - target)
        grads = [(g, r.adjoint(g, max_bounces=depth, spp=spp, frame_seed=seed)) for g in (g_pos, g_l2)]
    (g, (ga, ge)), (gl, (gla, gle)) = grads
    assert all(np.isfinite(x).all() for x in (ga, ge, gla, gle))
    gi = float(np.sum(g * img))
    # float32 atomics sum ~10^6 warp contributions into one emitter gradient
    assert abs(s * float(ge[light]) - gi) <= 2e-3 * gi, (s * float(ge[light]), gi)
    d_lambda = (np.sum(g * img_p) - np.sum(g * img_m)) / (2 * eps)
    lhs = 0.5 * float(np.sum(ga.astype(np.float64)))
    assert abs(lhs - d_lambda) <= 5e-3 * d_lambda, (lhs, d_lambda)
    scale = float(np.sum(np.abs(gl) * img))
    assert abs(s * float(gle[light]) - float(np.sum(gl * img))) <= 2e-3 * scale
    d_lambda = (np.sum(gl * img_p) - np.sum(gl * img_m)) / (2 * eps)
    assert abs(0.5 * float(np.sum(gla.astype(np.float64))) - d_lambda) <= 5e-3 * scale
