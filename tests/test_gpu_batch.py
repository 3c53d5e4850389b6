"""GPU: batched rendering (wf_batch_*) of many scenes through one pool of paths.

Every path keeps the random numbers and the summation order it has in a
single-scene render, so each scene's image from the batch must equal, bit for
bit, the image Renderer.render makes of the same scene alone, whatever the pool
capacity, regeneration threshold and block size, with the CUDA-graph loop or
the host loop.  One scene is also checked directly against the CPU oracle."""
import numpy as np
import pytest

import wavefrontpathtracing_gb300 as wf
from wavefrontpathtracing_gb300 import Batch, Renderer, scenes
from tests.helpers import load_scene_into, oracle_scene_from_renderer

pytestmark = pytest.mark.gpu

BVH = dict(interval_count=16, max_leaf_prims=4)
RENDER = dict(max_bounces=6, nee=1, rr_start_depth=3)
SEED = 77


def small_batch():
    # seed 6: Lambert, metal and dielectric spheres, three resolutions, spp 1..3
    return scenes.batch_scenes(count=6, seed=6, tri_range=(300, 6000), resolutions=(16, 24, 40), spps=(1, 2, 3))


def make_batch(r, meshes, descs):
    ids = [r.create_mesh_from_triangles(t, **BVH) for t in meshes]
    b = Batch(r)
    for d in descs:
        b.begin_scene(d.width, d.height, d.spp, d.view, d.env)
        for mesh, l2w, mat in d.instances:
            b.submit(ids[mesh], l2w, mat)
        b.end_scene()
    return b


class OneScene:
    """A batch scene as a scenes.SceneDesc-like description (own mesh list)."""

    def __init__(self, meshes, d):
        used = sorted({m for m, _, _ in d.instances})
        remap = {m: k for k, m in enumerate(used)}
        self.meshes = [meshes[m] for m in used]
        self.instances = [(remap[m], l2w, mat) for m, l2w, mat in d.instances]
        self.view, self.width, self.height = d.view, d.width, d.height
        self.settings = dict(env=d.env, **RENDER)
        self.bvh_options = dict(interval_count=16, subdivide_single_prim=0, max_leaf_prims=4)


def single_image(meshes, d):
    desc = OneScene(meshes, d)
    with Renderer(d.width, d.height) as r:
        load_scene_into(r, desc)
        r.render(spp=d.spp, frame_seed=SEED, accumulate=False, **RENDER)
        return r.read_image()


@pytest.fixture(scope="module")
def batch_case():
    meshes, descs = small_batch()
    return meshes, descs, [single_image(meshes, d) for d in descs]


def assert_same(got, want, what):
    bad = np.nonzero((got.view(np.uint32) != want.view(np.uint32)).any(axis=-1))
    assert bad[0].size == 0, f"{what}: {bad[0].size} pixels differ, first at {list(zip(bad[0][:4], bad[1][:4]))}"


@pytest.mark.parametrize("cfg", [
    dict(capacity=1024, regen_threshold=1.0, block=256, use_graph=1),
    dict(capacity=1024, regen_threshold=0.5, block=128, use_graph=0),
    dict(capacity=1500, regen_threshold=0.9, block=512, use_graph=1),
    dict(capacity=1 << 16, regen_threshold=1.0, block=256, use_graph=1),
])
def test_batch_images_equal_single_scene_renders(batch_case, cfg):
    meshes, descs, want = batch_case
    with Renderer(8, 8) as r:
        b = make_batch(r, meshes, descs)
        b.set_config(**cfg)
        b.render(frame_seed=SEED, **RENDER)
        st = b.stats()
        for k, d in enumerate(descs):
            got = b.read_image(k)
            assert got[..., :3].mean() > 0.0
            assert_same(got, want[k], f"scene {k}")
        b.close()
    assert st["paths"] == sum(d.paths for d in descs)
    assert st["scenes"] == len(descs)
    assert st["graph_launches"] == (1 if cfg["use_graph"] else 0)
    assert st["rays_extend"] >= st["paths"] and st["rays_connect"] > 0
    # a pool smaller than the batch needs several admissions of camera paths
    if cfg["capacity"] < st["paths"]:
        assert st["iterations"] > RENDER["max_bounces"] + 1


def test_batch_rerender_and_config_change_are_deterministic(batch_case):
    meshes, descs, want = batch_case
    with Renderer(8, 8) as r:
        b = make_batch(r, meshes, descs)
        for cfg in (dict(capacity=2048), dict(capacity=1024, regen_threshold=0.75), dict(capacity=2048)):
            b.set_config(**cfg)
            b.render(frame_seed=SEED, **RENDER)
            for k in range(len(descs)):
                assert_same(b.read_image(k), want[k], f"{cfg} scene {k}")
        b.close()


def test_batch_autotune_picks_a_valid_config(batch_case):
    meshes, descs, want = batch_case
    with Renderer(8, 8) as r:
        b = make_batch(r, meshes, descs)
        cfg = b.autotune(frame_seed=SEED, **RENDER)
        assert cfg["capacity"] in (1 << 19, 1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24)
        assert round(cfg["regen_threshold"], 4) in (0.5, 0.75, 0.9, 1.0)
        assert cfg["block"] in (128, 256, 512)
        assert b.config() == cfg
        b.render(frame_seed=SEED, **RENDER)
        for k in range(len(descs)):
            assert_same(b.read_image(k), want[k], f"scene {k}")
        b.close()


def test_batch_scene_against_the_oracle(orc, batch_case):
    meshes, descs, _ = batch_case
    d = descs[1]
    desc = OneScene(meshes, d)
    with Renderer(d.width, d.height) as r:
        ids = load_scene_into(r, desc)
        sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
        b = Batch(r)
        b.begin_scene(d.width, d.height, d.spp, d.view, d.env)
        for mesh, l2w, mat in desc.instances:
            b.submit(ids[mesh], l2w, mat)
        b.end_scene()
        b.set_config(capacity=1024)
        b.render(frame_seed=SEED, **RENDER)
        got = b.read_image(0)
        b.close()
    acc, _ = sc.render(d.view, d.width, d.height, spp=d.spp, frame_seed=SEED, env_color=d.env, threads=4, **RENDER)
    want = np.zeros_like(acc)
    want[..., :3] = acc[..., :3] / acc[..., 3:]
    want[..., 3] = acc[..., 3]
    assert_same(got, want, "oracle")


def test_batch_call_order_and_argument_errors(batch_case):
    meshes, descs, _ = batch_case
    with Renderer(8, 8) as r:
        b = Batch(r)
        with pytest.raises(wf.WFError) as e:
            b.render(frame_seed=1, **RENDER)
        assert e.value.status == -7                      # no scenes
        with pytest.raises(wf.WFError) as e:
            b.set_config(capacity=100)
        assert e.value.status == -1
        with pytest.raises(wf.WFError):
            b.set_config(regen_threshold=1.5)
        with pytest.raises(wf.WFError):
            b.set_config(block=96)
        d = descs[0]
        b.begin_scene(d.width, d.height, d.spp, d.view, d.env)
        with pytest.raises(wf.WFError) as e:
            b.render(frame_seed=1, **RENDER)
        assert e.value.status == -7                      # scene still open
        with pytest.raises(wf.WFError) as e:
            b.submit(12345, np.eye(4))
        assert e.value.status == -1                      # unknown mesh
        b.end_scene()
        with pytest.raises(wf.WFError) as e:
            b.read_image(0)
        assert e.value.status == -7                      # nothing rendered
        b.close()
