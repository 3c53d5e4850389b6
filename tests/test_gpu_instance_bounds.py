"""GPU: tight instance boxes (wf_init_params.instance_bounds = 1).

Each instance's world box is computed on the device from up to 4096 frontier
boxes of its BLAS.  It must hold every transformed vertex (checked in float64
on the host), lie within the reference's box (the transformed root box, up to
the outward rounding pad), and shrink the scene's total box area; rays traced
through a TLAS over these boxes must find exactly the hits of the reference
boxes' TLAS."""
import numpy as np
import pytest

from wavefrontpathtracing_gb300 import Renderer, scenes
from wavefrontpathtracing_gb300.abi import ray_dtype
from tests.helpers import load_scene_into

pytestmark = pytest.mark.gpu


def area(lo, hi):
    e = np.maximum(hi - lo, 0.0)
    return 2.0 * (e[..., 0] * e[..., 1] + e[..., 1] * e[..., 2] + e[..., 2] * e[..., 0])


def random_rays(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, dtype=ray_dtype)
    rays["origin"] = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    rays["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = np.float32(3.0e38)
    return rays


@pytest.mark.parametrize("tlas_metric", [0, 2])
def test_tight_instance_boxes(tlas_metric):
    desc = scenes.instanced_scene(width=64, height=36, instances=300, freqs=(8, 12), spp=1, max_bounces=2)
    boxes, hits = {}, {}
    rays = random_rays(200_000, np.array([-5.0, -5.0, -5.0]), np.array([105.0, 115.0, 105.0]), seed=9)
    # half of them aimed at instance centres, so that many graze instance boxes
    rng = np.random.default_rng(10)
    centres = np.array([np.asarray(l2w, np.float64).reshape(4, 4)[:3, 3] for _, l2w, _ in desc.instances[:-1]])
    aim = centres[rng.integers(0, len(centres), size=100_000)] + rng.normal(scale=1.0, size=(100_000, 3))
    d = aim - rays["origin"][:100_000]
    rays["dir"][:100_000] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    for bounds in (0, 1):
        with Renderer(desc.width, desc.height, tlas_metric=tlas_metric, instance_bounds=bounds) as r:
            load_scene_into(r, desc)
            bi = r.scene_instances()
            boxes[bounds] = (bi["aabb_min"].astype(np.float64), bi["aabb_max"].astype(np.float64))
            hits[bounds] = r.trace(rays)
    lo1, hi1 = boxes[1]
    lo0, hi0 = boxes[0]
    # every transformed vertex inside its instance's tight box
    for k, (mesh, l2w, _) in enumerate(desc.instances):
        t = np.asarray(desc.meshes[mesh])
        p = np.concatenate([t[v]["position"] for v in ("v0", "v1", "v2")]).astype(np.float64)
        m = np.asarray(l2w, dtype=np.float32).astype(np.float64).reshape(4, 4)
        w = p @ m[:3, :3].T + m[:3, 3]
        assert (w >= lo1[k]).all() and (w <= hi1[k]).all(), k
    # within the reference box up to the rounding pad
    pad = 1e-5 * (np.abs(lo0) + np.abs(hi0) + (hi0 - lo0))
    assert (lo1 >= lo0 - pad).all() and (hi1 <= hi0 + pad).all()
    a0, a1 = area(lo0, hi0).sum(), area(lo1, hi1).sum()
    assert a1 < 0.75 * a0, (a1, a0)
    # the same hits through either TLAS
    h0, h1 = hits[0], hits[1]
    assert (h0["instance"] != 0xFFFFFFFF).mean() > 0.04   # 8% of uniformly random rays alone hit
    for f in ("instance", "primitive"):
        assert np.array_equal(h0[f], h1[f]), f
    assert np.array_equal(h0["t"].view(np.uint32), h1["t"].view(np.uint32))
    assert np.array_equal(h0["bary"].view(np.uint32), h1["bary"].view(np.uint32))


def test_unknown_instance_bounds_are_refused():
    from wavefrontpathtracing_gb300 import WFError
    with pytest.raises(WFError):
        Renderer(8, 8, instance_bounds=2)
