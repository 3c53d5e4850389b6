"""GPU parity of the 4-wide BLAS layouts (wf_init_params.blas_layout = 1:
quantized, 2: exact).

The traversal reads 64-byte nodes of up to four children with 8-bit planes
(csrc/wf_qbvh.cu) and takes closest hits by the order-independent tie rule
(smallest t, then smallest (instance, primitive)).  Its closest hits equal
the oracle's under the same rule bit for bit (instance, primitive, t and
barycentrics), its any-hit answers (hit or not) equal the oracle's, and so do
whole renders with every material, next-event estimation and Russian
roulette; on these scenes (no exact-t ties) they also equal the binary
layout's results."""
import numpy as np
import pytest

from wavefrontpathtracing_gb300 import Renderer, scenes
from tests.helpers import load_scene_into, oracle_scene_from_renderer
from tests.test_gpu_trace import assert_hits_equal, random_rays

pytestmark = pytest.mark.gpu


def scene_pair(orc, desc, layout):
    r = Renderer(desc.width, desc.height, blas_layout=layout, tlas_metric=2)
    ids = load_scene_into(r, desc)
    sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
    return r, sc


CASES = {
    "box": (lambda: scenes.box_scene(width=128, height=128), 0.02, 0.98),
    "instanced": (lambda: scenes.instanced_scene(width=160, height=90, instances=96, freqs=(6, 9, 12, 15), spp=1),
                  0.0, 100.0),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("layout", [1, 2])
def test_quantized_layout_hits_equal_oracle(orc, name, layout):
    make, lo, hi = CASES[name]
    desc = make()
    r, sc = scene_pair(orc, desc, layout)
    try:
        rays = np.concatenate([orc.primary_rays(desc.view, desc.width, desc.height), random_rays(30000, lo, hi, 4)])
        want, _, ovf = sc.trace(rays, flags=orc.TIE_RULE, threads=8)
        assert ovf == 0
        got = r.trace(rays)
        assert_hits_equal(got, want, f"{name} closest (tie rule)")
        ref, _, _ = sc.trace(rays, threads=8)
        assert_hits_equal(got, ref, f"{name} closest (reference order)")
        # any hit with a random tmax: whether each ray hits
        sh = random_rays(30000, lo, hi, 5, tmax=(hi - lo) * 0.5)
        want_a, _, _ = sc.trace(sh, flags=orc.ANY_HIT, threads=8)
        got_a = r.trace(sh, any_hit=True)
        assert np.array_equal(got_a["instance"] != 0xFFFFFFFF, want_a["instance"] != 0xFFFFFFFF)
        assert 100 < (got_a["instance"] != 0xFFFFFFFF).sum() < len(sh) - 100
    finally:
        r.close()


@pytest.mark.parametrize("layout", [1, 2])
def test_quantized_layout_soup_hits_equal_oracle(orc, layout):
    soup = scenes.triangle_soup(300_000, seed=11)
    desc = scenes.SceneDesc("soup", [soup], [(0, np.eye(4), scenes.material())],
                            scenes.make_view((0.5, 0.5, -0.5), (0.5, 0.5, 0.5), 90.0, 16, 16), 16, 16,
                            dict(env=(0, 0, 0)), dict(interval_count=16, subdivide_single_prim=0, max_leaf_prims=4))
    r, sc = scene_pair(orc, desc, layout)
    try:
        for kind in ("coherent", "incoherent"):
            rays = scenes.soup_rays(160, seed=7, kind=kind)
            want, _, _ = sc.trace(rays, flags=orc.TIE_RULE, threads=8)
            assert_hits_equal(r.trace(rays), want, f"soup {kind}")
            assert_hits_equal(r.trace(rays, reorder=True), want, f"soup {kind} reordered")
    finally:
        r.close()


@pytest.mark.parametrize("layout", [1, 2])
@pytest.mark.parametrize("name", ["instanced", "mixed_box"])
def test_quantized_layout_render_equals_oracle_and_binary_layout(orc, name, layout):
    """Every material, NEE and Russian roulette: the image equals the oracle's
    (tie rule) bit for bit and the binary layout's image, with the shadow rays
    in their own launches (both streams or the main one) or fused with the
    next depth's extension rays."""
    if name == "instanced":
        desc, lit = scenes.instanced_scene(width=96, height=54, instances=96, freqs=(6, 9, 12, 15), spp=4), 0.01
    else:
        desc, lit = scenes.mixed_box_scene(96, 72), 0.9
    w, h = desc.width, desc.height
    kw = dict(max_bounces=8, spp=4, frame_seed=9, nee=1, rr_start_depth=3, accumulate=False)
    imgs = []
    for lay in (layout, 0):
        r, sc = scene_pair(orc, desc, lay)
        try:
            r.render(**kw)
            imgs.append(r.read_image())
            if lay != 0:
                # the fused and serial schedules trace the same rays over the quantized nodes
                for sched in (dict(fused_connect=True), dict(serial_connect=True)):
                    r.render(**kw, **sched)
                    assert np.array_equal(r.read_image().view(np.uint32), imgs[0].view(np.uint32)), sched
                acc, _ = sc.render(desc.view, w, h, max_bounces=8, spp=4, frame_seed=9, nee=1, rr_start_depth=3,
                                   threads=8, tie_rule=True)
                want = np.zeros_like(acc)
                want[..., :3] = acc[..., :3] / acc[..., 3:]
                want[..., 3] = acc[..., 3]
                assert np.array_equal(imgs[0].view(np.uint32), want.view(np.uint32))
        finally:
            r.close()
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
    assert (imgs[0][..., :3] > 0).mean() > lit
