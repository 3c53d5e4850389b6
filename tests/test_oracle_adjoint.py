"""CPU: the oracle's path-replay adjoint (orc_adjoint_f64), the checker of the
GPU adjoint, against FP64 central finite differences of the oracle's own
image loss, with next-event estimation on.

With the random numbers fixed, a Lambert albedo moves no ray (the samplers
and MIS weights do not depend on it) and no roulette decision (roulette off
here), so the FP64 image is a polynomial in the albedos and strengths and a
central difference with h = 1e-4 agrees with the exact gradient to about
1e-7 relative.  With roulette on, the replay holds the survival
probabilities constant; that case is compared between the GPU and this
oracle (tests/test_gpu_adjoint.py), not against differences, whose fixed-seed
decisions flip under a perturbation."""
import numpy as np
import pytest

from wavefrontpathtracing_gb300 import scenes
from tests.helpers import oracle_scene_from_desc

W = H = 24
LIGHT = 2   # the box scene's emissive ceiling quad
KW = dict(max_bounces=4, spp=8, frame_seed=3)


def loss_and_image(sc, desc, albedo, strength, target, nee):
    sc.set_albedo(albedo)
    sc.set_emission(LIGHT, strength)
    acc, _ = sc.render(desc.view, W, H, nee=nee, f64=True, threads=4, **KW)
    img = acc[..., :3] / acc[..., 3:]
    return float(np.sum((img - target) ** 2)), img


@pytest.mark.parametrize("nee", [0, 1])
def test_oracle_adjoint_equals_finite_differences(orc, nee):
    desc = scenes.box_scene(width=W, height=H, subdivision=2, max_bounces=4)
    sc = oracle_scene_from_desc(orc, desc)
    n = sc.triangle_count
    rng = np.random.default_rng(4)
    _, target = loss_and_image(sc, desc, rng.uniform(0.1, 0.9, (n, 3)), 10.0, np.zeros((H, W, 3)), nee)
    base = np.full((n, 3), 0.5)
    l0, img = loss_and_image(sc, desc, base, 10.0, target, nee)
    assert l0 > 0
    ga, ge = sc.adjoint(desc.view, W, H, 2.0 * (img - target), nee=nee, **KW)
    scale = np.abs(ga).max()
    assert scale > 0 and ge[LIGHT] != 0
    h = 1e-4
    # parameters that receive light: the largest gradients, and some random ones
    picks = list(np.argsort(-np.abs(ga).reshape(-1))[:6]) + list(rng.choice(3 * n, 6, replace=False))
    for k in picks:
        t, c = divmod(int(k), 3)
        ap, am = base.copy(), base.copy()
        ap[t, c] += h
        am[t, c] -= h
        fd = (loss_and_image(sc, desc, ap, 10.0, target, nee)[0] - loss_and_image(sc, desc, am, 10.0, target, nee)[0]) / (2 * h)
        assert abs(ga[t, c] - fd) <= 1e-6 * max(abs(fd), 1e-3 * scale), (t, c, ga[t, c], fd)
    sp, sm = float(np.float32(10.0 + 1e-3)), float(np.float32(10.0 - 1e-3))   # strengths are float32
    fd = (loss_and_image(sc, desc, base, sp, target, nee)[0] - loss_and_image(sc, desc, base, sm, target, nee)[0]) / (sp - sm)
    assert abs(ge[LIGHT] - fd) <= 1e-6 * abs(fd), (ge[LIGHT], fd)
