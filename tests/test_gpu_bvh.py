"""GPU parity: the GPU binned-SAH BLAS builder (wf_bvh_build / wf_mesh_create)
against the reference's own builder (golden blobs) and the oracle, byte for
byte: node order, node boxes, primitive order."""
import hashlib
import os

import numpy as np
import pytest

from wavefrontpathtracing_gb300 import Renderer, scenes
from wavefrontpathtracing_gb300.abi import triangle_dtype

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "builders.npz")


def tris_from_positions(pos):
    pos = np.asarray(pos, dtype=np.float32).reshape(-1, 3, 3)
    t = np.zeros(len(pos), dtype=triangle_dtype)
    t["v0"]["position"], t["v1"]["position"], t["v2"]["position"] = pos[:, 0], pos[:, 1], pos[:, 2]
    return t


@pytest.fixture(scope="module")
def r():
    with Renderer(8, 8) as rr:
        yield rr


def first_difference(a, b):
    n = min(len(a), len(b))
    d = np.nonzero(a[:n] != b[:n])[0]
    return (int(d[0]) if d.size else n, len(a), len(b))


def test_gpu_bvh_matches_reference_goldens(r):
    g = np.load(GOLDEN)
    keys = sorted({tuple(k.split("/")[1:3]) for k in g.files if k.startswith("bvh/")})
    assert len(keys) >= 30
    for name, opt in keys:
        ic, single = (int(x[2:]) if x.startswith("ic") else int(x[1:]) for x in opt.split("_"))
        tris = tris_from_positions(g[f"pos/{name}"])
        blob = r.bvh_build(tris, ic, bool(single))
        key = f"bvh/{name}/{opt}"
        if key in g.files:
            assert np.array_equal(blob, g[key]), (key, first_difference(blob, g[key]))
        else:
            assert blob.nbytes == int(g[key + "/size"][0]), key
            assert hashlib.sha256(blob.tobytes()).digest() == g[key + "/sha256"].tobytes(), key


@pytest.mark.parametrize("n,seed,snap", [(700, 1, False), (1025, 2, False), (5000, 3, True), (60000, 4, False),
                                         (300000, 5, True)])
@pytest.mark.parametrize("ic,single,max_leaf", [(8, 0, 0), (16, 0, 4), (12, 1, 0)])
def test_gpu_bvh_matches_oracle(orc, r, n, seed, snap, ic, single, max_leaf):
    if single and n > 60000:
        pytest.skip("one triangle per leaf at this size is covered by the smaller cases")
    tris = scenes.triangle_soup(n, seed=seed, mu=-4.0)
    if snap:  # coarse grid: equal centroids, flat boxes, many SAH ties
        for v in ("v0", "v1", "v2"):
            tris[v]["position"] = np.round(tris[v]["position"] * 32) / 32
    want = orc.bvh_build(tris, ic, bool(single), max_leaf)
    got = r.bvh_build(tris, ic, bool(single), max_leaf)
    assert np.array_equal(got, want), first_difference(got, want)


def test_gpu_bvh_instanced_meshes(orc, r):
    for f, seed in ((50, 11), (9, 3)):
        tris = scenes.displaced_icosphere(f, seed=seed)
        want = orc.bvh_build(tris, 16, False, 4)
        got = r.bvh_build(tris, 16, False, 4)
        assert np.array_equal(got, want), (f, first_difference(got, want))


def test_mesh_create_uses_gpu_blas_and_traces(orc):
    desc = scenes.box_scene(width=32, height=32)
    with Renderer(32, 32) as rr:
        for t in desc.meshes:
            m = rr.create_mesh_from_triangles(t, interval_count=16, max_leaf_prims=4)
            assert np.array_equal(rr.mesh_blas(m), orc.bvh_build(t, 16, False, 4))


def test_degenerate_inputs(orc, r):
    # all centroids equal (every axis degenerate): the reference rotates the
    # index range by one and keeps a single leaf
    one = scenes.triangle_soup(1, seed=1)
    same = np.repeat(one, 17)
    for single in (False, True):
        assert np.array_equal(r.bvh_build(same, 8, single), orc.bvh_build(same, 8, single))
    # leaves larger than one warp's subtree: a root of 3000 equal triangles, and
    # 2500 equal triangles beside 2500 random ones (a large leaf below the root)
    many = np.repeat(one, 3000)
    assert np.array_equal(r.bvh_build(many, 8, False), orc.bvh_build(many, 8, False))
    mixed = np.concatenate([np.repeat(one, 2500), scenes.triangle_soup(2500, seed=4)])
    for ic, ml in ((8, 0), (16, 4)):
        assert np.array_equal(r.bvh_build(mixed, ic, False, ml), orc.bvh_build(mixed, ic, False, ml))
    flat = scenes.triangle_soup(3000, seed=9)
    for v in ("v0", "v1", "v2"):
        flat[v]["position"][:, 1] = 0.25   # coplanar: zero extent on y
    assert np.array_equal(r.bvh_build(flat, 16, False, 2), orc.bvh_build(flat, 16, False, 2))


def test_signed_zero_bounds_match_the_reference_fold(orc, r):
    """Bounds that are zero take the sign of the first zero the reference's
    glm fold meets in index-list order; mix both signs on purpose."""
    tris = scenes.triangle_soup(6000, seed=21, mu=-3.0)
    rng = np.random.default_rng(5)
    for v in ("v0", "v1", "v2"):
        p = tris[v]["position"]
        mask = rng.random(p.shape) < 0.3
        p[mask] = np.where(rng.random(mask.sum()) < 0.5, np.float32(-0.0), np.float32(0.0))
        tris[v]["position"] = p
    assert (np.signbit(tris["v0"]["position"]) & (tris["v0"]["position"] == 0)).any()
    for ic, single, ml in ((8, False, 0), (16, False, 4)):
        want = orc.bvh_build(tris, ic, single, ml)
        got = r.bvh_build(tris, ic, single, ml)
        assert np.array_equal(got, want), first_difference(got, want)


def test_blob_capacity_contract(orc, r):
    """wf_bvh_build: a buffer of the exact size or of WF_BVH_BLOB_MAX(n) takes
    one call; a smaller one gets WF_ERR_CAPACITY with the needed size and is
    left untouched."""
    import ctypes

    from wavefrontpathtracing_gb300 import BvhOptions, ptr

    WF_ERR_CAPACITY = -3

    tris = scenes.triangle_soup(3000, seed=11, mu=-4.0)
    want = orc.bvh_build(tris, 16, False, 4)
    assert len(want) <= 12 + 104 * len(tris)
    o = BvhOptions(16, 0, 4)
    for cap in (len(want), 12 + 104 * len(tris)):
        buf = np.full(cap, 0xAB, dtype=np.uint8)
        n = ctypes.c_uint64(cap)
        assert r.L.wf_bvh_build(r.h, ptr(tris), len(tris), ctypes.byref(o), ptr(buf), ctypes.byref(n)) == 0
        assert n.value == len(want)
        assert np.array_equal(buf[:n.value], want)
    small = np.full(len(want) - 1, 0xAB, dtype=np.uint8)
    n = ctypes.c_uint64(small.nbytes)
    assert r.L.wf_bvh_build(r.h, ptr(tris), len(tris), ctypes.byref(o), ptr(small), ctypes.byref(n)) == WF_ERR_CAPACITY
    assert n.value == len(want)
    assert (small == 0xAB).all()
    n = ctypes.c_uint64(0)
    assert r.L.wf_bvh_build(r.h, ptr(tris), len(tris), ctypes.byref(o), None, ctypes.byref(n)) == WF_ERR_CAPACITY
    assert n.value == len(want)
