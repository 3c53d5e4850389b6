"""CPU: the oracle's builder restatement against the reference's own builders.

Pins oracle/orc_build.c to (a) the golden blobs in tests/golden/builders.npz,
generated by tests/golden/make_golden.py from the reference's bvh_builder.cpp /
tlas_builder.cpp, and (b) where oracle/_ref/libref_bvh.so was compiled from the
reference sources, to fresh random meshes.
"""
import hashlib
import os

import numpy as np
import pytest

from wavefrontpathtracing_gb300.abi import bvh_instance_dtype, bvh_node_dtype, triangle_dtype

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "builders.npz")


def tris_from_positions(pos):
    pos = np.asarray(pos, dtype=np.float32).reshape(-1, 3, 3)
    t = np.zeros(len(pos), dtype=triangle_dtype)
    t["v0"]["position"], t["v1"]["position"], t["v2"]["position"] = pos[:, 0], pos[:, 1], pos[:, 2]
    return t


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def bvh_keys(golden):
    out = []
    for k in golden.files:
        if k.startswith("bvh/"):
            parts = k.split("/")
            out.append((parts[1], parts[2]))
    return sorted(set(out))


def test_bvh_matches_golden(orc, golden):
    checked = 0
    for name, opt in bvh_keys(golden):
        ic, single = (int(x[2:]) if x.startswith("ic") else int(x[1:]) for x in opt.split("_"))
        tris = tris_from_positions(golden[f"pos/{name}"])
        blob = orc.bvh_build(tris, ic, bool(single))
        key = f"bvh/{name}/{opt}"
        if key in golden.files:
            assert np.array_equal(blob, golden[key]), key
        else:
            assert blob.nbytes == int(golden[key + "/size"][0]), key
            assert hashlib.sha256(blob.tobytes()).digest() == golden[key + "/sha256"].tobytes(), key
        checked += 1
    assert checked >= 30


def test_tlas_matches_golden(orc, golden):
    names = [k.split("/")[1] for k in golden.files if k.startswith("tlas/")]
    assert len(names) == 6
    for name in names:
        inst = golden[f"inst/{name}"].view(bvh_instance_dtype)
        assert np.array_equal(orc.tlas_build(inst), golden[f"tlas/{name}"]), name


def test_bvh_blob_invariants(orc):
    from wavefrontpathtracing_gb300 import scenes
    tris = scenes.triangle_soup(3000, seed=11)
    blob = orc.bvh_build(tris, 16, False, 4)
    h = blob[:12].view(np.uint32)
    nodes = blob[12:h[1]].view(bvh_node_dtype)
    idx = blob[h[2]:].view(np.uint32)
    assert h[0] == 12 and sorted(idx.tolist()) == list(range(3000))
    leaves = nodes[nodes["prim_count"] > 0]
    assert leaves["prim_count"].sum() == 3000
    # max_leaf_prims forces splits of larger nodes whenever a plane exists
    assert leaves["prim_count"].max() <= 4
    interior = np.nonzero(nodes["prim_count"] == 0)[0]
    interior = interior[interior != 1]
    assert (nodes["left_first"][interior] > interior).all()


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_bvh_matches_reference_random(orc, seed):
    if orc.ref_lib() is None:
        pytest.skip("reference builders not compiled here (oracle/build_ref.sh)")
    from wavefrontpathtracing_gb300 import scenes
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 5000))
    tris = scenes.triangle_soup(n, seed=seed + 100)
    # snap some coordinates to a coarse grid: equal centroids, flat boxes, ties
    if seed % 2:
        for v in ("v0", "v1", "v2"):
            tris[v]["position"] = np.round(tris[v]["position"] * 16) / 16
    for ic, single in ((8, False), (16, False), (4, True), (32, False)):
        assert np.array_equal(orc.bvh_build(tris, ic, single), orc.ref_bvh_build(tris, ic, single)), (n, ic, single)


@pytest.mark.parametrize("n", [1, 2, 5, 33, 128, 256])
def test_tlas_matches_reference_random(orc, n):
    if orc.ref_lib() is None:
        pytest.skip("reference builders not compiled here (oracle/build_ref.sh)")
    rng = np.random.default_rng(n)
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    c = rng.random((n, 3)) * 10
    inst["aabb_min"] = (c - rng.random((n, 3))).astype(np.float32)
    inst["aabb_max"] = (c + rng.random((n, 3))).astype(np.float32)
    if n > 2:  # duplicate boxes exercise the first-minimum tie rule
        inst["aabb_min"][1] = inst["aabb_min"][0]
        inst["aabb_max"][1] = inst["aabb_max"][0]
    assert np.array_equal(orc.tlas_build(inst), orc.ref_tlas_build(inst))


def _tlas_nodes(blob):
    hdr = blob[:8].view(np.uint32)
    n_nodes = (int(hdr[1]) - int(hdr[0])) // 32
    raw = blob[int(hdr[0]):int(hdr[0]) + 32 * n_nodes]
    f = raw.view(np.float32).reshape(-1, 8)
    u = raw.view(np.uint32).reshape(-1, 8)
    return f[:, 0:3], f[:, 4:7], u[:, 3], u[:, 7]


@pytest.mark.parametrize("metric", [2, 3])
@pytest.mark.parametrize("n", [1, 2, 3, 17, 1000, 5000])
def test_tlas_ploc_is_a_valid_tree(orc, n, metric):
    """tlas_metric 2 (parallel locally-ordered clustering) and 3 (top-down
    SAH sweep): leaves 1..n in instance order, every instance reached exactly
    once from the root, every box the union of its children's."""
    rng = np.random.default_rng(n)
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    c = rng.random((n, 3)) * 100
    inst["aabb_min"] = (c - rng.random((n, 3))).astype(np.float32)
    inst["aabb_max"] = (c + rng.random((n, 3))).astype(np.float32)
    if n > 3:
        inst[3] = inst[2]                      # a duplicate box
    blob = orc.tlas_build(inst, metric=metric)
    mn, mx, lr, ii = _tlas_nodes(blob)
    assert len(mn) == 2 * n
    for i in range(n):
        assert lr[1 + i] == 0 and ii[1 + i] == i
    seen = []
    stack = [0]
    while stack:
        k = stack.pop()
        if lr[k] == 0:
            seen.append(int(ii[k]))
            continue
        a, b = int(lr[k]) >> 16, int(lr[k]) & 0xFFFF
        assert np.array_equal(mn[k], np.minimum(mn[a], mn[b])) and np.array_equal(mx[k], np.maximum(mx[a], mx[b]))
        stack += [a, b]
    assert sorted(seen) == list(range(n))


@pytest.mark.parametrize("metric", [2, 3])
def test_tlas_ploc_all_centres_equal(orc, metric):
    n = 300
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    inst["aabb_min"] = -1.0
    inst["aabb_max"] = 1.0
    mn, mx, lr, ii = _tlas_nodes(orc.tlas_build(inst, metric=metric))
    assert len(mn) == 2 * n and lr[0] != 0


def test_tlas_sweep_beats_clustering_on_sah(orc):
    """The sweep's tree has the smaller surface-area cost (sum of interior
    box areas over the root's) on random instance boxes."""
    n = 1000
    rng = np.random.default_rng(12)
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    c = rng.random((n, 3)) * 100
    r = rng.uniform(0.5, 2.0, (n, 1))
    inst["aabb_min"] = (c - r).astype(np.float32)
    inst["aabb_max"] = (c + r).astype(np.float32)

    def sah(blob):
        mn, mx, lr, _ = _tlas_nodes(blob)
        e = np.maximum(mx - mn, 0.0).astype(np.float64)
        a = e[:, 0] * e[:, 1] + e[:, 1] * e[:, 2] + e[:, 2] * e[:, 0]
        return a[1:][lr[1:] != 0].sum() / a[0]

    assert sah(orc.tlas_build(inst, metric=3)) < sah(orc.tlas_build(inst, metric=2))
