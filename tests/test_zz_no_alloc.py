"""GPU: wf_tlas_build_noalloc, the entry point for callers that cannot allocate
device memory (per-frame render threads, engines with a fixed device-memory budget).

It is called through the C ABI on device buffers the test owns, twice in a
row (different sizes and pairing metrics, so the shared static working list
is reused), and its nodes must equal those of the allocating entry point
wf_tlas_build byte for byte — the tolerance every builder test here uses.
This file is collected last so that a stop at its first failure has already
run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import wavefrontpathtracing_gb300 as wf
from wavefrontpathtracing_gb300.abi import bvh_instance_dtype

pytestmark = pytest.mark.gpu


def random_instances(n, seed):
    rng = np.random.default_rng(seed)
    inst = np.zeros(n, dtype=bvh_instance_dtype)
    c = rng.random((n, 3)) * 100.0
    inst["aabb_min"] = (c - rng.random((n, 3)) * 3.0).astype(np.float32)
    inst["aabb_max"] = (c + rng.random((n, 3)) * 3.0).astype(np.float32)
    inst["world_to_local"] = np.eye(4, dtype=np.float32).reshape(16)
    if n > 3:
        inst[2] = inst[1]   # a duplicate box exercises the first-minimum tie rule
    return inst


def test_noalloc_tlas_matches_allocating_build_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = wf.load()
    for call, (n, metric, seed) in enumerate([(1000, 0, 11), (5000, 1, 12)]):
        inst = random_instances(n, seed)
        with wf.Renderer(8, 8, tlas_metric=metric) as r:
            blob = r.tlas_build(inst)
        want = blob[8:8 + 64 * n]                       # the 2n tlas_node_t after the 8-byte header
        boxes = np.concatenate([inst["aabb_min"], inst["aabb_max"]], axis=1).astype(np.float32)
        d_boxes = torch.from_numpy(boxes.copy()).cuda()
        d_nodes = torch.full((16 * n,), -1.0, dtype=torch.float32, device="cuda")   # 2n nodes x 8 floats
        torch.cuda.synchronize()
        rc = L.wf_tlas_build_noalloc(ctypes.c_void_p(d_boxes.data_ptr()), n, ctypes.c_void_p(d_nodes.data_ptr()),
                                     metric, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, L.wf_last_error()
        torch.cuda.synchronize()
        got = d_nodes.cpu().numpy().view(np.uint8)
        assert np.array_equal(got, want), f"call {call}: first differing byte {np.argmax(got != want)}"


def test_noalloc_tlas_edge_sizes():
    """No instance (exactly one zero node is written), one instance (the walk
    has nothing to pair) and the full static capacity of 8192 instances."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = wf.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, metric, seed in [(0, 0, 0), (1, 0, 21), (8192, 0, 22), (1, 1, 23)]:
        d_nodes = torch.full((16 * max(n, 1),), -1.0, dtype=torch.float32, device="cuda")
        if n == 0:
            rc = L.wf_tlas_build_noalloc(None, 0, ctypes.c_void_p(d_nodes.data_ptr()), metric, stream)
            assert rc == 0, L.wf_last_error()
            torch.cuda.synchronize()
            got = d_nodes.cpu().numpy()
            assert np.all(got[:8].view(np.uint32) == 0) and np.all(got[8:] == -1.0)
            continue
        inst = random_instances(n, seed)
        with wf.Renderer(8, 8, tlas_metric=metric) as r:
            want = r.tlas_build(inst)[8:8 + 64 * n]
        boxes = np.concatenate([inst["aabb_min"], inst["aabb_max"]], axis=1).astype(np.float32)
        d_boxes = torch.from_numpy(boxes.copy()).cuda()
        torch.cuda.synchronize()
        rc = L.wf_tlas_build_noalloc(ctypes.c_void_p(d_boxes.data_ptr()), n, ctypes.c_void_p(d_nodes.data_ptr()),
                                     metric, stream)
        assert rc == 0, L.wf_last_error()
        torch.cuda.synchronize()
        got = d_nodes.cpu().numpy().view(np.uint8)
        assert np.array_equal(got, want), f"n={n}: first differing byte {np.argmax(got != want)}"


def test_noalloc_rejects_more_than_its_static_capacity():
    L = wf.load()
    rc = L.wf_tlas_build_noalloc(ctypes.c_void_p(16), 8193, ctypes.c_void_p(16), 0, None)
    assert rc == -3 and b"8192" in L.wf_last_error()
