"""GPU: failure detection without a GPU fault.

Faults are injected on the host side of the device work: an iteration budget
of the batched pipeline's device loop too small to finish (the loop stops on
its own and reports WF_ERR_TIMEOUT through the status word), and a device
memory cap too small for the render buffers (allocation refused before the
driver, WF_ERR_OOM).  After each, the same objects must work normally."""
import ctypes

import numpy as np
import pytest

import wavefrontpathtracing_gb300 as wf
from wavefrontpathtracing_gb300 import Batch, Renderer, scenes
from tests.helpers import load_scene_into

pytestmark = pytest.mark.gpu

RENDER = dict(max_bounces=4, nee=1, rr_start_depth=2)


def small_batch(r):
    meshes, descs = scenes.batch_scenes(count=3, seed=6, tri_range=(300, 2000), resolutions=(16, 24), spps=(1, 2))
    ids = [r.create_mesh_from_triangles(t, interval_count=8) for t in meshes]
    b = Batch(r)
    for d in descs:
        b.begin_scene(d.width, d.height, d.spp, d.view, d.env)
        for mesh, l2w, mat in d.instances:
            b.submit(ids[mesh], l2w, mat)
        b.end_scene()
    return b, descs


@pytest.mark.parametrize("use_graph", [1, 0])
def test_batch_iteration_budget_times_out_and_recovers(use_graph):
    with Renderer(8, 8) as r:
        b, descs = small_batch(r)
        b.set_config(capacity=1024, use_graph=use_graph)
        b.render(frame_seed=3, **RENDER)
        want = [b.read_image(k) for k in range(len(descs))]
        b.set_config(capacity=1024, use_graph=use_graph, max_iterations=2)
        with pytest.raises(wf.WFError) as e:
            b.render(frame_seed=3, **RENDER)
        assert e.value.status == -4                       # WF_ERR_TIMEOUT
        assert b.stats()["iterations"] <= 4
        b.set_config(capacity=1024, use_graph=use_graph, max_iterations=0)
        b.render(frame_seed=3, **RENDER)
        for k in range(len(descs)):
            assert np.array_equal(b.read_image(k).view(np.uint32), want[k].view(np.uint32))
        b.close()


def test_device_memory_cap_refuses_and_recovers():
    L = wf.load()
    desc = scenes.box_scene(width=64, height=64, max_bounces=3)
    try:
        with Renderer(64, 64) as r:
            load_scene_into(r, desc)
            used = ctypes.c_uint64()
            wf.check(L.wf_get_device_memory_usage(ctypes.byref(used)))
            assert used.value > 0
            wf.check(L.wf_set_device_memory_limit(used.value + 4096))   # no room for the render buffers
            with pytest.raises(wf.WFError) as e:
                r.render(max_bounces=3, spp=1)
            assert e.value.status == -2                   # WF_ERR_OOM
            with pytest.raises(wf.WFError):
                r.create_mesh_from_triangles(desc.meshes[1])
            wf.check(L.wf_set_device_memory_limit(0))
            r.render(max_bounces=3, spp=1)
            assert r.read_image()[..., :3].mean() > 0.0
        after = ctypes.c_uint64()
        wf.check(L.wf_get_device_memory_usage(ctypes.byref(after)))
        assert after.value < used.value                   # the context's memory went back
    finally:
        L.wf_set_device_memory_limit(0)


def chain_blas(depth):
    """A prebuilt BLAS whose interior nodes form a chain `depth` pairs long,
    each pair = (interior child, leaf); the interior child's box starts nearer
    along +z, so near-first traversal descends the chain and pushes one leaf
    per level.  The leaves' triangles lie off the ray x = y = 0."""
    from wavefrontpathtracing_gb300.abi import bvh_node_dtype
    n = depth + 1
    nodes = np.zeros(2 * depth + 2, dtype=bvh_node_dtype)
    nodes[0] = ((-1, -1, 0), 2, (1, 1, 10), 0)
    leaf = 0
    for k in range(1, depth + 1):
        z = 0.01 * k
        if k < depth:
            nodes[2 * k] = ((-1, -1, z), 2 * k + 2, (1, 1, 10), 0)
        else:
            nodes[2 * k] = ((-1, -1, z), leaf, (1, 1, 10), 1)
            leaf += 1
        nodes[2 * k + 1] = ((-1, -1, z + 0.005), leaf, (1, 1, 10), 1)
        leaf += 1
    assert leaf == n
    tris = np.zeros(n, dtype=scenes.triangle_dtype)
    z = 0.02 + 0.01 * np.arange(n)
    tris["v0"]["position"] = np.stack([np.full(n, 0.5), np.full(n, 0.5), z], 1)
    tris["v1"]["position"] = np.stack([np.full(n, 0.6), np.full(n, 0.5), z], 1)
    tris["v2"]["position"] = np.stack([np.full(n, 0.5), np.full(n, 0.6), z], 1)
    btri = np.concatenate([tris["v0"]["position"], tris["v1"]["position"], tris["v2"]["position"]], 1)
    btri = btri.astype(np.float32)
    hdr = np.array([12, 12 + 32 * len(nodes), 12 + 32 * len(nodes) + 36 * n], np.uint32)
    blob = np.concatenate([hdr.view(np.uint8), nodes.view(np.uint8), btri.view(np.uint8).reshape(-1),
                           np.arange(n, dtype=np.uint32).view(np.uint8)])
    return tris, blob


def test_traversal_stack_overflow_is_reported_not_trapped(orc):
    """A BLAS path deeper than the 64-entry stack: the ray that needs more
    reports a miss and the call returns WF_ERR_STACK (the oracle counts the
    same overflow); the context stays usable."""
    tris, blob = chain_blas(80)
    rays = np.zeros(2, dtype=wf.abi.ray_dtype)
    rays["origin"] = [(0.0, 0.0, -1.0), (5.0, 5.0, -1.0)]   # down the chain; wide of the root box
    rays["dir"] = (0.0, 0.0, 1.0)
    rays["tmax"] = np.finfo(np.float32).max
    from tests.helpers import single_instance_scene
    with Renderer(8, 8) as r:
        mesh = r.create_mesh_prebuilt(tris, blob)
        r.begin_scene(scenes.make_view((0.0, 0.0, -1.0), (0.0, 0.0, 1.0), 30.0, 8, 8))
        r.submit_render_mesh(mesh, np.eye(4))
        r.end_scene()
        with pytest.raises(wf.WFError) as e:
            r.trace(rays)
        assert e.value.status == -5                        # WF_ERR_STACK
        hits = r.trace(rays[1:])                           # usable afterwards
        assert hits["instance"][0] == 0xFFFFFFFF
    oi = np.zeros(1, dtype=orc.instance_dtype)
    oi["local_to_world"] = oi["world_to_local"] = np.eye(4, dtype=np.float32).reshape(16)
    _, _, overflows = orc.Scene([(tris, blob)], orc.tlas_build(single_instance_bvh(blob)), oi).trace(rays)
    assert overflows == 1


def single_instance_bvh(blob):
    from wavefrontpathtracing_gb300.abi import bvh_instance_dtype
    inst = np.zeros(1, dtype=bvh_instance_dtype)
    inst["world_to_local"] = np.eye(4, dtype=np.float32).reshape(16)
    root = blob[12:44].view(np.float32)
    inst["aabb_min"], inst["aabb_max"] = root[0:3], root[4:7]
    return inst
