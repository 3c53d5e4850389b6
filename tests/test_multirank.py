"""CPU: the multi-rank bench path (one process per GPU under torchrun), run as
two gloo ranks on the host.

Paths are independent, so ranks never exchange path data: each renders its own
frames (distinct seeds) and only the timing is reduced — the job time is the
slowest rank's and the job's rays are every rank's (weak scaling)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    r, w, local = bench.dist_env()
    dist = bench.init_pg(w)
    try:
        gpu_ms = [40.0, 55.0][rank]          # rank 1 is the slow one
        rays = [1_000_000, 3_000_000][rank]
        t_max, rays_all, value = bench.aggregate_weak(dist, gpu_ms, rays)
        bench.barrier(dist)
        seeds = [bench.frame_seed(i, r) for i in range(4)]
        q.put((r, local, t_max, rays_all, value, seeds))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_timing_only():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (r, local, t_max, rays_all, value, seeds) in enumerate(out):
        assert r == rank and local == rank
        assert t_max == 55.0                     # slowest rank
        assert rays_all == 4_000_000             # every rank's rays
        assert value == pytest.approx(4_000_000 / 0.055 / 1e6)
    s0, s1 = out[0][5], out[1][5]
    assert len(set(s0) | set(s1)) == 8           # no frame seed shared between ranks


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.init_pg(1) is None
    t_max, rays_all, value = bench.aggregate_weak(None, 20.0, 2_000_000)
    assert (t_max, rays_all) == (20.0, 2_000_000) and value == pytest.approx(100.0)
