"""Benchmark: path-traced Mrays/s and spp/s at 1080p on the instanced scene.

Workload (one step = one frame): the instanced configuration — 8 noise-
displaced icospheres (1.70M unique triangles), 1,024 random instances
(217.6M instanced triangles) plus one area light, 60/25/15 % Lambert / GGX
metal / dielectric, 1920x1080, 16 samples per pixel, max depth 8, Russian
roulette from depth 3, next-event estimation through the connect stage.

Our arm (default): value = (extension + shadow rays) / GPU time of the K
timed frames (CUDA events recorded by the library on its own stream around
each frame); e2e = the same metric through the C ABI with host buffers — per
frame the scene is re-submitted (1,025 instances, TLAS rebuilt on the GPU, as
the reference rebuilds its TLAS every frame, renderer.cpp:637-669) and the
1080p RGBA float image is read back to the host, frames pipelined as a
real-time caller keeps them in flight (the next scene submitted during a
render, each image copied during the next render, the last copy waited for).

Beside the headline: the roofline per depth (extension and shadow-ray
launches, algorithmic bytes of an instrumented pass over the timed CUDA-event
time of each depth's launch) and over the secondary depths alone; the same
frame with the reference's TLAS (tlas_metric 0); the CPU baseline with the
reference TLAS and with the GPU line's own TLAS on the same pixels; the traversal
micro-benchmark at 4.2M rays per set (closest / any hit, coherent /
incoherent, as given / Morton-ordered, with its CPU baseline); the plain small,
differentiable and batched configurations; the megakernel A/B.

Reference arm (--impl reference): the reference's algorithm on the host CPU
cores: the oracle's restatement of its builders, traversal and shading
(reference TLAS metric), all threads, each step a bounded sample of pixels of
the same frame.

Prints one JSON line (rank 0).  Multi-GPU (torchrun): each rank renders its
own frame (different seeds), weak scaling, max time over ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s & spp/s @1080p vs plain wavefront; adjoint grad-spp/s; % HBM peak"
WORKLOAD = "instanced scene 1920x1080, 16 spp, max depth 8, RR from 3, NEE"
W, H, SPP, DEPTH, RR = 1920, 1080, 16, 8, 3
L2_BYTES = 256 << 20
# algorithmic bytes per extend ray, reference layouts: ray 32 + hit 20, and per
# fetch: TLAS node 32, bvh_instance_t 92, BLAS node 32, triangle 36 + index 4
B_RAY, B_HIT, B_TNODE, B_INST, B_BNODE, B_TRI = 32, 20, 32, 92, 32, 40
B_SRAY = 32   # a shadow ray's origin/tmax and direction/path (its contribution is read only when unoccluded)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_pg(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate_weak(dist, gpu_ms, rays):
    """Weak scaling: every rank traced its own frames; the job took the slowest
    rank's time and processed every rank's rays.  Returns (max ms, total rays,
    Mrays/s of the whole job)."""
    t_max = max_over_ranks(dist, gpu_ms)
    rays_all = sum_over_ranks(dist, rays)
    return t_max, rays_all, rays_all / (t_max / 1e3) / 1e6


def frame_seed(step, rank):
    """Distinct frame seeds per rank, so ranks render different samples."""
    return 1 + step + 7919 * rank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.p, self.path = device, None, None

    def __enter__(self):
        try:
            # the raw samples go to $WF_CLOCKS_DIR (default: the system's temporary directory)
            d = os.environ.get("WF_CLOCKS_DIR") or tempfile.gettempdir()
            os.makedirs(d, exist_ok=True)
            self.path = os.path.join(d, f"clocks_{os.getpid()}.csv")
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(rays_per_launch):
    """DRAM bytes per extension launch from the committed ncu summary
    (profiles/extend_instanced_1080p.json: read + written bytes per ray over
    the nine extension launches of a reduced frame, and the git commit it was
    captured at), scaled to this frame's rays per launch."""
    p = os.path.join(ROOT, "profiles", "extend_instanced_1080p.json")
    if not os.path.exists(p):
        return None, None
    d = json.load(open(p))
    if "dram_bytes_per_ray" in d:
        return int(d["dram_bytes_per_ray"] * rays_per_launch), {
            "file": "profiles/extend_instanced_1080p.json", "commit": d.get("commit"),
            "captured": d.get("workload"), "dram_bytes_per_ray": d["dram_bytes_per_ray"]}
    return d.get("dram_bytes_per_launch"), {"file": "profiles/extend_instanced_1080p.json", "commit": d.get("commit")}


# Instance world boxes of the main frame (wf_init_params.instance_bounds).
DEFAULT_INSTANCE_BOUNDS = 1
# Shadow rays traced with the next depth's extension rays from this depth on
# (wf_render_options.fused_from_depth): 2 measured 1 % faster than 0 on the frame.
DEFAULT_FUSED_FROM_DEPTH = 2


def tlas_reference_leg(local, desc, steps, torch, l2buf):
    """The benchmark frame on the GPU with the reference's TLAS (tlas_metric
    0: its agglomerative walk and pairing metric, tlas_builder.cpp:6-110)
    instead of the clustering build: rays/s and TLAS node loads per extension
    ray, to separate the TLAS's share of the speed-up from the kernels'."""
    import wavefrontpathtracing_gb300 as wf
    kw = dict(max_bounces=DEPTH, spp=SPP, nee=1, rr_start_depth=RR, accumulate=False)
    with wf.Renderer(W, H, device=local, tlas_metric=0) as r0:
        build_scene(r0, desc)
        for i in range(2):
            r0.render(frame_seed=500 + i, profile=True, **kw)
        ms, rays = 0.0, 0
        for i in range(steps):
            flush_l2(torch, l2buf)
            if torch is not None:
                torch.cuda.synchronize()
            r0.render(frame_seed=frame_seed(i, 0), profile=True, **kw)
            st = r0.stats()
            ms += st["ms_total"]
            rays += st["rays_extend"] + st["rays_connect"]
        r0.render(frame_seed=1, count_traffic=True, **kw)
        c0 = r0.stats()
    return {"tlas_metric": "reference", "value": round(rays / (ms / 1e3) / 1e6, 3), "unit": "Mrays/s",
            "ms_per_step": round(ms / steps, 3), "steps": steps,
            "spp_per_s": round(SPP * steps / (ms / 1e3), 3),
            "tlas_node_loads_per_ray": round(c0["tlas_node_loads"] / max(1, c0["rays_extend"]), 1)}


def build_scene(r, desc):
    from tests.helpers import load_scene_into
    return load_scene_into(r, desc)


def oracle_scene(desc):
    """Oracle scene for the CPU legs, from the oracle's own builders with the
    reference's TLAS metric (untimed)."""
    from oracle import oracle as orc
    from tests.helpers import oracle_scene_from_desc
    return oracle_scene_from_desc(orc, desc)


CPU_BANDS = 8


def cpu_sample(sc, desc, seconds, threads, seed, n=None):
    """Renders CPU_BANDS bands of consecutive pixels spread evenly over the
    frame (band k centred on pixel (k + 1/2) W H / CPU_BANDS) on the host, about
    `seconds` of work in all, calibrated by a short first pass unless n (the
    pixel count) is given.  Returns (Mrays/s, description, rays, seconds, n)."""
    npix = W * H

    def run(n):
        nb = max(1, n // CPU_BANDS)
        rays, t = 0, 0.0
        for k in range(CPU_BANDS):
            p0 = min(npix - nb, max(0, int((k + 0.5) * npix / CPU_BANDS) - nb // 2))
            t0 = time.perf_counter()
            _, st = sc.render(desc.view, W, H, max_bounces=DEPTH, spp=SPP, frame_seed=seed, nee=1,
                              rr_start_depth=RR, threads=threads, pixel_range=(p0, p0 + nb))
            t += time.perf_counter() - t0
            rays += sum(st["extend_rays"]) + sum(st["shadow_rays"])
        return rays, t, nb * CPU_BANDS

    if n is None:
        # calibrate on a pass of at least a tenth of the target (each call has
        # a fixed start-up cost that a tiny pass would overweight)
        n = 2048
        while True:
            rays, dt, m = run(n)
            if dt >= 0.1 * seconds or n >= npix:
                break
            n = min(npix, n * 4)
        n = int(min(npix, max(n, n * seconds / max(dt, 1e-3))))
    rays, dt, n = run(n)
    return (rays / dt / 1e6, f"{n} pixels x {SPP} spp of the 1920x1080 frame in {CPU_BANDS} bands spread over it "
            f"({rays} rays, {dt:.1f} s)", rays, dt, n)


def run_reference(args, rank, world):
    dist = init_pg(world)
    if rank != 0:
        return
    from wavefrontpathtracing_gb300 import scenes
    desc = scenes.instanced_scene(width=W, height=H, spp=SPP, max_bounces=DEPTH)
    sc = oracle_scene(desc)
    threads = os.cpu_count() or 1
    per_step = max(3.0, min(20.0, 150.0 / max(1, args.steps + args.warmup)))
    for i in range(args.warmup):
        cpu_sample(sc, desc, per_step, threads, seed=100 + i)
    rays_total, t_total, desc_s = 0, 0.0, ""
    for i in range(args.steps):
        _, desc_s, rays, dt, _ = cpu_sample(sc, desc, per_step, threads, seed=1 + i)
        rays_total += rays
        t_total += dt
    v = rays_total / t_total / 1e6
    line = {"metric": METRIC, "value": round(v, 3), "unit": "Mrays/s", "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * t_total / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene)",
            "config": {"workload": WORKLOAD, "tlas_metric": "reference", "sample": desc_s},
            "cpu_baseline": {"value": round(v, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": desc_s},
            "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def adjoint_leg(device, tlas_metric):
    """Differentiable configuration: box scene (20,506 triangles) at 512x512,
    64 spp, depth 6; per-triangle albedo 0.5, emitter strength 10, L2 loss to a
    target rendered with albedo U[0.1, 0.9] (seed 2).  Returns forward and
    adjoint samples per pixel per second (GPU time, CUDA events)."""
    import wavefrontpathtracing_gb300 as wf
    from wavefrontpathtracing_gb300 import scenes
    from tests.helpers import load_scene_into
    w = h = 512
    spp, depth, seed = 64, 6, 5
    desc = scenes.box_scene(width=w, height=h, max_bounces=depth)
    with wf.Renderer(w, h, device=device, tlas_metric=tlas_metric) as r:
        load_scene_into(r, desc)
        n = r.scene_triangle_count()
        rng = np.random.default_rng(2)
        r.set_albedo(rng.uniform(0.1, 0.9, (n, 3)).astype(np.float32))
        r.render(max_bounces=depth, spp=spp, frame_seed=seed, accumulate=False)
        target = r.read_image()[..., :3]
        r.set_albedo(np.full((n, 3), 0.5, np.float32))
        r.set_emission(2, 10.0)
        fwd, adj = [], []
        for it in range(3):
            r.render(max_bounces=depth, spp=spp, frame_seed=seed, accumulate=False, profile=False)
            img = r.read_image()[..., :3]
            fwd.append(r.stats()["ms_total"])
            r.adjoint(2.0 * (img - target), max_bounces=depth, spp=spp, frame_seed=seed)
            adj.append(r.stats()["ms_total"])
        f_ms, a_ms = min(fwd[1:]), min(adj[1:])
        return {"config": "box scene 512x512, 64 spp, depth 6, 20,506 per-triangle albedos + emitter strength",
                "forward_spp_per_s": round(spp / (f_ms / 1e3), 2), "grad_spp_per_s": round(spp / (a_ms / 1e3), 2),
                "ratio": round(f_ms / a_ms, 3), "forward_ms": round(f_ms, 3), "adjoint_ms": round(a_ms, 3)}


def batched_leg(device, tlas_metric, steps=3, count=64, config=None):
    """Batched configuration: 64 scenes (displaced icosphere soups, triangles
    log-uniform in [1k, 2M]; square images of side 64..1024; spp 1, 4 or 16;
    depth 6, NEE, RR from 3) rendered as one batch (one CUDA-graph launch, pool
    parameters from the autotuner) against the same 64 scenes rendered one
    after another with wf_render (the plain single-scene wavefront loop).  Both
    sides are timed on the device with CUDA events; the plain side is the sum
    of the 64 renders' GPU times.  Camera paths per second over all scenes.
    config: (capacity, regeneration threshold, block[, use_graph]) to use
    instead of the autotuner's choice (profiling captures; use_graph 0 = the
    host loop, the same kernels launched one by one)."""
    import wavefrontpathtracing_gb300 as wf
    from wavefrontpathtracing_gb300 import scenes
    depth, rr, seed = 6, 3, 11
    t_gen = time.perf_counter()
    meshes, descs = scenes.batch_scenes(count=count)
    gen_s = time.perf_counter() - t_gen
    paths = sum(d.paths for d in descs)
    kw = dict(max_bounces=depth, nee=1, rr_start_depth=rr)
    out = {"config": f"{count} scenes, {sum(len(m) for m in meshes[2:])} soup triangles "
                     f"(per scene {min(d.sphere_triangles for d in descs)}..{max(d.sphere_triangles for d in descs)}), "
                     f"{paths} camera paths, depth {depth}, NEE, RR from {rr}",
           "scene_generation_s": round(gen_s, 1)}
    # --- batched
    with wf.Renderer(8, 8, device=device, tlas_metric=tlas_metric) as r:
        ids = [r.create_mesh_from_triangles(t, interval_count=16, max_leaf_prims=4) for t in meshes]
        b = wf.Batch(r)
        for d in descs:
            b.begin_scene(d.width, d.height, d.spp, d.view, d.env)
            for mesh, l2w, mat in d.instances:
                b.submit(ids[mesh], l2w, mat)
            b.end_scene()
        t_tune = time.perf_counter()
        if config is None:
            cfg = b.autotune(frame_seed=seed, **kw)
        else:
            b.set_config(capacity=int(config[0]), regen_threshold=float(config[1]), block=int(config[2]),
                         use_graph=int(config[3]) if len(config) > 3 else 1)
            cfg = b.config()
        tune_s = time.perf_counter() - t_tune
        bms, bst = [], None
        for i in range(steps):
            b.render(frame_seed=seed, **kw)
            bst = b.stats()
            bms.append(bst["ms_total"])
        sample = [b.read_image(k) for k in (0, count // 2, count - 1)]
        b.close()
    # --- plain: one wf_render per scene, one context per image size
    pms = [0.0] * steps
    plain_rays = 0
    plain_launches = 0
    equal = True
    for side in sorted({d.width for d in descs}):
        group = [(k, d) for k, d in enumerate(descs) if d.width == side]
        with wf.Renderer(side, side, device=device, tlas_metric=tlas_metric) as r:
            mid = {}
            for k, d in group:
                for mesh, _, _ in d.instances:
                    if mesh not in mid:
                        mid[mesh] = r.create_mesh_from_triangles(meshes[mesh], interval_count=16, max_leaf_prims=4)
            for k, d in group:
                r.begin_scene(d.view, d.env)
                for mesh, l2w, mat in d.instances:
                    r.submit_render_mesh(mid[mesh], l2w, mat)
                r.end_scene()
                r.render(spp=d.spp, frame_seed=seed, accumulate=False, **kw)   # warm-up
                for i in range(steps):
                    r.render(spp=d.spp, frame_seed=seed, accumulate=False, **kw)
                    st = r.stats()
                    pms[i] += st["ms_total"]
                    if i == 0:
                        plain_rays += st["rays_extend"] + st["rays_connect"]
                        plain_launches += st["launches"]
                if k in (0, count // 2, count - 1):
                    img = r.read_image()
                    equal = equal and bool(np.array_equal(img.view(np.uint32),
                                                          sample[(0, count // 2, count - 1).index(k)].view(np.uint32)))
    b_ms, p_ms = min(bms), min(pms)
    rays = bst["rays_extend"] + bst["rays_connect"]
    out.update({"autotuned": cfg, "autotune_s": round(tune_s, 1),
                "batched_ms": round(b_ms, 3), "plain_ms": round(p_ms, 3),
                "speedup_vs_plain": round(p_ms / b_ms, 3),
                "batched_spp_per_s": round(paths / (b_ms / 1e3), 1), "plain_spp_per_s": round(paths / (p_ms / 1e3), 1),
                "batched_mrays_per_s": round(rays / (b_ms / 1e3) / 1e6, 1),
                "plain_mrays_per_s": round(plain_rays / (p_ms / 1e3) / 1e6, 1),
                "rays_equal": rays == plain_rays, "images_equal_sampled": equal,
                "iterations": bst["iterations"], "graph_launches": bst["graph_launches"],
                "device_kernels": bst["kernel_launches"], "plain_launches": plain_launches})
    return out


def builders_leg(r, desc):
    """BLAS build of the largest instanced mesh and TLAS build of the 1,025
    instance boxes: the GPU builders through the C ABI (host arrays in, blob
    out) against the oracle's restatement of the reference's single-threaded
    C++ builders (byte-identical output)."""
    from oracle import oracle as orc
    tris = max(desc.meshes, key=len)
    t0 = time.perf_counter()
    g = r.bvh_build(tris, interval_count=16, max_leaf_prims=4)
    gpu_blas = time.perf_counter() - t0
    t0 = time.perf_counter()
    c = orc.bvh_build(tris, 16, False, 4)
    cpu_blas = time.perf_counter() - t0
    inst = r.scene_instances()
    out = {"mesh_triangles": len(tris), "gpu_blas_ms": round(1e3 * gpu_blas, 2), "cpu_blas_ms": round(1e3 * cpu_blas, 1),
           "blas_equal": bool(np.array_equal(g, c)), "tlas_instances": len(inst)}
    t0 = time.perf_counter()
    ct = orc.tlas_build(inst, metric=0)
    out["cpu_tlas_reference_ms"] = round(1e3 * (time.perf_counter() - t0), 2)
    for metric, name in ((0, "reference"), (2, "clustering"), (3, "sah_sweep")):
        import wavefrontpathtracing_gb300 as wf
        with wf.Renderer(8, 8, tlas_metric=metric) as q:
            q.tlas_build(inst)                          # warm-up (module load, allocation)
            t0 = time.perf_counter()
            gt = q.tlas_build(inst)
            out[f"gpu_tlas_{name}_ms"] = round(1e3 * (time.perf_counter() - t0), 3)
        if metric == 0:
            out["tlas_equal"] = bool(np.array_equal(gt, ct))
    return out


def plain_small_leg(device, tlas_metric):
    """The plain small configuration: box of 12 quads + icosphere (subdivision
    5, radius 0.3) + emissive ceiling quad, 20,506 triangles; 256x256, 1 spp,
    depth 4, Lambert only, no NEE.  GPU frame time (CUDA events, best of 5)
    against the oracle's port of the reference's CPU path on all host cores
    for the same frame (scene from the GPU's own blobs), the images compared
    bit for bit; BLAS builds of its meshes on the GPU (through the C ABI) and
    by the oracle's restatement of the reference's single-threaded builder."""
    import wavefrontpathtracing_gb300 as wf
    from wavefrontpathtracing_gb300 import scenes
    from oracle import oracle as orc
    from tests.helpers import oracle_scene_from_renderer
    orc.build()
    desc = scenes.box_scene(width=256, height=256, max_bounces=4)
    o = desc.bvh_options
    with wf.Renderer(256, 256, device=device, tlas_metric=tlas_metric) as r:
        t0 = time.perf_counter()
        ids = [r.create_mesh_from_triangles(t, interval_count=o["interval_count"], max_leaf_prims=o["max_leaf_prims"])
               for t in desc.meshes]
        gpu_build_ms = (time.perf_counter() - t0) * 1e3
        r.begin_scene(desc.view, desc.settings["env"])
        for mesh, l2w, mat in desc.instances:
            r.submit_render_mesh(ids[mesh], l2w, mat)
        r.end_scene()
        ms = []
        for i in range(6):
            r.render(max_bounces=4, spp=1, frame_seed=1, accumulate=False)
            ms.append(r.stats()["ms_total"])
        st = r.stats()
        img = r.read_image()
        sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
    t0 = time.perf_counter()
    for t in desc.meshes:
        orc.bvh_build(t, o["interval_count"], False, o["max_leaf_prims"])
    cpu_build_ms = (time.perf_counter() - t0) * 1e3
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    acc, ost = sc.render(desc.view, 256, 256, max_bounces=4, spp=1, frame_seed=1, threads=threads)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    want = np.zeros_like(acc)
    want[..., :3] = acc[..., :3] / acc[..., 3:]
    want[..., 3] = acc[..., 3]
    rays = st["rays_extend"] + st["rays_connect"]
    gpu_ms = min(ms[1:])
    return {"config": f"box scene 256x256, 1 spp, depth 4, {desc.triangle_count} triangles, Lambert, no NEE",
            "gpu_ms": round(gpu_ms, 3), "gpu_mrays_per_s": round(rays / (gpu_ms / 1e3) / 1e6, 1),
            "cpu_ms": round(cpu_ms, 1), "cpu_mrays_per_s": round(sum(ost["extend_rays"]) / (cpu_ms / 1e3) / 1e6, 2),
            "cpu_cores": threads, "cpu_kind": "port",
            "images_equal": bool(np.array_equal(img.view(np.uint32), want.view(np.uint32))),
            "gpu_blas_build_ms": round(gpu_build_ms, 2), "cpu_blas_build_ms": round(cpu_build_ms, 2)}


def flush_l2(torch, buf):
    if buf is not None:
        buf.add_(1)


def run_ours(args, rank, world, local):
    dist = init_pg(world)
    import wavefrontpathtracing_gb300 as wf
    from wavefrontpathtracing_gb300 import scenes
    try:
        import torch
        torch.cuda.set_device(local)
        l2buf = torch.zeros(L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")
    except Exception:
        torch, l2buf = None, None
    desc = scenes.instanced_scene(width=W, height=H, spp=SPP, max_bounces=DEPTH)
    r = wf.Renderer(W, H, device=local, tlas_metric=args.tlas_metric, blas_layout=args.blas_layout,
                    instance_bounds=args.instance_bounds)
    ids = build_scene(r, desc)

    def frame(seed, profile):
        r.render(max_bounces=DEPTH, spp=SPP, frame_seed=seed, nee=1, rr_start_depth=RR, accumulate=False,
                 profile=profile, fused_connect=args.fused_connect, tail_paths=args.tail_paths,
                 fused_from_depth=args.fused_from_depth)
        return r.stats()

    for i in range(args.warmup):
        frame(1000 + i + 97 * rank, True)
    r.synchronize()
    # --- device-resident timing
    barrier(dist)
    gpu_ms, rays, launches, ext_ms, ext_launches = 0.0, 0, 0, 0.0, 0
    ext_depth_ms, con_depth_ms = np.zeros(16), np.zeros(16)
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush_l2(torch, l2buf)
            if torch is not None:
                torch.cuda.synchronize()
            s = frame(frame_seed(i, rank), True)
            last = s
            gpu_ms += s["ms_total"]
            rays += s["rays_extend"] + s["rays_connect"]
            launches += s["launches"]
            ext_ms += s["ms_extend"]
            ext_launches += s["launches_extend"]
            ext_depth_ms += np.array(s["ms_extend_depth"])
            con_depth_ms += np.array(s["ms_connect_depth"])
        r.synchronize()
    barrier(dist)
    t_max, rays_all, value = aggregate_weak(dist, gpu_ms, rays)
    spp_per_s = world * SPP * args.steps / (t_max / 1e3)
    # --- solo launch times (untimed): frames with the shadow rays on the main
    # stream, so that no extension and shadow-ray launches overlap and each
    # launch's CUDA-event time is its own
    SOLO = 3
    solo_ext, solo_con = np.zeros(16), np.zeros(16)
    if not args.fused_connect:
        for i in range(SOLO):
            flush_l2(torch, l2buf)
            r.render(max_bounces=DEPTH, spp=SPP, frame_seed=frame_seed(i, rank), nee=1, rr_start_depth=RR,
                     accumulate=False, profile=True, serial_connect=True, tail_paths=args.tail_paths)
            so = r.stats()
            solo_ext += np.array(so["ms_extend_depth"])
            solo_con += np.array(so["ms_connect_depth"])
    # --- megakernel A/B (use_wavefront_pathtracing = 0): the same frame, whole paths per thread
    mega = None
    if not args.no_megakernel:
        mms = []
        for i in range(3):
            r.render(max_bounces=DEPTH, spp=SPP, frame_seed=frame_seed(i, rank), nee=1, rr_start_depth=RR,
                     accumulate=False, megakernel=True)
            mms.append(r.stats()["ms_total"])
        m_ms = min(mms[1:])
        mega = {"ms_per_frame": round(m_ms, 3), "spp_per_s": round(SPP / (m_ms / 1e3), 2),
                "wavefront_ms_per_frame": round(t_max / args.steps, 3),
                "wavefront_speedup": round(m_ms / (t_max / args.steps), 3)}
    # --- algorithmic bytes of the extend kernel (counted pass, same seeds, untimed)
    r.render(max_bounces=DEPTH, spp=SPP, frame_seed=1, nee=1, rr_start_depth=RR, accumulate=False,
             count_traffic=True)
    c = r.stats()
    alg_bytes = (c["rays_extend"] * (B_RAY + B_HIT) + c["tlas_node_loads"] * B_TNODE + c["instance_loads"] * B_INST
                 + c["blas_node_loads"] * B_BNODE + c["triangle_tests"] * B_TRI)
    alg_bytes -= c["paths"] * B_RAY   # camera rays are made in the depth-0 launch, not read
    def shadow_bytes(d):
        """Algorithmic bytes of the shadow rays of depth d (the counted pass)."""
        f = c["shadow_fetch_depth"][d]
        return (int(c["shadow_rays_depth"][d]) * B_SRAY + f[0] * B_TNODE + f[1] * B_INST + f[2] * B_BNODE
                + f[3] * B_TRI)

    # from this depth on, an extension launch also traces the previous depth's shadow rays
    fuse_from = 1 if args.fused_connect else args.fused_from_depth
    if fuse_from:
        alg_bytes += sum(shadow_bytes(d - 1) for d in range(max(1, fuse_from), DEPTH + 1))
    # the launches measured are the staged extension launches: with a tail, the
    # rays of its depths (under 1 % of them on this frame) leave the count
    tail_d = int(last["tail_depth"])
    if tail_d:
        q = [int(x) for x in c["extend_rays_depth"][:DEPTH + 1]]
        alg_bytes = alg_bytes * sum(q[:tail_d]) / max(1, sum(q))
    bytes_per_launch = alg_bytes / max(1, ext_launches / args.steps)
    ms_per_launch = ext_ms / max(1, ext_launches)
    achieved = bytes_per_launch / (ms_per_launch / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic, traffic_src = ncu_traffic(c["rays_extend"] / max(1, ext_launches / args.steps))
    # per depth: the extension launches (depth 0 makes its camera rays) and the
    # shadow-ray launches, algorithmic bytes of the counted pass over the
    # timed frames' CUDA-event time of that depth's launch
    def depth_rows(ext_ms_d, con_ms_d, frames, fuse_live):
        """Per depth: rays, algorithmic bytes (the counted pass) and the
        CUDA-event time of the extension / shadow-ray launch of that depth
        (fuse_live: the frames fused shadow rays into the extension launches)."""
        ext_rows, con_rows = [], []
        for d in range(DEPTH + 1):
            n_d, f = int(c["extend_rays_depth"][d]), c["extend_fetch_depth"][d]
            ms_d = ext_ms_d[d] / frames
            if n_d and ms_d > 0:
                b = (n_d * (B_HIT + (0 if d == 0 else B_RAY)) + f[0] * B_TNODE + f[1] * B_INST + f[2] * B_BNODE
                     + f[3] * B_TRI)
                fused = fuse_live and fuse_from and d >= max(1, fuse_from)
                if fused:
                    b += shadow_bytes(d - 1)   # the launch also traced the shadow rays of depth d - 1
                ext_rows.append({"depth": d, "rays": n_d, "alg_bytes": int(b), "ms": round(ms_d, 4),
                                 **({"with_shadow_rays_of_depth": d - 1} if fused else {}),
                                 "achieved_gbs": round(b / (ms_d / 1e3) / 1e9, 1),
                                 "frac": round(b / (ms_d / 1e3) / 1e9 / peak, 4),
                                 "fetches_per_ray": round((f[0] + f[2]) / n_d, 1)})
            n_s, f = int(c["shadow_rays_depth"][d]), c["shadow_fetch_depth"][d]
            ms_s = con_ms_d[d] / frames
            if d < DEPTH and n_s and ms_s > 0:
                b = n_s * B_SRAY + f[0] * B_TNODE + f[1] * B_INST + f[2] * B_BNODE + f[3] * B_TRI
                con_rows.append({"depth": d, "rays": n_s, "alg_bytes": int(b), "ms": round(ms_s, 4),
                                 "frac": round(b / (ms_s / 1e3) / 1e9 / peak, 4)})
        return ext_rows, con_rows

    def total(rows):
        b, t = sum(x["alg_bytes"] for x in rows), sum(x["ms"] for x in rows)
        return {"alg_bytes": int(b), "ms": round(t, 4), "achieved_gbs": round(b / (t / 1e3) / 1e9, 1) if t else None,
                "frac": round(b / (t / 1e3) / 1e9 / peak, 4) if t else None}

    per_depth, secondary, connect, solo = None, None, None, None
    if not args.fused_connect:
        # the timed frames (shadow rays overlapping the next depth's extension
        # rays on a second stream, so each launch's time includes the other's
        # competition) ...
        per_depth, con = depth_rows(ext_depth_ms, con_depth_ms, args.steps, True)
        secondary = total([x for x in per_depth if x["depth"] >= 1])
        connect = {"launches": con, **total(con)}
        # ... and the solo frames (every launch alone)
        s_ext, s_con = depth_rows(solo_ext, solo_con, SOLO, False)
        solo = {"frames": SOLO, "schedule": "shadow rays on the main stream after shade (no overlap)",
                "extend_per_depth": s_ext, "extend": total(s_ext),
                "extend_secondary": total([x for x in s_ext if x["depth"] >= 1]),
                "connect_per_depth": s_con, "connect": total(s_con)}
    # --- end to end through the C ABI with host buffers: every frame submits
    # its instances (host arrays), rebuilds the TLAS, renders and copies the
    # image to the host.  Frames are pipelined as a real-time caller runs
    # them: frame i's scene is submitted while frame i - 1 renders, its image
    # is copied on the copy stream while frame i + 1 renders (into page-locked
    # host images: a pageable buffer's copy speed depends on the host's page
    # state, 1-60 GB/s on the same box), and the last copies are waited for
    # inside the timed region.  With F frames in flight (--frames-in-flight,
    # default 2) consecutive frames go to F contexts of the same scene in
    # turn, one per frame in flight (each context has its own streams and
    # buffers), so one frame's nearly idle deep depths overlap the next
    # frame's first depths; F = 1 is also timed and reported.
    def e2e_loop(ctxs, insts, imgs, steps):
        rays, pending = 0, [False] * len(ctxs)
        b0 = [c.stats() for c in ctxs]
        barrier(dist)
        t0 = time.perf_counter()
        for i in range(steps):
            k = i % len(ctxs)
            c = ctxs[k]
            c.begin_scene(desc.view, desc.settings["env"])
            c.submit_render_meshes(*insts[k])
            c.end_scene()
            if pending[k]:   # this context's previous frame, read before its render resets the counters
                s = c.stats()
                rays += s["rays_extend"] + s["rays_connect"]
            c.render(max_bounces=DEPTH, spp=SPP, frame_seed=frame_seed(i, rank), nee=1, rr_start_depth=RR,
                     accumulate=False, fused_connect=args.fused_connect, tail_paths=args.tail_paths,
                     fused_from_depth=args.fused_from_depth)
            c.read_image_async(imgs[k])
            pending[k] = True
        for k, c in enumerate(ctxs):
            c.synchronize()
            if pending[k]:
                s = c.stats()
                rays += s["rays_extend"] + s["rays_connect"]
        dt = max_over_ranks(dist, time.perf_counter() - t0)
        b1 = [c.stats() for c in ctxs]
        h2d = sum(b["h2d_bytes"] - a["h2d_bytes"] for a, b in zip(b0, b1)) // max(1, steps)
        d2h = sum(b["d2h_bytes"] - a["d2h_bytes"] for a, b in zip(b0, b1)) // max(1, steps)
        return sum_over_ranks(dist, rays) / dt / 1e6, h2d, d2h

    def scene_arrays(ids_):
        return (np.array([ids_[m] for m, _, _ in desc.instances], dtype=np.uint32),
                np.stack([np.asarray(t, dtype=np.float32) for _, t, _ in desc.instances]),
                np.array([m for _, _, m in desc.instances], dtype=wf.abi.material_ext_dtype))

    e2e_value = e2e_single = None
    h2d = d2h = 0
    fif = max(1, args.frames_in_flight)
    if not args.no_e2e:
        imgs = [torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True).numpy() if torch is not None
                else np.zeros((H, W, 4), dtype=np.float32) for _ in range(fif)]
        e2e_single, h2d, d2h = e2e_loop([r], [scene_arrays(ids)], imgs[:1], args.steps)
        e2e_value = e2e_single
        if fif > 1:
            extra = []
            for _ in range(fif - 1):
                rx = wf.Renderer(W, H, device=local, tlas_metric=args.tlas_metric, blas_layout=args.blas_layout,
                                 instance_bounds=args.instance_bounds)
                extra.append((rx, build_scene(rx, desc)))
            ctxs = [r] + [x for x, _ in extra]
            insts = [scene_arrays(ids)] + [scene_arrays(i_) for _, i_ in extra]
            e2e_loop(ctxs, insts, imgs, fif)   # each context's buffers allocated, untimed
            e2e_value, h2d, d2h = e2e_loop(ctxs, insts, imgs, args.steps)
            for x, _ in extra:
                x.close()
    # --- CPU baseline (rank 0 only, N = 1 only): the oracle on a bounded sample
    # with the reference's TLAS (tlas_metric 0), and the same pixels with the
    # acceleration structures the GPU line traced (read back from the device)
    cpu, cpu_clustering = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sc = oracle_scene(desc)
        v, sdesc, _, _, n_px = cpu_sample(sc, desc, args.cpu_seconds, threads, seed=1)
        cpu = {"value": round(v, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": sdesc + "; reference TLAS metric"}
        from oracle import oracle as orc
        from tests.helpers import oracle_scene_from_renderer
        sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
        v2, sdesc2, _, _, _ = cpu_sample(sc, desc, args.cpu_seconds, threads, seed=1, n=n_px)
        cpu_clustering = {"value": round(v2, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                          "sample": sdesc2 + "; the GPU line's own TLAS and instance boxes"}
        del sc
    # --- builders: GPU vs the oracle's restatement of the reference's single-threaded C++ builders
    builders = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        builders = builders_leg(r, desc)
    r.close()
    # --- the same frame on the GPU with the reference's TLAS (tlas_metric 0)
    tlas_ref = None
    if rank == 0 and not args.no_tlas_reference and args.tlas_metric != 0:
        tlas_ref = tlas_reference_leg(local, desc, max(3, min(args.steps, 5)), torch, l2buf)
    # --- the traversal micro-benchmark at 4.2M rays per set
    traversal = None
    if rank == 0 and world == 1 and not args.no_traversal:
        info, res = traversal_runs(local, args.soup_triangles, 2048, max(3, min(args.steps, 5)), 3,
                                   orders=(False, True), cpu=not args.no_cpu_baseline, cpu_seconds=2.0,
                                   blas_layout=args.blas_layout)
        traversal = {"config": TRAVERSAL_CONFIG.format(n=args.soup_triangles, rays=2048 * 2048, side=2048),
                     **info, "results": res}
        if args.blas_layout == 0:
            # the DRAM-latency-bound sets again over the quantized 4-wide BLAS
            # (wf_init_params.blas_layout = 1; its algorithmic bytes are its own
            # 64-byte node fetches)
            qinfo, qres = traversal_runs(local, args.soup_triangles, 2048, max(3, min(args.steps, 5)), 3,
                                         kinds=("incoherent",), orders=(False, True), cpu=False, blas_layout=1)
            traversal["quantized_4wide"] = {"gpu_bvh_build_s": qinfo["gpu_bvh_build_s"], "results": qres}
    small = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        small = plain_small_leg(local, args.tlas_metric)
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = adjoint_leg(local, args.tlas_metric)
    batched = None
    if rank == 0 and not args.no_batched:
        batched = batched_leg(local, args.tlas_metric)
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(t_max / args.steps, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded procedural scene, no assets)",
                "config": {"workload": WORKLOAD if (W, H) == (1920, 1080) else f"{WORKLOAD} at {W}x{H}",
                           "triangles": desc.triangle_count,
                           "instanced_triangles": desc.instanced_triangle_count, "instances": len(desc.instances),
                           "tlas_metric": ["reference", "merged-box walk", "parallel clustering",
                                           "top-down SAH sweep"][args.tlas_metric],
                           "blas_layout": ["binary child pairs", "quantized 4-wide", "exact 4-wide"][args.blas_layout],
                           "instance_bounds": ["transformed BLAS root box",
                                               "BLAS frontier boxes (tight)"][args.instance_bounds],
                           "trace_schedule": ("fused" if args.fused_connect else
                                              f"separate, shadow rays fused from depth {args.fused_from_depth}"
                                              if args.fused_from_depth else "separate"),
                           "l2": "256 MiB buffer written between timed frames; working set > L2"},
                "spp_per_s": round(spp_per_s, 3),
                "rays_per_step": rays // args.steps,
                "gpu_launches": launches,
                "stages_ms": {k: round(last[f"ms_{k}"], 3) for k in ("generate", "extend", "shade", "connect", "post",
                                                                        "tail")},
                "tail_depth": int(last["tail_depth"]),
                "traversal_per_ray": {
                    "extend": {"nodes": round((c["tlas_node_loads"] + c["blas_node_loads"]) / max(1, c["rays_extend"]), 1),
                               "tlas_nodes": round(c["tlas_node_loads"] / max(1, c["rays_extend"]), 1),
                               "instances": round(c["instance_loads"] / max(1, c["rays_extend"]), 2),
                               "triangles": round(c["triangle_tests"] / max(1, c["rays_extend"]), 2)},
                    "shadow": {"nodes": round((c["shadow_tlas_node_loads"] + c["shadow_blas_node_loads"])
                                              / max(1, c["rays_connect"]), 1),
                               "tlas_nodes": round(c["shadow_tlas_node_loads"] / max(1, c["rays_connect"]), 1),
                               "instances": round(c["shadow_instance_loads"] / max(1, c["rays_connect"]), 2),
                               "triangles": round(c["shadow_triangle_tests"] / max(1, c["rays_connect"]), 2)}},
                "queue_sizes": {"extend": [int(x) for x in last["extend_rays_depth"][:DEPTH + 1]],
                                "shadow": [int(x) for x in last["shadow_rays_depth"][:DEPTH]]},
                "e2e": {"value": round(e2e_value, 3) if e2e_value else None, "unit": "Mrays/s",
                        "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                        "frames_in_flight": fif,
                        "single_context": round(e2e_single, 3) if e2e_single else None},
                "roofline": {"bound": "hbm",
                             "kernel": ("k_trace_pair (extend d + shadow rays d-1)" if args.fused_connect
                                        else f"k_trace (extend; from depth {args.fused_from_depth} with the "
                                             f"shadow rays of the previous depth)" if args.fused_from_depth
                                        else "k_trace (extend)"),
                             "achieved": round(achieved, 1),
                             "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_source": traffic_src,
                             # depth 0 carries 82 % of the rays: 16 identical camera rays per pixel share a
                             # warp, so one fetch serves 16 of them; the secondary depths are the real traversal
                             "per_depth": per_depth, "frac_secondary": secondary["frac"] if secondary else None,
                             "secondary": secondary, "connect": connect, "solo": solo,
                             "alg_bytes_per_launch": int(bytes_per_launch),
                             "ms_per_launch": round(ms_per_launch, 4),
                             # DRAM bytes actually moved (ncu, per launch) over the live launch time
                             "dram_gbs": round(traffic / (ms_per_launch / 1e3) / 1e9, 1) if traffic else None,
                             "dram_frac": round(traffic / (ms_per_launch / 1e3) / 1e9 / peak, 4) if traffic else None},
                "clocks": clk.summary()}
        if cpu:
            line["cpu_baseline"] = cpu
        if cpu_clustering:
            line["cpu_baseline_clustering_tlas"] = cpu_clustering
        if tlas_ref:
            line["gpu_reference_tlas"] = tlas_ref
        if traversal:
            line["traversal"] = traversal
        if builders:
            line["builders"] = builders
        if small:
            line["plain_small"] = small
        if adjoint:
            line["adjoint"] = adjoint
        if batched:
            line["batched"] = batched
        if mega:
            line["megakernel"] = mega
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


CPU_TRACE_SAMPLE = 200_000   # first sample of rays per set traced by the oracle for the CPU baseline
CPU_TRACE_SECONDS = 5.0      # the sample then grows to about this much CPU time
TRAVERSAL_CONFIG = ("{n} soup triangles (centroids uniform in the unit cube, log-normal edges mu=-5 sigma=0.5, "
                    "seed 7), one BLAS (16 bins, <= 4 triangles per leaf) under a 1-instance TLAS; {rays} rays per "
                    "set: coherent pinhole rays ({side}^2, camera 0.5 in front of the cube, 90-degree field of "
                    "view) and incoherent rays (origins in the cube, uniform directions); closest hit and any hit "
                    "(tmax U[0,1])")


def traversal_runs(local, n_tris, side, steps, warmup, kinds=("coherent", "incoherent"), orders=(True,),
                   cpu_seconds=CPU_TRACE_SECONDS, cpu=True, cpu_build=False, blas_layout=0):
    """Traversal micro-benchmark: n_tris soup triangles in one BLAS under a
    1-instance TLAS; side^2 rays per set.  For every ray set, query kind
    (closest / any hit) and ray order (as given / origins' Morton order,
    WF_TRACE_REORDER with the sort inside the timed call) one result: GPU time
    per call (CUDA events, L2 flushed between calls), algorithmic bytes (the
    reference layouts' fetches, counted by an instrumented pass), the
    end-to-end rate with host rays and hits, and (cpu) the oracle's port of
    the reference's scalar traversal on all host cores over a random sample of
    the set, its hits compared with the GPU's.  Returns (info, results)."""
    import torch
    import wavefrontpathtracing_gb300 as wf
    from wavefrontpathtracing_gb300 import scenes
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    tris = scenes.triangle_soup(n_tris, seed=7)
    info = {"soup_generation_s": round(time.perf_counter() - t0, 1)}
    peak, peak_kind = measured_peaks()
    results = []
    with wf.Renderer(16, 16, device=local, blas_layout=blas_layout) as r:
        t0 = time.perf_counter()
        mesh = r.create_mesh_from_triangles(tris, interval_count=16, max_leaf_prims=4)
        info["gpu_bvh_build_s"] = round(time.perf_counter() - t0, 3)
        r.begin_scene(scenes.make_view((0.5, 0.5, -0.5), (0.5, 0.5, 0.5), 90.0, 16, 16))
        r.submit_render_mesh(mesh, np.eye(4))
        r.end_scene()
        blob = r.mesh_blas(mesh)
        info["blas_bytes"] = len(blob)
        sc = None
        if cpu:
            # the oracle's port of the reference's scalar traversal over the same BLAS / TLAS bytes
            from oracle import oracle as orc
            orc.build()
            bi = r.scene_instances()
            oi = np.zeros(1, dtype=orc.instance_dtype)
            oi["local_to_world"] = np.eye(4, dtype=np.float32).reshape(16)
            oi["world_to_local"] = bi[0]["world_to_local"]
            sc = orc.Scene([(tris, blob)], r.scene_tlas(), oi)
            if cpu_build:
                # the reference's single-threaded C++ BLAS build (the oracle's restatement) of the same soup
                t0 = time.perf_counter()
                ref_blob = orc.bvh_build(tris, 16, False, 4)
                info["cpu_bvh_build_s"] = round(time.perf_counter() - t0, 2)
                info["blas_equal_to_cpu_build"] = bool(np.array_equal(ref_blob, blob))
                del ref_blob
        del blob
        for kind in kinds:
            rays = scenes.soup_rays(side, seed=7, kind=kind)
            for any_hit in (False, True):
                if any_hit:
                    rays["tmax"] = np.random.default_rng(9).uniform(0, 1, len(rays)).astype(np.float32)
                d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
                d_hits = torch.zeros(len(rays) * 20, dtype=torch.uint8, device="cuda")
                l2 = torch.zeros(L2_BYTES // 4, dtype=torch.float32, device="cuda")
                r.trace_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), any_hit=any_hit, count_traffic=True)
                c = r.stats()
                alg = (len(rays) * (B_RAY + B_HIT) + c["tlas_node_loads"] * B_TNODE + c["instance_loads"] * B_INST
                       + c["blas_node_loads"] * B_BNODE + c["triangle_tests"] * B_TRI)
                cpu_res = None
                for reorder in orders:
                    torch.cuda.synchronize()
                    for _ in range(warmup):
                        r.trace_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), any_hit=any_hit,
                                       reorder=reorder)
                    r.synchronize()
                    ms = []
                    for _ in range(steps):
                        l2.add_(1)
                        torch.cuda.synchronize()
                        r.trace_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), any_hit=any_hit,
                                       reorder=reorder)
                        ms.append(r.stats()["ms_total"])
                    t = float(np.mean(ms))
                    hits = d_hits.cpu().numpy().view(wf.abi.hit_dtype)
                    # end to end through wf_trace (rays in and hits out in page-locked host
                    # memory, copied by the call): the mean of 3 calls
                    h_rays = torch.empty(len(rays) * 32, dtype=torch.uint8, pin_memory=True)
                    h_rays.numpy()[:] = np.frombuffer(rays.tobytes(), np.uint8)
                    h_hits = torch.empty(len(rays) * 20, dtype=torch.uint8, pin_memory=True)
                    flags = (wf.abi.TRACE_ANY_HIT if any_hit else 0) | (wf.abi.TRACE_REORDER if reorder else 0)

                    def call():
                        wf.check(r.L.wf_trace(r.h, ctypes.c_void_p(h_rays.data_ptr()), len(rays),
                                              ctypes.c_void_p(h_hits.data_ptr()), flags))
                    call()
                    t1 = time.perf_counter()
                    for _ in range(3):
                        call()
                    e2e_s = (time.perf_counter() - t1) / 3
                    assert np.array_equal(h_hits.numpy().view(wf.abi.hit_dtype), hits)
                    res = {"rays": kind, "query": "any" if any_hit else "closest",
                           "order": "morton" if reorder else "as given", "n": len(rays), "ms": round(t, 3),
                           "mrays_per_s": round(len(rays) / (t / 1e3) / 1e6, 2),
                           "e2e_mrays_per_s": round(len(rays) / e2e_s / 1e6, 2),
                           "alg_bytes": int(alg), "achieved_gbs": round(alg / (t / 1e3) / 1e9, 1),
                           "peak": peak, "peak_kind": peak_kind, "frac": round(alg / (t / 1e3) / 1e9 / peak, 4),
                           "fetches_per_ray": round((c["blas_node_loads"] + c["tlas_node_loads"]) / len(rays), 2),
                           "triangle_tests_per_ray": round(c["triangle_tests"] / len(rays), 2),
                           "hit_fraction": round(float((hits["instance"] != 0xFFFFFFFF).mean()), 4)}
                    if sc is not None and cpu_res is None:
                        # a random sample of the set, grown after a first pass to about cpu_seconds
                        threads = os.cpu_count() or 1
                        n_cpu = min(len(rays), CPU_TRACE_SAMPLE)
                        for _ in range(2):
                            pick = np.sort(np.random.default_rng(5).choice(len(rays), n_cpu, replace=False))
                            t1 = time.perf_counter()
                            want, _, _ = sc.trace(rays[pick], flags=1 if any_hit else 0, threads=threads)
                            cpu_s = time.perf_counter() - t1
                            n_next = min(len(rays), int(n_cpu * cpu_seconds / max(cpu_s, 1e-3)))
                            if n_next <= 2 * n_cpu:
                                break
                            n_cpu = n_next
                        cpu_res = {"value": round(len(pick) / cpu_s / 1e6, 3), "unit": "Mrays/s", "cores": threads,
                                   "kind": "port", "sample": f"{len(pick)} random rays of the set ({cpu_s:.2f} s)",
                                   "sample_hits_equal": bool(np.array_equal(hits[pick].view(np.uint32),
                                                                            want.view(np.uint32)))}
                    if cpu_res is not None:
                        res["cpu_baseline"] = cpu_res
                    results.append(res)
                del d_rays, d_hits, l2
    return info, results


def run_traversal(args, rank, world, local):
    """The traversal micro-benchmark on its own: one JSON line per ray set and
    query kind (8M soup triangles, 16.8M rays per set by default)."""
    if rank != 0:
        return
    info, results = traversal_runs(local, args.soup_triangles, args.soup_side, args.steps, args.warmup,
                                   kinds=args.ray_kinds.split(","), orders=(args.reorder == "on",),
                                   cpu=not args.no_cpu_baseline, cpu_build=not args.no_cpu_baseline,
                                   blas_layout=args.blas_layout)
    for res in results:
        line = {"metric": "traversal Mrays/s", "value": res["mrays_per_s"], "unit": "Mrays/s", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True,
                "dtype": "f32", "data": "synthetic (seeded triangle soup)",
                "config": {"workload": f"traversal micro-benchmark, {args.soup_triangles} soup triangles, {res['n']} "
                                       f"{res['rays']} rays, {res['query']} hit",
                           "ray_order": ("origins' Morton codes (stable radix sort inside the timed call)"
                                         if res["order"] == "morton" else "as given"),
                           "hit_fraction": res["hit_fraction"], **info},
                "e2e": {"value": res["e2e_mrays_per_s"], "unit": "Mrays/s", "h2d_bytes_per_step": res["n"] * 32,
                        "d2h_bytes_per_step": res["n"] * 20},
                "roofline": {"bound": "hbm", "kernel": "k_trace (AoS)", "achieved": res["achieved_gbs"],
                             "peak": res["peak"], "peak_kind": res["peak_kind"], "unit": "GB/s", "frac": res["frac"],
                             "alg_bytes_per_launch": res["alg_bytes"], "fetches_per_ray": res["fetches_per_ray"],
                             "triangle_tests_per_ray": res["triangle_tests_per_ray"]}}
        if "cpu_baseline" in res:
            line["cpu_baseline"] = res["cpu_baseline"]
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instance-bounds", type=int, default=DEFAULT_INSTANCE_BOUNDS, choices=[0, 1],
                    help="instance world boxes: 0 = the transformed BLAS root box (the reference's), "
                         "1 = from the BLAS frontier boxes (tight)")
    ap.add_argument("--tlas-metric", type=int, default=3,
                    help="TLAS build: 0 = reference walk and metric, 1 = merged-box walk, 2 = parallel clustering, "
                         "3 = top-down SAH sweep")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--blas-layout", type=int, default=0, choices=[0, 1, 2],
                    help="BLAS layout the traversal reads: 0 = the reference's binary child pairs, 1 = quantized "
                         "4-wide nodes, 2 = exact 4-wide nodes (both 4-wide: order-independent tie rule for "
                         "closest hits)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--frames-in-flight", type=int, default=2,
                    help="end-to-end leg: frames in flight, one context each (1 = one context, each frame "
                         "after the previous)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-rendering leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-scenes leg")
    ap.add_argument("--no-megakernel", action="store_true", help="skip the megakernel A/B leg")
    ap.add_argument("--no-traversal", action="store_true", help="skip the traversal micro-benchmark leg")
    ap.add_argument("--no-tlas-reference", action="store_true",
                    help="skip the frame rendered with the reference's TLAS (tlas_metric 0)")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-config", default=None,
                    help="batched workload: CAPACITY,THRESHOLD,BLOCK[,USE_GRAPH] instead of the autotuner "
                         "(profiling captures)")
    ap.add_argument("--tail-paths", type=int, default=0,
                    help="queue size below which a wave's remaining bounces run per path in one launch "
                         "(0 = never)")
    ap.add_argument("--fused-connect", action="store_true",
                    help="shadow rays of depth d in one launch with the extension rays of depth d + 1")
    ap.add_argument("--fused-from-depth", type=int, default=DEFAULT_FUSED_FROM_DEPTH,
                    help="separate schedule: from this depth on, each extension launch also traces the previous "
                         "depth's shadow rays (0 = never)")
    ap.add_argument("--workload", default="instanced", choices=["instanced", "traversal", "batched"])
    ap.add_argument("--soup-triangles", type=int, default=8_000_000)
    ap.add_argument("--soup-side", type=int, default=4096, help="rays per set = side^2")
    ap.add_argument("--ray-kinds", default="coherent,incoherent", help="traversal ray sets to run")
    ap.add_argument("--reorder", default="on", choices=["on", "off"],
                    help="traversal workload: trace rays in their origins' Morton order (WF_TRACE_REORDER)")
    ap.add_argument("--res", default="1920x1080", help="image size WxH (the workload is 1920x1080; smaller sizes "
                                                       "are for profiling captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global W, H
    W, H = (int(x) for x in args.res.lower().split("x"))
    rank, world, local = dist_env()
    if args.workload == "traversal":
        run_traversal(args, rank, world, local)
    elif args.workload == "batched":
        if rank == 0:
            cfg = args.batch_config.split(",") if args.batch_config else None
            res = batched_leg(local, args.tlas_metric, steps=args.steps, count=args.batch_scenes, config=cfg)
            print(json.dumps({"metric": "batched camera paths/s vs plain wavefront", "value": res["batched_spp_per_s"],
                              "unit": "paths/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": res["batched_ms"], "higher_is_better": True, "dtype": "f32",
                              "data": "synthetic (seeded procedural scenes)", "config": {"workload": res["config"]},
                              "batched": res}), flush=True)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
