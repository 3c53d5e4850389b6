"""GPU parity: the full wavefront loop (generate -> extend -> shade -> connect)
against the CPU oracle.

The kernels and the FP32 oracle draw the same random numbers and perform the
same float operations, and every pixel receives its contributions in the same
order, so the accumulated images are compared bit for bit, together with the
number of rays traced per call.  The FP64 oracle bounds the error of the FP32
arithmetic itself (image RMSE, tolerance written in the test)."""
import ctypes

import numpy as np
import pytest

import wavefrontpathtracing_gb300 as wf
from wavefrontpathtracing_gb300 import Renderer, scenes
from tests.helpers import load_scene_into, oracle_scene_from_renderer

pytestmark = pytest.mark.gpu


def render_both(orc, desc, spp, frame_seed=5, nee=None, rr=None, wave=0, prebuilt=True, threads=8, **renderer_kw):
    o = desc.bvh_options
    st = desc.settings
    nee = st["nee"] if nee is None else nee
    rr = st["rr_start_depth"] if rr is None else rr
    w, h = desc.width, desc.height
    blobs = [orc.bvh_build(t, o["interval_count"], False, o["max_leaf_prims"]) for t in desc.meshes] \
        if prebuilt else None
    with Renderer(w, h, wave_capacity=wave, **renderer_kw) as r:
        ids = load_scene_into(r, desc, prebuilt_blobs=blobs)
        sc, _ = oracle_scene_from_renderer(orc, desc, r, ids)
        r.render(max_bounces=st["max_bounces"], spp=spp, frame_seed=frame_seed, nee=nee, rr_start_depth=rr)
        img = r.read_image()
        stats = r.stats()
        ldr = r.read_image_ldr()
    acc, ost = sc.render(desc.view, w, h, max_bounces=st["max_bounces"], spp=spp, frame_seed=frame_seed, nee=nee,
                         rr_start_depth=rr, env_color=st["env"], threads=threads)
    want = np.zeros_like(acc)
    want[..., :3] = acc[..., :3] / acc[..., 3:]
    want[..., 3] = acc[..., 3]
    return img, want, stats, ost, ldr, sc


def assert_images_equal(got, want):
    bad = np.nonzero((got.view(np.uint32) != want.view(np.uint32)).any(axis=-1))
    assert bad[0].size == 0, f"{bad[0].size} pixels differ, first at {list(zip(bad[0][:5], bad[1][:5]))}"


def test_box_scene_reference_shading_bit_exact(orc):
    """Lambert only, no NEE, no RR: the reference's shade.hlsl semantics."""
    desc = scenes.box_scene(width=96, height=96, max_bounces=4)
    img, want, stats, ost, _, _ = render_both(orc, desc, spp=2)
    assert img[..., :3].mean() > 0.02
    assert_images_equal(img, want)
    assert stats["rays_extend"] == sum(ost["extend_rays"])
    assert stats["rays_connect"] == 0


def test_box_scene_waves_smaller_than_the_image(orc):
    desc = scenes.box_scene(width=64, height=48, max_bounces=3)
    img, want, stats, ost, _, _ = render_both(orc, desc, spp=3, wave=1000)
    assert_images_equal(img, want)
    assert stats["rays_extend"] == sum(ost["extend_rays"])


@pytest.mark.parametrize("renderer_kw", [{}, {"instance_bounds": 1, "tlas_metric": 2}])
def test_mixed_materials_nee_rr_bit_exact(orc, renderer_kw):
    """Lambert / GGX metal / dielectric, next-event estimation through the
    connect stage, Russian roulette from depth 3; also with the TLAS built
    over tight instance boxes (the oracle traverses the same TLAS)."""
    desc = scenes.instanced_scene(width=80, height=60, instances=60, freqs=(8, 12), spp=4, max_bounces=8)
    img, want, stats, ost, _, _ = render_both(orc, desc, spp=4, **renderer_kw)
    assert img[..., :3].max() > 0.0
    assert_images_equal(img, want)
    assert stats["rays_extend"] == sum(ost["extend_rays"])
    assert stats["rays_connect"] == sum(ost["shadow_rays"]) > 0


def test_box_scene_with_nee(orc):
    desc = scenes.box_scene(width=64, height=64, max_bounces=4)
    img, want, stats, ost, _, _ = render_both(orc, desc, spp=2, nee=1, rr=2)
    assert_images_equal(img, want)
    assert stats["rays_connect"] == sum(ost["shadow_rays"]) > 0


def srgb8(x):
    x = np.clip(x, 0, 1).astype(np.float32)
    y = np.where(x <= np.float32(0.0031308), x * np.float32(12.92),
                 np.float32(1.055) * np.power(x, np.float32(1 / 2.4)) - np.float32(0.055))
    return (np.clip(y, 0, 1) * 255 + 0.5).astype(np.uint8)


def test_post_process_ldr(orc):
    desc = scenes.box_scene(width=48, height=48, max_bounces=3)
    img, want, _, _, ldr, _ = render_both(orc, desc, spp=2)
    rgb = want[..., :3]
    rgb = rgb / (1 + rgb)                      # Reinhard (post_process.hlsl:58-60)
    ref = srgb8(rgb)
    assert np.abs(ldr[..., :3].astype(int) - ref.astype(int)).max() <= 1
    assert (ldr[..., 3] == 255).all()


def test_accumulation_across_calls_equals_one_call(orc):
    desc = scenes.box_scene(width=32, height=32, max_bounces=3)
    o = desc.bvh_options
    blobs = [orc.bvh_build(t, o["interval_count"], False, o["max_leaf_prims"]) for t in desc.meshes]
    with Renderer(32, 32) as r:
        load_scene_into(r, desc, prebuilt_blobs=blobs)
        r.render(max_bounces=3, spp=3, frame_seed=9)
        one = r.read_image()
        r.render(max_bounces=3, spp=1, frame_seed=9, accumulate=False)
        r.render(max_bounces=3, spp=2, frame_seed=9)
        two = r.read_image()
    assert np.array_equal(one[..., 3], two[..., 3])
    # same samples (0,1,2), same per-pixel addition order -> identical sums
    assert np.array_equal(one.view(np.uint32), two.view(np.uint32))


def test_fp64_oracle_rmse(orc):
    """Image error of the FP32 pipeline against the FP64 oracle driven by the
    same random numbers: RMSE <= 1e-3 on the tone-mapped box image at 16 spp."""
    desc = scenes.box_scene(width=64, height=64, max_bounces=4)
    img, want, _, _, _, sc = render_both(orc, desc, spp=16)
    a64, _ = sc.render(desc.view, 64, 64, max_bounces=4, spp=16, frame_seed=5, f64=True, threads=8)
    ref = a64[..., :3] / a64[..., 3:]
    tm = lambda x: x / (1.0 + x)
    rmse = float(np.sqrt(np.mean((tm(img[..., :3].astype(np.float64)) - tm(ref)) ** 2)))
    assert rmse <= 1e-3, rmse


@pytest.mark.parametrize("name", ["box", "instanced_small"])
def test_megakernel_equals_wavefront(orc, name):
    """use_wavefront_pathtracing = 0 (pathtracer.hlsl): whole paths per thread,
    the same traversal order and shading arithmetic, so the same image bit for
    bit and the same number of rays."""
    if name == "box":
        desc = scenes.box_scene(width=48, height=40, max_bounces=4)
        kw = dict(max_bounces=4, spp=3, nee=1, rr_start_depth=2)
    else:
        desc = scenes.instanced_scene(width=64, height=36, instances=48, freqs=(6, 9), spp=2, max_bounces=6)
        kw = dict(max_bounces=6, spp=2, nee=1, rr_start_depth=3)
    with Renderer(desc.width, desc.height) as r:
        load_scene_into(r, desc)
        r.render(frame_seed=21, accumulate=False, **kw)
        wave = r.read_image()
        sw = r.stats()
        r.render(frame_seed=21, accumulate=False, megakernel=True, **kw)
        mega = r.read_image()
        sm = r.stats()
    assert wave[..., :3].mean() > 0.0
    assert_images_equal(mega, wave)
    assert sm["rays_extend"] == sw["rays_extend"] and sm["rays_connect"] == sw["rays_connect"]
    assert sm["launches"] < sw["launches"]


@pytest.mark.parametrize("wave_paths", [0, 1000])
def test_fused_and_separate_connect_agree(orc, wave_paths):
    """The shadow rays of depth d traced in their own launches on a second
    stream (the default), in one launch with the extension rays of depth
    d + 1, in their own launches on the main stream, or fused from depth 2
    on: the same rays, the same image bit for bit, fewer launches when fused;
    an unknown schedule is refused."""
    desc = scenes.instanced_scene(width=64, height=36, instances=48, freqs=(6, 9), spp=2, max_bounces=6)
    kw = dict(max_bounces=6, spp=2, nee=1, rr_start_depth=3, wave_paths=wave_paths)
    with Renderer(desc.width, desc.height) as r:
        load_scene_into(r, desc)
        r.render(frame_seed=33, accumulate=False, fused_connect=True, **kw)
        fused = r.read_image()
        sf = r.stats()
        r.render(frame_seed=33, accumulate=False, **kw)
        sep = r.read_image()
        ss = r.stats()
        r.render(frame_seed=33, accumulate=False, serial_connect=True, **kw)
        ser = r.read_image()
        sr = r.stats()
        r.render(frame_seed=33, accumulate=False, fused_from_depth=2, **kw)
        hyb = r.read_image()
        sh = r.stats()
        with pytest.raises(wf.WFError):
            o = wf.abi.RenderOptions(1, 1, 0xFFFFFFFF, 0, 0, 0, 3)
            s = wf.abi.RenderSettings(1, 1, 0, 2, 1, 0, 1.0)
            wf.check(r.L.wf_render(r.h, ctypes.byref(s), ctypes.byref(o), 1))
    assert sf["rays_connect"] > 0
    assert_images_equal(fused, sep)
    assert_images_equal(ser, sep)
    assert_images_equal(hyb, sep)
    for k in ("rays_extend", "rays_connect", "extend_rays_depth", "shadow_rays_depth"):
        assert np.array_equal(np.asarray(sf[k]), np.asarray(ss[k])), k
        assert np.array_equal(np.asarray(sr[k]), np.asarray(ss[k])), k
        assert np.array_equal(np.asarray(sh[k]), np.asarray(ss[k])), k
    assert sf["launches"] < sh["launches"] < ss["launches"]
    assert sf["launches"] < ss["launches"]


def test_submit_many_equals_one_by_one(orc):
    desc = scenes.instanced_scene(width=48, height=32, instances=40, freqs=(5, 7), spp=1, max_bounces=4)
    imgs, insts = [], []
    for many in (False, True):
        with Renderer(desc.width, desc.height, tlas_metric=1) as r:
            ids = [r.create_mesh_from_triangles(t, interval_count=16, max_leaf_prims=4) for t in desc.meshes]
            r.begin_scene(desc.view, desc.settings["env"])
            if many:
                r.submit_render_meshes([ids[m] for m, _, _ in desc.instances],
                                       np.stack([np.asarray(t, np.float32) for _, t, _ in desc.instances]),
                                       np.array([m for _, _, m in desc.instances]))
            else:
                for m, t, mat in desc.instances:
                    r.submit_render_mesh(ids[m], t, mat)
            r.end_scene()
            insts.append(r.scene_instances())
            r.render(max_bounces=4, spp=2, frame_seed=3, nee=1, rr_start_depth=2, accumulate=False)
            imgs.append(r.read_image())
    assert insts[0].tobytes() == insts[1].tobytes()
    assert_images_equal(imgs[1], imgs[0])


def test_pipelined_frames_with_async_readback_equal_blocking_ones():
    """The e2e loop's pattern: frame i + 1's scene submitted (wf_scene_end
    returns before its TLAS is built) while frame i's image is still being
    copied by wf_read_image_async (page-locked and pageable buffers), a
    resize of nothing in between: every image equals the same frame rendered
    and read back blocking, and the instance records carry the tight boxes."""
    torch = pytest.importorskip("torch")
    desc = scenes.instanced_scene(width=64, height=40, instances=48, freqs=(5, 7), spp=2, max_bounces=5)
    mesh_ids = None

    def scene(r):
        r.begin_scene(desc.view, desc.settings["env"])
        r.submit_render_meshes([mesh_ids[m] for m, _, _ in desc.instances],
                               np.stack([np.asarray(t, np.float32) for _, t, _ in desc.instances]),
                               np.array([m for _, _, m in desc.instances]))
        r.end_scene()

    kw = dict(max_bounces=5, spp=2, nee=1, rr_start_depth=2, accumulate=False)
    with Renderer(desc.width, desc.height, tlas_metric=2, instance_bounds=1) as r:
        mesh_ids = [r.create_mesh_from_triangles(t, interval_count=16, max_leaf_prims=4) for t in desc.meshes]
        outs = [torch.empty((desc.height, desc.width, 4), dtype=torch.float32, pin_memory=True).numpy(),
                np.zeros((desc.height, desc.width, 4), np.float32),
                torch.empty((desc.height, desc.width, 4), dtype=torch.float32, pin_memory=True).numpy()]
        for i, out in enumerate(outs):
            scene(r)
            r.render(frame_seed=11 + i, **kw)
            r.read_image_async(out)
        r.synchronize()
        got = [o.copy() for o in outs]
        boxes = r.scene_instances()
        want = []
        for i in range(len(outs)):
            scene(r)
            r.render(frame_seed=11 + i, **kw)
            want.append(r.read_image())
    with Renderer(desc.width, desc.height, tlas_metric=2, instance_bounds=1) as r2:
        mesh_ids = [r2.create_mesh_from_triangles(t, interval_count=16, max_leaf_prims=4) for t in desc.meshes]
        scene(r2)
        r2.synchronize()
        assert boxes.tobytes() == r2.scene_instances().tobytes()
    for g, w in zip(got, want):
        assert_images_equal(g, w)
    assert not np.array_equal(got[0], got[1])


def test_frames_in_flight_on_two_contexts_equal_one_context():
    """The end-to-end bench's pattern: consecutive frames alternate between
    two contexts of the same scene (each its own streams and buffers, their
    launches overlapping on the GPU), scenes resubmitted and images read
    back asynchronously; every image equals the same frame rendered alone."""
    torch = pytest.importorskip("torch")
    desc = scenes.instanced_scene(width=56, height=40, instances=40, freqs=(5, 7), spp=2, max_bounces=6)
    kw = dict(max_bounces=6, spp=2, nee=1, rr_start_depth=2, accumulate=False, fused_from_depth=2)

    def make():
        r = Renderer(desc.width, desc.height, tlas_metric=2, instance_bounds=1)
        ids = [r.create_mesh_from_triangles(t, interval_count=16, max_leaf_prims=4) for t in desc.meshes]
        arrays = ([ids[m] for m, _, _ in desc.instances],
                  np.stack([np.asarray(t, np.float32) for _, t, _ in desc.instances]),
                  np.array([m for _, _, m in desc.instances]))
        return r, arrays

    ctxs = [make(), make()]
    try:
        outs = [torch.empty((desc.height, desc.width, 4), dtype=torch.float32, pin_memory=True).numpy()
                for _ in range(4)]
        for i in range(4):
            r, arrays = ctxs[i % 2]
            r.begin_scene(desc.view, desc.settings["env"])
            r.submit_render_meshes(*arrays)
            r.end_scene()
            r.render(frame_seed=40 + i, **kw)
            r.read_image_async(outs[i])
        for r, _ in ctxs:
            r.synchronize()
        got = [o.copy() for o in outs]
        r, arrays = ctxs[0]
        for i in range(4):
            r.begin_scene(desc.view, desc.settings["env"])
            r.submit_render_meshes(*arrays)
            r.end_scene()
            r.render(frame_seed=40 + i, **kw)
            assert_images_equal(got[i], r.read_image())
    finally:
        for r, _ in ctxs:
            r.close()


def test_per_depth_queue_sizes_match_the_oracle(orc):
    desc = scenes.instanced_scene(width=48, height=32, instances=60, freqs=(5, 8), spp=2, max_bounces=5)
    img, want, stats, ost, _, _ = render_both(orc, desc, spp=2, frame_seed=9, nee=1, rr=2)
    assert_images_equal(img, want)
    assert stats["extend_rays_depth"][:6] == ost["extend_rays"][:6]
    assert stats["shadow_rays_depth"][:6] == ost["shadow_rays"][:6]
    assert sum(stats["extend_rays_depth"]) == stats["rays_extend"]


def test_checkpoint_resume_equals_uninterrupted_render(tmp_path):
    """Accumulator checkpoint: 2 spp, save, a new context loads and adds 3
    more spp with the same frame seed == 5 spp in one context, bit for bit."""
    desc = scenes.box_scene(width=40, height=32, max_bounces=3)
    path = str(tmp_path / "accum.bin")
    with Renderer(40, 32) as r:
        load_scene_into(r, desc)
        r.render(max_bounces=3, spp=2, frame_seed=6, accumulate=True)
        r.save_accumulator(path)
    with Renderer(40, 32) as r:
        load_scene_into(r, desc)
        assert r.load_accumulator(path) == (2, 6)
        r.render(max_bounces=3, spp=3, frame_seed=6, accumulate=True)
        resumed = r.read_image()
    with Renderer(40, 32) as r:
        load_scene_into(r, desc)
        r.render(max_bounces=3, spp=5, frame_seed=6, accumulate=True)
        whole = r.read_image()
    assert (resumed[..., 3] == 5).all()
    assert_images_equal(resumed, whole)
    # another view or image size is refused
    other = scenes.box_scene(width=40, height=32, max_bounces=3)
    other.view = scenes.make_view((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), 40.0, 40, 32)
    import wavefrontpathtracing_gb300 as wf
    with Renderer(40, 32) as r:
        load_scene_into(r, other)
        with pytest.raises(wf.WFError):
            r.load_accumulator(path)
    with Renderer(20, 16) as r:
        small = scenes.box_scene(width=20, height=16, max_bounces=3)
        load_scene_into(r, small)
        with pytest.raises(wf.WFError):
            r.load_accumulator(path)


@pytest.mark.parametrize("where,wave_paths,fused", [("depth1", 0, False), ("middle", 0, False),
                                                   ("middle", 1500, False), ("depth1", 0, True),
                                                   ("middle", 0, True), ("middle", 1500, "from2")])
def test_tail_kernel_equals_wavefront(orc, where, wave_paths, fused):
    """The tail: once a wave's queue (projected from the previous wave's
    queue sizes) falls below tail_paths, its remaining bounces run one path per
    thread in one launch.  Same rays, same per-depth queue sizes, the same image
    bit for bit as the stage-per-depth loop, in fewer launches; also under the
    fused schedule, whose previous depth's shadow rays the tail would
    otherwise never see traced."""
    desc = scenes.instanced_scene(width=64, height=36, instances=48, freqs=(6, 9), spp=2, max_bounces=6)
    kw = dict(max_bounces=6, spp=2, nee=1, rr_start_depth=3, wave_paths=wave_paths, fused_connect=fused is True,
              fused_from_depth=2 if fused == "from2" else 0)
    with Renderer(desc.width, desc.height) as r:
        load_scene_into(r, desc)
        r.render(frame_seed=41, accumulate=False, **kw)
        want = r.read_image()
        sw = r.stats()
        q = [int(x) for x in sw["extend_rays_depth"][:7]]
        limit = (1 << 31) if where == "depth1" else (q[2] + q[3]) // 2 + 1
        assert where == "depth1" or q[3] < limit <= q[2]
        r.render(frame_seed=41, accumulate=False, tail_paths=limit, **kw)   # the queue sizes are known now
        got = r.read_image()
        st = r.stats()
    assert_images_equal(got, want)
    for k in ("rays_extend", "rays_connect", "extend_rays_depth", "shadow_rays_depth"):
        assert np.array_equal(np.asarray(st[k]), np.asarray(sw[k])), k
    assert st["launches"] < sw["launches"]
