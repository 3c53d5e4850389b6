"""GPU: textured materials, the equirect environment and the render view modes
against the CPU oracle.

The box scene gets random vertex uv (outside [0, 1], so wrap addressing is
exercised), an RGBA8 base-colour texture on the walls, an RG8
metallic-roughness texture on a metal sphere, an RGBA32F emission texture on
the light (sampled both on direct hits and by next-event estimation) and an
RGBA32F equirect environment.  Texel conversion is exact for these formats
(c / 255 in float), the bilinear weights, wrap and the environment's own
atan2 / asin are the same float operations on both sides, so images are
compared bit for bit, path traced and in every debug view."""
import numpy as np
import pytest

from wavefrontpathtracing_gb300 import Batch, Renderer, abi, scenes
from tests.helpers import load_scene_into, oracle_scene_from_renderer

pytestmark = pytest.mark.gpu

W, H = 64, 48


def textures(seed=4):
    rng = np.random.default_rng(seed)
    base8 = rng.integers(0, 256, (8, 8, 4), dtype=np.uint8)
    mr8 = rng.integers(0, 256, (4, 4, 2), dtype=np.uint8)
    emis = rng.uniform(0.5, 1.5, (4, 4, 4)).astype(np.float32)
    env = rng.uniform(0.0, 2.0, (8, 16, 4)).astype(np.float32)
    # the float texels both sides sample (wf_texture_create's conversion)
    base_f = base8.astype(np.float32) / np.float32(255.0)
    mr_f = np.zeros((4, 4, 4), np.float32)
    mr_f[..., :2] = mr8.astype(np.float32) / np.float32(255.0)
    mr_f[..., 3] = 1.0
    return [(base8, abi.TEXTURE_RGBA8, base_f), (mr8, abi.TEXTURE_RG8, mr_f), (emis, abi.TEXTURE_RGBA32F, emis),
            (env, abi.TEXTURE_RGBA32F, env)]


def textured_box(seed=4):
    desc = scenes.box_scene(width=W, height=H, subdivision=3, max_bounces=4)
    rng = np.random.default_rng(seed)
    for t in desc.meshes:
        for v in ("v0", "v1", "v2"):
            t[v]["uv"] = rng.uniform(-1.0, 2.0, (len(t), 2)).astype(np.float32)
    (_, _, m0), (_, _, m1), (_, _, m2) = desc.instances
    m0 = m0.copy()
    m0["base"]["base_color_index"] = 1
    m1 = scenes.material(base=(0.9, 0.7, 0.4), bsdf=scenes.BSDF_METAL, roughness=0.6, metallic=1.0)
    m1["base"]["metallic_roughness_index"] = 2
    m2 = m2.copy()
    m2["base"]["emissive_index"] = 3
    desc.instances = [(0, np.eye(4), m0), (1, np.eye(4), m1), (2, np.eye(4), m2)]
    desc.settings.update(nee=1, rr_start_depth=2, env=(1.0, 1.0, 1.0))
    return desc


def render_pair(orc, desc, view_mode=0, spp=2, seed=9, env_texture=4):
    tex = textures()
    st = desc.settings
    with Renderer(W, H) as r:
        ids = [r.create_texture(raw, fmt) for raw, fmt, _ in tex]
        assert ids == [1, 2, 3, 4]
        mesh_ids = load_scene_into(r, desc)
        r.begin_scene(desc.view, st["env"], env_texture=env_texture)   # again, with the environment texture
        for mesh, l2w, mat in desc.instances:
            r.submit_render_mesh(mesh_ids[mesh], l2w, mat)
        r.end_scene()
        sc, _ = oracle_scene_from_renderer(orc, desc, r, mesh_ids)
        r.render(max_bounces=st["max_bounces"], spp=spp, frame_seed=seed, nee=st["nee"],
                 rr_start_depth=st["rr_start_depth"], accumulate=False, view_mode=view_mode)
        got = r.read_image()
        ldr = r.read_image_ldr()
    sc.set_textures([f for _, _, f in tex], env_texture=env_texture)
    acc, _ = sc.render(desc.view, W, H, max_bounces=st["max_bounces"], spp=spp, frame_seed=seed, nee=st["nee"],
                       rr_start_depth=st["rr_start_depth"], env_color=st["env"], threads=4, view_mode=view_mode)
    want = np.zeros_like(acc)
    want[..., :3] = acc[..., :3] / acc[..., 3:]
    want[..., 3] = acc[..., 3]
    return got, want, ldr


def assert_same(got, want, what):
    bad = np.nonzero((got.view(np.uint32) != want.view(np.uint32)).any(axis=-1))
    assert bad[0].size == 0, f"{what}: {bad[0].size} pixels differ, first at {list(zip(bad[0][:4], bad[1][:4]))}"


def test_textured_materials_and_environment_bit_exact(orc):
    desc = textured_box()
    got, want, _ = render_pair(orc, desc)
    assert got[..., :3].mean() > 0.05
    assert_same(got, want, "path traced")


def test_constant_environment_and_textures_bit_exact(orc):
    got, want, _ = render_pair(orc, textured_box(), env_texture=0)
    assert_same(got, want, "constant env")


@pytest.mark.parametrize("mode", list(range(1, 12)))
def test_render_view_modes_bit_exact(orc, mode):
    got, want, ldr = render_pair(orc, textured_box(), view_mode=mode, spp=1)
    assert_same(got, want, f"view mode {mode}")
    # post_process.hlsl: no tonemap in a view mode, sRGB only for base colour / emission
    img = np.nan_to_num(got[..., :3], nan=0.0)
    bad = ~np.isfinite(got[..., :3]).all(axis=-1)
    x = np.clip(img, 0.0, 1.0)
    if mode in (6, 9):
        x = np.where(x <= 0.0031308, x * 12.92, 1.055 * np.power(x, 1.0 / 2.4) - 0.055)
    ref = np.floor(np.clip(x, 0, 1) * 255.0 + 0.5).astype(np.int32)
    ref[bad] = (255, 0, 255)
    assert np.abs(ldr[..., :3].astype(np.int32) - ref).max() <= 1


def test_view_modes_do_not_accumulate(orc):
    desc = textured_box()
    with Renderer(W, H) as r:
        for raw, fmt, _ in textures():
            r.create_texture(raw, fmt)
        load_scene_into(r, desc)
        r.render(max_bounces=2, spp=1, frame_seed=1, view_mode=abi.RENDER_VIEW_MODE_WORLD_NORMAL)
        a = r.read_image()
        r.render(max_bounces=2, spp=1, frame_seed=2, view_mode=abi.RENDER_VIEW_MODE_WORLD_NORMAL)
        b = r.read_image()
        assert np.array_equal(a, b) and (a[..., 3] == 1.0).all()


def test_texture_formats_convert_like_the_reference_defaults(orc):
    """A 1x1 texture of each format seen through the base-colour view."""
    quad = scenes.quad((-1.0, -1.0, 0.0), (0.0, 2.0, 0.0), (2.0, 0.0, 0.0))   # faces -z, towards the camera
    view = scenes.make_view((0.0, 0.0, -2.0), (0.0, 0.0, 0.0), 30.0, 8, 8)
    cases = [(np.array([[[10, 128, 255, 7]]], np.uint8), abi.TEXTURE_RGBA8),
             (np.array([[[10, 128, 255, 7]]], np.uint8), abi.TEXTURE_RGBA8_SRGB),
             (np.array([[[10, 200]]], np.uint8), abi.TEXTURE_RG8),
             (np.array([[[0.25, 2.5, -1.0, 1.0]]], np.float32), abi.TEXTURE_RGBA32F)]

    def srgb(c):
        c = c / 255.0
        return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)

    want = [np.array([10, 128, 255]) / 255.0, srgb(np.array([10, 128, 255])), np.array([10 / 255.0, 200 / 255.0, 0.0]),
            np.array([0.25, 2.5, -1.0])]
    with Renderer(8, 8) as r:
        mesh = r.create_mesh_from_triangles(quad, interval_count=8)
        for (raw, fmt), w in zip(cases, want):
            tid = r.create_texture(raw, fmt)
            m = scenes.material(base=(1.0, 1.0, 1.0))
            m["base"]["base_color_index"] = tid
            r.begin_scene(view)
            r.submit_render_mesh(mesh, np.eye(4), m)
            r.end_scene()
            r.render(max_bounces=1, spp=1, view_mode=abi.RENDER_VIEW_MODE_MATERIAL_BASE_COLOR)
            px = r.read_image()[4, 4, :3]
            np.testing.assert_allclose(px, w, rtol=1e-6, atol=1e-7)


def test_unknown_texture_ids_are_rejected():
    import wavefrontpathtracing_gb300 as wf
    with Renderer(8, 8) as r:
        mesh = r.create_mesh_from_triangles(scenes.quad((0, 0, 0), (1, 0, 0), (0, 1, 0)))
        r.begin_scene(scenes.make_view((0.5, 0.5, -1), (0.5, 0.5, 0), 45.0, 8, 8))
        m = scenes.material()
        m["base"]["emissive_index"] = 3
        with pytest.raises(wf.WFError) as e:
            r.submit_render_mesh(mesh, np.eye(4), m)
        assert e.value.status == -1
        with pytest.raises(wf.WFError):
            r.begin_scene(scenes.make_view((0.5, 0.5, -1), (0.5, 0.5, 0), 45.0, 8, 8), env_texture=1)
        with pytest.raises(wf.WFError):
            r.create_texture(np.zeros((0, 4, 4), np.uint8))


def test_batch_with_textures_equals_single_render(orc):
    desc = textured_box()
    tex = textures()
    st = desc.settings
    with Renderer(W, H) as r:
        [r.create_texture(raw, fmt) for raw, fmt, _ in tex]
        ids = load_scene_into(r, desc)
        r.begin_scene(desc.view, st["env"], env_texture=4)
        for mesh, l2w, mat in desc.instances:
            r.submit_render_mesh(ids[mesh], l2w, mat)
        r.end_scene()
        r.render(max_bounces=st["max_bounces"], spp=2, frame_seed=3, nee=1, rr_start_depth=2, accumulate=False)
        single = r.read_image()
        b = Batch(r)
        b.begin_scene(W, H, 2, desc.view, st["env"], env_texture=4)
        for mesh, l2w, mat in desc.instances:
            b.submit(ids[mesh], l2w, mat)
        b.end_scene()
        b.set_config(capacity=1024)
        b.render(max_bounces=st["max_bounces"], frame_seed=3, nee=1, rr_start_depth=2)
        assert_same(b.read_image(0), single, "batch")
        b.close()


# ------------------------------------------------- block-compressed textures

def srgb_lut():
    k = np.arange(256) / 255.0
    return np.where(k <= 0.04045, k / 12.92, ((k + 0.055) / 1.055) ** 2.4).astype(np.float32)


def to_float(rgba8, srgb):
    """wf_texture_create's 8-bit conversion: c / 255 (or the sRGB curve) for
    colour, c / 255 for alpha."""
    lin = np.arange(256, dtype=np.float32) / np.float32(255.0)
    col = (srgb_lut() if srgb else lin)[rgba8[..., :3]]
    return np.concatenate([col, lin[rgba8[..., 3:]]], axis=-1)


def random_blocks(fmt, n, seed):
    """n seeded blocks; BC7 blocks spread over its eight modes and the
    reserved one (random bytes would be half mode 0)."""
    rng = np.random.default_rng(seed)
    if fmt in (abi.TEXTURE_BC7, abi.TEXTURE_BC7_SRGB):
        from tests.golden.make_bc_hw import bc7_blocks
        b = bc7_blocks(rng)
        return b[rng.permutation(len(b))[:n]] if n <= len(b) else b
    small = fmt in (abi.TEXTURE_BC1, abi.TEXTURE_BC1_SRGB, abi.TEXTURE_BC4)
    return rng.integers(0, 256, (n, 8 if small else 16), dtype=np.uint8)


SRGB_BC = (abi.TEXTURE_BC1_SRGB, abi.TEXTURE_BC2_SRGB, abi.TEXTURE_BC3_SRGB, abi.TEXTURE_BC7_SRGB)


@pytest.mark.parametrize("fmt", [abi.TEXTURE_BC1, abi.TEXTURE_BC1_SRGB, abi.TEXTURE_BC2, abi.TEXTURE_BC2_SRGB,
                                 abi.TEXTURE_BC3, abi.TEXTURE_BC3_SRGB, abi.TEXTURE_BC4, abi.TEXTURE_BC5,
                                 abi.TEXTURE_BC7, abi.TEXTURE_BC7_SRGB])
def test_block_compressed_textures_decode_like_the_oracle(orc, fmt):
    """Random BC blocks of a ragged image (partial edge blocks: 13 x 9, or
    63 x 514 for BC7's 2,064 blocks of every mode), expanded on the GPU by
    wf_texture_create, read back: the oracle's decode, converted to float as
    the library converts 8-bit texels, bit for bit."""
    w, h = (63, 514) if fmt in (abi.TEXTURE_BC7, abi.TEXTURE_BC7_SRGB) else (13, 9)
    blocks = random_blocks(fmt, ((w + 3) // 4) * ((h + 3) // 4), fmt).reshape(-1)
    with Renderer(8, 8) as r:
        tid = r.create_texture_raw(blocks, w, h, fmt)
        got = r.read_texture(tid)
    want = to_float(orc.decode_bc(fmt, blocks, w, h), fmt in SRGB_BC)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


from tests.test_image_decode import BC_SAMPLER_TOLERANCE  # noqa: E402


@pytest.mark.parametrize("fmt", [abi.TEXTURE_BC1, abi.TEXTURE_BC2, abi.TEXTURE_BC3, abi.TEXTURE_BC4,
                                 abi.TEXTURE_BC5, abi.TEXTURE_BC7])
def test_block_decoder_equals_the_texture_sampler(fmt):
    """wf_texture_create's decode against this GPU's texture sampler reading
    the same blocks through a block-compressed CUDA texture (tests/
    hw_sampler.cu; the reference's D3D12 path decodes them in the sampler
    too): BC7 bit for bit (its texels are exact 8-bit values by definition),
    BC1-BC5 within the interpolation the formats leave open (per channel,
    BC_SAMPLER_TOLERANCE).  BC4 / BC5 compare their one / two channels."""
    from tests import hw_sampler
    bw, bh = 16, 129 if fmt == abi.TEXTURE_BC7 else 8
    blocks = random_blocks(fmt, bw * bh, 100 + fmt).reshape(-1)
    hw = hw_sampler.decode(fmt, blocks, bw, bh)
    with Renderer(8, 8) as r:
        got = r.read_texture(r.create_texture_raw(blocks, 4 * bw, 4 * bh, fmt))
    ch = {abi.TEXTURE_BC4: 1, abi.TEXTURE_BC5: 2}.get(fmt, 4)
    if fmt == abi.TEXTURE_BC7:
        assert np.abs(hw * 255.0 - np.rint(hw * 255.0)).max() < 1e-3
        assert np.array_equal(np.rint(got * 255.0), np.rint(hw * 255.0))
    else:
        diff = np.abs(got[..., :ch].astype(np.float64) - hw[..., :ch]) * 255.0
        tol = np.asarray(BC_SAMPLER_TOLERANCE[fmt])
        assert np.all(diff.reshape(-1, ch).max(0) <= tol), (diff.reshape(-1, ch).max(0), tol)


def test_texture_files_load_as_the_reference_loads_them(orc, tmp_path):
    """load_texture_file: a DDS of BC1 blocks (sRGB, as base colours load), a
    Radiance HDR file (float texels as stored) and a PNG written here."""
    from tests.test_image_decode import dds_header, random_rgbe, write_hdr, write_png
    w, h = 10, 6
    blocks = np.random.default_rng(8).integers(0, 256, 3 * 2 * 8, dtype=np.uint8)
    (tmp_path / "t.dds").write_bytes(dds_header(w, h, fourcc=b"DXT1") + blocks.tobytes())
    px = random_rgbe(5, 12, 9)
    (tmp_path / "t.hdr").write_bytes(write_hdr(px))
    rgba = np.random.default_rng(4).integers(0, 256, (7, 9, 4))
    (tmp_path / "t.png").write_bytes(write_png(rgba, 6, 8))
    with Renderer(8, 8) as r:
        a = r.read_texture(r.load_texture_file(str(tmp_path / "t.dds"), srgb=True))
        b = r.read_texture(r.load_texture_file(str(tmp_path / "t.hdr")))
        c = r.read_texture(r.load_texture_file(str(tmp_path / "t.png")))
    assert np.array_equal(c.reshape(7, 9, 4), to_float(rgba.astype(np.uint8), False))
    assert np.array_equal(a.view(np.uint32), to_float(orc.decode_bc(abi.TEXTURE_BC1, blocks, w, h), True).view(np.uint32))
    import wavefrontpathtracing_gb300 as wf
    want, _, _, _ = wf.decode_image(write_hdr(px))
    assert np.array_equal(b.view(np.uint32), want.view(np.uint32))


def test_bc7_dds_loads_as_the_sampler_decodes_it(orc, tmp_path):
    """A DX10 DDS of BC7 blocks (DXGI_FORMAT_BC7_UNORM, every mode), loaded
    as a base colour (sRGB) and as linear data: the oracle's decode, which
    equals the GPU texture sampler's for BC7, converted as 8-bit texels."""
    from tests.test_image_decode import dds_header
    w, h = 30, 21
    blocks = random_blocks(abi.TEXTURE_BC7, ((w + 3) // 4) * ((h + 3) // 4), 77).reshape(-1)
    (tmp_path / "t.dds").write_bytes(dds_header(w, h, dxgi=98) + blocks.tobytes())
    want8 = orc.decode_bc(abi.TEXTURE_BC7, blocks, w, h)
    with Renderer(8, 8) as r:
        srgb = r.read_texture(r.load_texture_file(str(tmp_path / "t.dds"), srgb=True))
        lin = r.read_texture(r.load_texture_file(str(tmp_path / "t.dds"), srgb=False))
    assert np.array_equal(srgb.view(np.uint32), to_float(want8, True).view(np.uint32))
    assert np.array_equal(lin.view(np.uint32), to_float(want8, False).view(np.uint32))
