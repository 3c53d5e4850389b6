"""FBX ingestion (the asset loader in front of wf_mesh_create /
wf_instance_submit; reference core/assets/asset_loader.cpp:613-920).

The files are written by the tests (tests/fbx_writer.py): quads and
triangles with per-corner, per-control-point and indexed layers, a mesh with
two materials split into two parts, a node hierarchy with every rotation
order, pre / post rotation and pivots, an invisible node, a mesh instanced
twice, phong and lambert materials with a PNG texture, Y-up centimetres and
Z-up metres, 32- and 64-bit records, raw and zlib arrays.  Where the
reference's own libraries are built (oracle/_ref/libref_assets.so: ufbx and
cgltf from the reference checkout behind oracle/ref_assets.c) every file is
also loaded through them and the two results are compared."""
import numpy as np
import pytest

from tests import fbx_writer as fw
from tests import ref_assets
from tests.test_gltf import encode_png
from wavefrontpathtracing_gb300 import fbx

needs_ref = pytest.mark.skipif(not ref_assets.available(), reason="reference loaders not built (oracle/_ref)")

CUBE_P = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
CUBE_F = [[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [2, 3, 7, 6], [1, 2, 6, 5], [0, 4, 7, 3]]


def cube_geometry(gid, compress=False, with_normals=True):
    normals, uvs, uv_index = [], [(0, 0), (1, 0), (1, 1), (0, 1), (0.5, 0.25)], []
    p = np.array(CUBE_P, float)
    for f in CUBE_F:
        n = np.cross(p[f[1]] - p[f[0]], p[f[2]] - p[f[0]])
        n = n / np.linalg.norm(n) * 2.0          # not unit length: the loader normalises
        normals += [n] * 4
        uv_index += [0, 1, 2, 4]
    return fw.geometry(gid, "cube", CUBE_P, CUBE_F, normals=normals if with_normals else None, uvs=uvs,
                       uv_index=uv_index, face_materials=[0, 1, 0, 1, 1, 0], compress=compress)


def strip_geometry(gid, compress=False):
    """Triangles and non-planar quads, normals and UVs by control point ("ByVertice" / "ByVertex")."""
    pts = [(0, 0, 0), (1, 0, 0.2), (2, 0, 0), (0, 1, 0), (1, 1, -0.3), (2, 1.2, 0), (0.9, 2, 0), (2.5, 2.5, 0.1)]
    polys = [[0, 1, 4, 3], [1, 2, 5], [1, 5, 4], [3, 4, 6], [4, 5, 7, 6]]
    rng = np.random.default_rng(3)
    normals = rng.normal(size=(len(pts), 3))
    uvs = rng.random((len(pts), 2))
    return fw.geometry(gid, "strip", pts, polys, normals=normals, normal_mapping="ByVertice", uvs=uvs,
                       uv_mapping="ByVertex", compress=compress)


def ngon_geometry(gid):
    pts = [(np.cos(a) * (1.0 + 0.3 * (k % 2)), np.sin(a) * (1.0 + 0.3 * (k % 2)), 0.0)
           for k, a in enumerate(np.linspace(0, 2 * np.pi, 9)[:-1])]
    return fw.geometry(gid, "ngon", pts, [list(range(8))], normals=[(0, 0, 1)] * 8, uvs=[(0, 0)] * 8)


def write_scene(path, settings=None, version=7400, compress=False, with_normals=True,
                textures=("tex.png", "spec.png")):
    objs = [cube_geometry(10, compress, with_normals), strip_geometry(11, compress), ngon_geometry(12),
            fw.model(20, "root", translation=(10, 20, 30), rotation=(10, 20, 30), scaling=(2, 2, 2)),
            fw.model(21, "child", translation=(5, 0, 0), rotation=(30, -45, 60), rotation_order=4,
                     pre_rotation=(0, 90, 0), post_rotation=(15, 0, 0), rotation_pivot=(1, 2, 3),
                     scaling_pivot=(0.5, 0, 0), scaling=(1, 2, 3)),
            fw.model(22, "strip_a", translation=(-50, 0, 0), rotation=(0, 0, 45), rotation_order=2),
            fw.model(23, "strip_b", translation=(0, -50, 0), rotation=(90, 0, 0), rotation_order=5),
            fw.model(24, "hidden", translation=(0, 0, 99), visible=False),
            fw.model(25, "ngon", rotation=(0, 0, 0), rotation_order=1, scaling=(3, 3, 3)),
            fw.material(30, "red", "phong", (1, 0, 0)), fw.material(31, "matte", "lambert", (0, 1, 0)),
            fw.material(32, "blue", "Phong", (0, 0, 1)),
            fw.texture(40, "tex", textures[0]), fw.texture(41, "spec", textures[1])]
    conns = [(20, 0), (21, 20), (22, 0), (23, 0), (24, 0), (25, 20),
             (10, 21), (30, 21), (31, 21),
             (11, 22), (11, 23), (11, 24), (32, 22), (32, 23),
             (12, 25), (31, 25),
             (40, 30, "DiffuseColor"), (41, 30, "SpecularColor"), (40, 31, "DiffuseColor")]
    fw.write(path, fw.scene(objs, conns, settings), version=version)


@pytest.fixture
def files(tmp_path):
    img = (np.arange(4 * 4 * 4).reshape(4, 4, 4) * 3 % 256).astype(np.uint8)
    (tmp_path / "tex.png").write_bytes(encode_png(img))
    (tmp_path / "spec.png").write_bytes(encode_png(img[::-1].copy()))
    out = {}
    out["yup_cm"] = tmp_path / "yup_cm.fbx"
    write_scene(out["yup_cm"])
    out["zup_m"] = tmp_path / "zup_m.fbx"
    write_scene(out["zup_m"], fw.global_settings(up=(2, 1), front=(1, -1), coord=(0, 1), unit=100.0))
    out["wide_zlib"] = tmp_path / "wide_zlib.fbx"
    write_scene(out["wide_zlib"], fw.global_settings(unit=2.54), version=7500, compress=True)
    return out, img


def test_records_and_scene(files):
    paths, img = files
    sc = fbx.load(paths["yup_cm"])
    # cube: two material parts (faces 0, 2, 5 / 1, 3, 4), strip: one part, ngon: one part
    assert len(sc.meshes) == 4
    sizes = [len(i) // 3 for _, i in sc.meshes]
    assert sizes == [6, 6, 7, 6]              # 3 quads per cube part; strip 2 quads + 3 triangles; ngon 6
    # instances: cube parts under "child", strip under strip_a and strip_b (hidden skipped), ngon
    assert [m for m, _, _ in sc.instances] == [0, 1, 2, 2, 3]
    assert [m for _, _, m in sc.instances] == [0, 1, 2, 2, 1]
    # unit scale (cm -> m) reaches positions and translations
    v, _ = sc.meshes[0]
    assert np.allclose(np.abs(v["position"]), 0.01)
    assert np.allclose(np.linalg.norm(v["normal"], axis=1), 1.0, atol=1e-6)
    # phong: white / metallic 1 / roughness 1 + its textures; lambert: the defaults, no textures
    red, matte, blue = sc.materials
    assert red["base_color_factor"] == [1.0, 1.0, 1.0, 1.0] and red["metallic_factor"] == 1.0
    assert red["base_color_image"] == 0 and red["metallic_roughness_image"] == 1
    assert np.array_equal(sc.images[0], img)
    assert matte["base_color_factor"] == [0.8, 0.8, 0.8, 1.0] and matte["roughness_factor"] == 0.5
    assert matte["base_color_image"] is None
    assert blue["base_color_image"] is None
    # n-gon: 8 corners -> 6 triangles covering the polygon's area
    v, idx = sc.meshes[3]
    p = v["position"][idx].reshape(-1, 3, 3).astype(np.float64)
    area = 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1).sum()
    ring = np.array([(np.cos(a) * (1.0 + 0.3 * (k % 2)), np.sin(a) * (1.0 + 0.3 * (k % 2)))
                     for k, a in enumerate(np.linspace(0, 2 * np.pi, 9)[:-1])]) * 0.01
    shoelace = 0.5 * abs(np.dot(ring[:, 0], np.roll(ring[:, 1], -1)) - np.dot(ring[:, 1], np.roll(ring[:, 0], -1)))
    assert area == pytest.approx(shoelace, rel=1e-5)


def test_dds_and_png_textures(tmp_path, files):
    """A phong material whose diffuse texture is a DDS of BC1 blocks (as the
    reference's Sun Temple materials are) and whose specular texture is a
    PNG: the DDS is kept as its blocks for wf_texture_create, the PNG
    decoded."""
    from tests.test_image_decode import dds_header
    from wavefrontpathtracing_gb300 import abi
    from wavefrontpathtracing_gb300.gltf import BlockImage
    _, img = files
    blocks = np.random.default_rng(3).integers(0, 256, 2 * 2 * 8, dtype=np.uint8)
    (tmp_path / "diffuse.dds").write_bytes(dds_header(8, 8, fourcc=b"DXT1") + blocks.tobytes())
    path = tmp_path / "dds.fbx"
    write_scene(path, textures=("diffuse.dds", "spec.png"))
    sc = fbx.load(path)
    red = sc.materials[0]
    im = sc.images[red["base_color_image"]]
    assert isinstance(im, BlockImage) and im.format == abi.TEXTURE_BC1 and (im.width, im.height) == (8, 8)
    assert np.array_equal(np.asarray(im.raw).reshape(-1), blocks)
    assert np.array_equal(sc.images[red["metallic_roughness_image"]], img[::-1])


def test_forms_agree(files):
    """32-bit records / raw arrays vs 64-bit records / zlib arrays: the same
    geometry apart from the unit scale."""
    paths, _ = files
    a = fbx.load(paths["yup_cm"])
    b = fbx.load(paths["wide_zlib"])
    assert len(a.meshes) == len(b.meshes)
    for (va, ia), (vb, ib) in zip(a.meshes, b.meshes):
        assert np.array_equal(ia, ib)
        assert np.allclose(va["position"] * 2.54, vb["position"], rtol=1e-6)
        assert np.array_equal(va["uv"], vb["uv"])


def test_not_fbx_and_ascii_are_rejected(tmp_path):
    p = tmp_path / "a.fbx"
    p.write_bytes(b"; FBX 7.4.0 project file\nFBXHeaderExtension:  {\n}\n")
    with pytest.raises(ValueError, match="ASCII"):
        fbx.load(p)
    p.write_bytes(b"garbage")
    with pytest.raises(ValueError, match="not an FBX"):
        fbx.load(p)


def _compare_with_reference(path, ngon_mesh=3):
    """Materials, every mesh's vertices (position, normal, uv) and index
    buffer bit for bit (the n-gon: the same corners and triangle count), every
    instance's mesh, material and world transform."""
    got = fbx.load(path)
    ref = ref_assets.load(path)
    assert len(got.materials) == len(ref.materials)
    for k, (m, r) in enumerate(zip(got.materials, ref.materials)):
        for key in ("base_color_factor", "emissive_factor"):
            assert np.allclose(m[key], r[key]), (k, key)
        for key in ("metallic_factor", "roughness_factor", "emissive_strength"):
            assert m[key] == pytest.approx(r[key]), (k, key)
        names = got.texture_names[k]
        for slot, rn in zip(("base_color_image", "normal_image", "metallic_roughness_image", "emissive_image"),
                            r["names"]):
            assert names.get(slot, "") == rn, (k, slot)
    assert len(got.meshes) == len(ref.meshes)
    for k, ((v, idx), (rv, ridx)) in enumerate(zip(got.meshes, ref.meshes)):
        if k == ngon_mesh:
            # own ear clipping: the same number of triangles over the same corners
            assert len(idx) == len(ridx)
            assert sorted(map(tuple, v["position"].tolist())) == sorted(map(tuple, rv[:, :3].tolist()))
            continue
        assert np.array_equal(idx, ridx), k
        assert np.array_equal(v["position"], rv[:, 0:3]), k
        assert np.array_equal(v["normal"], rv[:, 3:6]), k
        assert np.array_equal(v["uv"], rv[:, 6:8]), k
    assert len(got.instances) == len(ref.instances)
    for (m, w, mat), (rm, rmat, rw) in zip(got.instances, ref.instances):
        assert m == rm and mat == rmat
        # ufbx composes transforms in float (quaternions): 1e-6 of the matrix's largest entry
        assert np.allclose(np.asarray(w, np.float32), rw, rtol=1e-5, atol=1e-6 * max(1.0, np.abs(rw).max()))


@needs_ref
@pytest.mark.parametrize("form", ["yup_cm", "zup_m", "wide_zlib"])
def test_matches_the_reference_loader(files, form):
    paths, _ = files
    _compare_with_reference(paths[form])


@needs_ref
def test_generated_normals_match_the_reference_loader(tmp_path):
    p = tmp_path / "nonormals.fbx"
    write_scene(p, with_normals=False)
    _compare_with_reference(p)


def _linear_texels(rgba8):
    return (rgba8.astype(np.float32) / np.float32(255.0)).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("dds", [False, True])
def test_loaded_scene_renders_like_the_oracle(files, orc, tmp_path, dds):
    """The loaded FBX scene through wf_texture_create / wf_mesh_create /
    wf_instance_submit_many, rendered against the oracle given the same
    triangles, instances and texels, bit for bit; also with the diffuse
    texture a DDS of BC1 blocks, expanded on the GPU (the oracle takes the
    texels of its own block decoder)."""
    from wavefrontpathtracing_gb300 import Renderer, scenes
    from wavefrontpathtracing_gb300.abi import triangle_dtype
    from wavefrontpathtracing_gb300.gltf import BlockImage
    from tests.helpers import oracle_scene_from_renderer
    from tests.test_gltf import srgb_texels
    paths, _ = files
    path = paths["zup_m"]
    if dds:
        from tests.test_image_decode import dds_header
        blocks = np.random.default_rng(5).integers(0, 256, 2 * 2 * 8, dtype=np.uint8)
        (tmp_path / "diffuse.dds").write_bytes(dds_header(8, 8, fourcc=b"DXT1") + blocks.tobytes())
        path = tmp_path / "dds_scene.fbx"
        write_scene(path, fw.global_settings(up=(2, 1), front=(1, -1), coord=(0, 1), unit=100.0),
                    textures=("diffuse.dds", "spec.png"))
    sc = fbx.load(path)
    pts = np.concatenate([(np.c_[sc.meshes[g][0]["position"], np.ones(len(sc.meshes[g][0]))] @ np.asarray(w).T)[:, :3]
                          for g, w, _ in sc.instances])
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    c, ext = (lo + hi) / 2, float(np.max(hi - lo))
    view = scenes.make_view(tuple(c + np.array([0.3, 0.4, -1.6]) * ext), tuple(c), 50.0, 48, 40)
    with Renderer(48, 40) as r:
        r.begin_scene(view, (0.3, 0.3, 0.3))
        done = fbx.submit(r, sc, bvh=dict(interval_count=8))
        r.end_scene()
        tris = []
        for v, i in sc.meshes:
            t = np.zeros(len(i) // 3, dtype=triangle_dtype)
            t["v0"], t["v1"], t["v2"] = v[i[0::3]], v[i[1::3]], v[i[2::3]]
            tris.append(t)

        class Desc:
            meshes = tris
            instances = [(g, done.transforms[k], done.instance_materials[k]) for k, (g, _, _) in enumerate(sc.instances)]
        osc, _ = oracle_scene_from_renderer(orc, Desc, r, done.mesh_ids)
        r.render(max_bounces=3, spp=2, frame_seed=6, nee=1, rr_start_depth=2, accumulate=False)
        got = r.read_image()
    texels = [None] * len(done.texture_ids)
    for (image, srgb), tid in done.texture_ids.items():
        im = sc.images[image]
        if isinstance(im, BlockImage):
            im = orc.decode_bc(im.format, np.asarray(im.raw), im.width, im.height)
        texels[tid - 1] = srgb_texels(im) if srgb else _linear_texels(im)
    osc.set_textures(texels)
    acc, _ = osc.render(view, 48, 40, max_bounces=3, spp=2, frame_seed=6, nee=1, rr_start_depth=2,
                        env_color=(0.3, 0.3, 0.3), threads=4)
    want = np.zeros_like(acc)
    want[..., :3] = acc[..., :3] / acc[..., 3:]
    want[..., 3] = acc[..., 3]
    assert (got[..., :3] != np.float32(0.3)).any()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
