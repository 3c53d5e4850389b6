"""glTF 2.0 ingestion (the asset loader in front of wf_mesh_create /
wf_instance_submit; reference core/assets/asset_loader.cpp:367-611).

The files are written by the tests themselves: a .glb with two meshes (one
with two primitives, 16- and 32-bit indices, an interleaved vertex buffer), a
node hierarchy mixing a matrix and translation / rotation / scale, three
materials (with and without pbrMetallicRoughness, emissive strength) and a PNG
texture whose rows use all five PNG filters; and the same scene as .gltf with
an external .bin and data-URI image."""
import base64
import json
import struct
import zlib

import numpy as np
import pytest

from tests import ref_assets
from wavefrontpathtracing_gb300 import gltf


# --------------------------------------------------------------------------- writers (test side)

def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def encode_png(rgba):
    """RGBA8 PNG; row y uses filter y % 5."""
    h, w, _ = rgba.shape
    raw = bytearray()
    prev = np.zeros(w * 4, np.int32)
    for y in range(h):
        line = rgba[y].reshape(-1).astype(np.int32)
        f = y % 5
        out = np.zeros_like(line)
        for x in range(len(line)):
            a = line[x - 4] if x >= 4 else 0
            b = prev[x]
            c = prev[x - 4] if x >= 4 else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]
            out[x] = (line[x] - pred) & 255
        raw.append(f)
        raw += bytes(out.astype(np.uint8))
        prev = line

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b""))


def quad_vertices(z):
    pos = np.array([[0, 0, z], [1, 0, z], [1, 1, z], [0, 1, z]], np.float32)
    nrm = np.tile(np.array([[0, 0, -1]], np.float32), (4, 1))
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    return pos, nrm, uv


def build_scene_doc(image_png):
    """(document, binary buffer) of the test scene."""
    blob = bytearray()
    views, accessors = [], []

    def add_view(data, stride=None):
        while len(blob) % 4:
            blob.append(0)
        views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": len(data), **({"byteStride": stride} if stride else {})})
        blob.extend(data)
        return len(views) - 1

    def add_accessor(view, ctype, count, kind, offset=0, **kw):
        accessors.append({"bufferView": view, "componentType": ctype, "count": count, "type": kind,
                          "byteOffset": offset, **kw})
        return len(accessors) - 1

    # primitive A: separate arrays, 16-bit indices
    pos, nrm, uv = quad_vertices(0.0)
    a_pos = add_accessor(add_view(pos.tobytes()), 5126, 4, "VEC3", min=[0, 0, 0], max=[1, 1, 0])
    a_nrm = add_accessor(add_view(nrm.tobytes()), 5126, 4, "VEC3")
    a_uv = add_accessor(add_view(uv.tobytes()), 5126, 4, "VEC2")
    a_i16 = add_accessor(add_view(np.array([0, 1, 2, 0, 2, 3], np.uint16).tobytes()), 5123, 6, "SCALAR")
    # primitive B: interleaved position / normal / uv (stride 32), 32-bit indices
    pos2, nrm2, uv2 = quad_vertices(0.5)
    inter = np.zeros((4, 8), np.float32)
    inter[:, 0:3], inter[:, 3:6], inter[:, 6:8] = pos2, nrm2, uv2 * 2.0
    v_int = add_view(inter.tobytes(), stride=32)
    b_pos = add_accessor(v_int, 5126, 4, "VEC3", 0)
    b_nrm = add_accessor(v_int, 5126, 4, "VEC3", 12)
    b_uv = add_accessor(v_int, 5126, 4, "VEC2", 24)
    b_i32 = add_accessor(add_view(np.array([0, 2, 1, 0, 3, 2], np.uint32).tobytes()), 5125, 6, "SCALAR")
    img_view = add_view(image_png)
    doc = {
        "asset": {"version": "2.0"},
        "scene": 0,
        "scenes": [{"nodes": [0]}],
        "nodes": [
            {"children": [1, 2], "translation": [1.0, 2.0, 3.0], "rotation": [0.0, 0.38268343, 0.0, 0.92387953],
             "scale": [2.0, 2.0, 2.0]},
            {"mesh": 0},
            {"mesh": 1, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0.5, -1.0, 4.0, 1]},
        ],
        "meshes": [
            {"primitives": [{"attributes": {"POSITION": a_pos, "NORMAL": a_nrm, "TEXCOORD_0": a_uv},
                             "indices": a_i16, "material": 0},
                            {"attributes": {"POSITION": b_pos, "NORMAL": b_nrm, "TEXCOORD_0": b_uv},
                             "indices": b_i32, "material": 1}]},
            {"primitives": [{"attributes": {"POSITION": a_pos, "NORMAL": a_nrm, "TEXCOORD_0": a_uv},
                             "indices": a_i16, "material": 2}]},
        ],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.25, 1.0, 1.0], "metallicFactor": 0.0,
                                      "roughnessFactor": 0.75, "baseColorTexture": {"index": 0}},
             "emissiveFactor": [0.1, 0.2, 0.3]},
            {"emissiveFactor": [1.0, 1.0, 1.0]},   # no pbrMetallicRoughness: the reference keeps the defaults
            {"pbrMetallicRoughness": {}, "emissiveFactor": [1.0, 0.5, 0.25], "emissiveTexture": {"index": 0},
             "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 8.0}}},
        ],
        "textures": [{"source": 0}],
        "images": [{"bufferView": img_view, "mimeType": "image/png"}],
        "accessors": accessors,
        "bufferViews": views,
        "buffers": [{"byteLength": len(blob)}],
    }
    return doc, bytes(blob)


def write_glb(path, doc, blob):
    js = json.dumps(doc).encode()
    js += b" " * ((4 - len(js) % 4) % 4)
    bn = blob + b"\0" * ((4 - len(blob) % 4) % 4)
    total = 12 + 8 + len(js) + 8 + len(bn)
    with open(path, "wb") as f:
        f.write(struct.pack("<4sII", b"glTF", 2, total))
        f.write(struct.pack("<II", len(js), 0x4E4F534A) + js)
        f.write(struct.pack("<II", len(bn), 0x004E4942) + bn)


def image():
    rng = np.random.default_rng(2)
    return rng.integers(0, 256, (6, 5, 4), dtype=np.uint8)


def expected_worlds():
    c, s = np.cos(np.pi / 4), np.sin(np.pi / 4)   # rotation by 45 degrees about y
    r = np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]])
    t = np.eye(4)
    t[:3, 3] = [1, 2, 3]
    root = t @ r @ np.diag([2.0, 2.0, 2.0, 1.0])
    m = np.eye(4)
    m[:3, 3] = [0.5, -1.0, 4.0]
    return root, root @ m


# --------------------------------------------------------------------------- tests

def test_png_decoder_all_filters():
    img = image()
    assert np.array_equal(gltf.decode_png(encode_png(img)), img)


def write_form(tmp_path, form, img):
    doc, blob = build_scene_doc(encode_png(img))
    if form == "glb":
        path = tmp_path / "scene.glb"
        write_glb(path, doc, blob)
    else:
        (tmp_path / "scene.bin").write_bytes(blob)
        doc["buffers"] = [{"byteLength": len(blob), "uri": "scene.bin"}]
        view = doc["bufferViews"][doc["images"][0]["bufferView"]]
        png = blob[view["byteOffset"]:view["byteOffset"] + view["byteLength"]]
        doc["images"] = [{"uri": "data:image/png;base64," + base64.b64encode(png).decode()}]
        path = tmp_path / "scene.gltf"
        path.write_text(json.dumps(doc))
    return path


@pytest.mark.parametrize("form", ["glb", "gltf"])
def test_load_scene(tmp_path, form):
    img = image()
    path = write_form(tmp_path, form, img)
    sc = gltf.load(str(path))
    assert len(sc.meshes) == 3 and len(sc.images) == 1 and np.array_equal(sc.images[0], img)
    (v0, i0), (v1, i1), (v2, i2) = sc.meshes
    pos, nrm, uv = quad_vertices(0.0)
    assert np.array_equal(v0["position"], pos) and np.array_equal(v0["normal"], nrm) and np.array_equal(v0["uv"], uv)
    assert list(i0) == [0, 1, 2, 0, 2, 3] and list(i1) == [0, 2, 1, 0, 3, 2]
    pos2, _, uv2 = quad_vertices(0.5)
    assert np.array_equal(v1["position"], pos2) and np.array_equal(v1["uv"], uv2 * 2.0)
    root, child = expected_worlds()
    assert [(g, m) for g, _, m in sc.instances] == [(0, 0), (1, 1), (2, 2)]
    np.testing.assert_allclose(sc.instances[0][1], root, atol=1e-6)
    np.testing.assert_allclose(sc.instances[2][1], child, atol=1e-6)
    m0, m1, m2 = sc.materials
    assert m0["base_color_factor"][:3] == [0.5, 0.25, 1.0] and m0["roughness_factor"] == 0.75
    assert m0["metallic_factor"] == 0.0 and m0["base_color_image"] == 0 and m0["emissive_strength"] == 0.0
    assert m1["emissive_factor"] == [0.0, 0.0, 0.0] and m1["metallic_factor"] == 1.0   # defaults kept
    assert m2["emissive_strength"] == 8.0 and m2["emissive_image"] == 0 and m2["base_color_factor"] == [1, 1, 1, 1]


@pytest.mark.skipif(not ref_assets.available(), reason="reference loaders not built (oracle/_ref)")
@pytest.mark.parametrize("form", ["glb", "gltf"])
def test_matches_the_reference_loader(tmp_path, form):
    """The same file through cgltf as the reference reads it
    (oracle/ref_assets.c over the reference's vendored cgltf): materials,
    every primitive's vertices and indices bit for bit, every instance's
    mesh, material and world transform."""
    path = write_form(tmp_path, form, image())
    got = gltf.load(str(path))
    ref = ref_assets.load(str(path))
    assert len(got.materials) == len(ref.materials)
    for m, r in zip(got.materials, ref.materials):
        for key in ("base_color_factor", "emissive_factor"):
            assert np.allclose(m[key], r[key])
        for key in ("metallic_factor", "roughness_factor", "emissive_strength"):
            assert m[key] == pytest.approx(r[key])
        assert [m[k] for k in ("base_color_image", "normal_image", "metallic_roughness_image",
                               "emissive_image")] == r["images"]
    assert len(got.meshes) == len(ref.meshes)
    for (v, idx), (rv, ridx) in zip(got.meshes, ref.meshes):
        assert np.array_equal(idx, ridx)
        assert np.array_equal(v["position"], rv[:, 0:3]) and np.array_equal(v["normal"], rv[:, 3:6])
        assert np.array_equal(v["uv"], rv[:, 6:8])
    assert len(got.instances) == len(ref.instances)
    for (g, w, mat), (rg, rmat, rw) in zip(got.instances, ref.instances):
        assert g == rg and mat == rmat
        assert np.allclose(np.asarray(w, np.float32), rw, rtol=1e-6, atol=1e-6)


def test_missing_attributes_are_rejected(tmp_path):
    doc, blob = build_scene_doc(encode_png(image()))
    del doc["meshes"][0]["primitives"][0]["attributes"]["TEXCOORD_0"]
    path = tmp_path / "bad.glb"
    write_glb(path, doc, blob)
    with pytest.raises(ValueError, match="TEXCOORD_0"):
        gltf.load(str(path))


def srgb_texels(rgba8):
    """wf_texture_create's sRGB conversion: per byte, in double, rounded to float."""
    v = np.arange(256) / 255.0
    lut = np.where(v <= 0.04045, v / 12.92, ((v + 0.055) / 1.055) ** 2.4).astype(np.float32)
    out = lut[rgba8].astype(np.float32)
    out[..., 3] = rgba8[..., 3].astype(np.float32) / np.float32(255.0)
    return out


@pytest.mark.gpu
def test_loaded_scene_renders_like_the_oracle(tmp_path, orc):
    """The loaded scene through wf_texture_create / wf_mesh_create /
    wf_instance_submit_many, rendered against the oracle given the same
    triangles, instances and texels, bit for bit."""
    from wavefrontpathtracing_gb300 import Renderer, scenes
    from wavefrontpathtracing_gb300.abi import triangle_dtype
    from tests.helpers import oracle_scene_from_renderer
    doc, blob = build_scene_doc(encode_png(image()))
    path = tmp_path / "scene.glb"
    write_glb(path, doc, blob)
    sc = gltf.load(str(path))
    view = scenes.make_view((1.5, 3.0, -6.0), (1.5, 2.0, 4.0), 50.0, 40, 32)
    with Renderer(40, 32) as r:
        r.begin_scene(view, (0.2, 0.2, 0.2))
        done = gltf.submit(r, sc, bvh=dict(interval_count=8))
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
        r.render(max_bounces=3, spp=2, frame_seed=4, nee=1, rr_start_depth=2, accumulate=False)
        got = r.read_image()
    assert done.texture_ids == {(0, True): 1}
    osc.set_textures([srgb_texels(sc.images[0])])
    acc, _ = osc.render(view, 40, 32, max_bounces=3, spp=2, frame_seed=4, nee=1, rr_start_depth=2,
                        env_color=(0.2, 0.2, 0.2), threads=4)
    want = np.zeros_like(acc)
    want[..., :3] = acc[..., :3] / acc[..., 3:]
    want[..., 3] = acc[..., 3]
    assert got[..., :3].mean() > 0.0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def reference_helmet():
    import os as _os
    root = _os.environ.get("WF_REFERENCE_ROOT") or _os.path.join(
        _os.path.dirname(_os.path.dirname(_os.path.abspath(__file__))), "..", "reference")
    p = _os.path.join(root, "assets", "meshes", "damaged_helmet", "DamagedHelmet.gltf")
    return p if _os.path.exists(p) else None


@pytest.mark.skipif(not ref_assets.available() or reference_helmet() is None,
                    reason="the reference checkout's DamagedHelmet or the reference loaders are not present")
def test_reference_damaged_helmet_loads_like_the_reference():
    """The reference's own asset (assets/meshes/damaged_helmet: glTF + .bin +
    five JPEG textures) through gltf.load against cgltf as the reference reads
    it: materials with their texture slots, the mesh's vertices and indices
    bit for bit, the instance; its JPEG textures decode (wf_image_decode)
    within 3/255 of the reference's stb_image."""
    from tests.test_image_decode import stb_decode, STB
    import os as _os
    path = reference_helmet()
    got = gltf.load(path)
    ref = ref_assets.load(path)
    assert len(got.materials) == len(ref.materials) == 1 and len(got.meshes) == len(ref.meshes) == 1
    m, r = got.materials[0], ref.materials[0]
    for key in ("base_color_factor", "emissive_factor"):
        assert np.allclose(m[key], r[key])
    assert [m[k] for k in ("base_color_image", "normal_image", "metallic_roughness_image",
                           "emissive_image")] == r["images"]
    (v, idx), (rv, ridx) = got.meshes[0], ref.meshes[0]
    assert len(idx) > 10000 and np.array_equal(idx, ridx)
    assert np.array_equal(v["position"], rv[:, 0:3]) and np.array_equal(v["normal"], rv[:, 3:6])
    assert np.array_equal(v["uv"], rv[:, 6:8])
    assert [(g, mat) for g, _, mat in got.instances] == [(rg, rmat) for rg, rmat, _ in ref.instances]
    assert len(got.images) == 5
    if _os.path.exists(STB):
        import json
        doc = json.load(open(path))
        for k, im in enumerate(doc["images"]):
            data = open(_os.path.join(_os.path.dirname(path), im["uri"]), "rb").read()
            d = np.abs(got.images[k].astype(np.int16) - stb_decode(data, False).astype(np.int16))
            assert d.max() <= 3 and d.mean() < 0.1, (im["uri"], d.max(), d.mean())
