"""glTF 2.0 scene ingestion in front of the C ABI.

The reference loads glTF with cgltf (core/assets/asset_loader.cpp:367-611):
one render mesh per mesh primitive, one material per glTF material, and one
instance per (node with a mesh, primitive) at the node's world transform
(scene.cpp:34, 100).  This module reads .gltf (external .bin files or data
URIs) and .glb files, decodes PNG images, and hands the result to a Renderer:
wf_texture_create for the images (base colour and emission as sRGB, normal
and metallic-roughness maps as linear, as asset_loader.cpp:405-409 states
the glTF rules), wf_mesh_create for the primitives and
wf_instance_submit_many for the instances.

Same rules as the reference: POSITION, NORMAL and TEXCOORD_0 are required
(the reference asserts on them, asset_loader.cpp:529-533); a material without
pbrMetallicRoughness keeps the defaults (white, metallic 1, roughness 1, no
emission); with it, the factors, emissiveFactor and
KHR_materials_emissive_strength are taken, the strength being 0 when the
extension is absent (cgltf's value there, which the reference copies, so such
materials do not emit) and 1 when it is present without a value.  Where the reference
would read out of bounds or garbage, this loader is defined instead: 8-bit
indices and primitives without indices are accepted, and each node's
primitives map to the meshes of that node's own glTF mesh.  Only triangle
primitives and PNG images are supported.
"""
import base64
import json
import os
import struct
import zlib

import numpy as np

from .abi import TEXTURE_RGBA8, TEXTURE_RGBA8_SRGB, material_ext_dtype, vertex_dtype

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}


# --------------------------------------------------------------------------- PNG

def decode_png(data):
    """Non-interlaced 8-bit PNG (grey, grey+alpha, RGB, RGBA, palette) -> h x w x 4 uint8."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG image")
    pos, idat, palette, trns = 8, [], None, None
    w = h = depth = ctype = interlace = None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if depth != 8 or interlace != 0:
        raise ValueError("only 8-bit, non-interlaced PNG images are supported")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    stride = w * channels
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(h, stride + 1)
    out = np.zeros((h, w, channels), np.int32)
    prev = np.zeros((w, channels), np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32).reshape(w, channels)
        if f == 0:
            cur = line
        elif f == 1:                     # Sub: a running sum along the row
            cur = np.cumsum(line, axis=0) & 255
        elif f == 2:                     # Up
            cur = (line + prev) & 255
        elif f in (3, 4):                # Average, Paeth: left to right, one pixel at a time
            cur = np.zeros_like(line)
            left = np.zeros(channels, np.int32)
            upleft = np.zeros(channels, np.int32)
            for x in range(w):
                up = prev[x]
                if f == 3:
                    pred = (left + up) >> 1
                else:
                    e = left + up - upleft
                    pa, pb, pc = np.abs(e - left), np.abs(e - up), np.abs(e - upleft)
                    pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, up, upleft))
                cur[x] = (line[x] + pred) & 255
                left, upleft = cur[x], up
        else:
            raise ValueError(f"unknown PNG filter {f}")
        out[y] = cur
        prev = cur
    px = out.astype(np.uint8).reshape(h, w, channels)
    rgba = np.zeros((h, w, 4), np.uint8)
    rgba[..., 3] = 255
    if ctype == 0:
        rgba[..., :3] = px
    elif ctype == 4:
        rgba[..., :3] = px[..., :1]
        rgba[..., 3] = px[..., 1]
    elif ctype == 2:
        rgba[..., :3] = px
    elif ctype == 6:
        rgba[:] = px
    else:
        idx = px[..., 0]
        rgba[..., :3] = palette[idx]
        if trns is not None:
            alpha = np.full(256, 255, np.uint8)
            alpha[:len(trns)] = trns
            rgba[..., 3] = alpha[idx]
    return rgba


# --------------------------------------------------------------------------- file access

def _read(path):
    """Returns (document, buffers) of a .gltf or .glb file."""
    with open(path, "rb") as f:
        blob = f.read()
    base = os.path.dirname(os.path.abspath(path))
    glb_bin = None
    if blob[:4] == b"glTF":
        _, version, length = struct.unpack("<4sII", blob[:12])
        if version != 2:
            raise ValueError("only glTF 2.0 binary files are supported")
        pos, doc = 12, None
        while pos < length:
            n, kind = struct.unpack("<II", blob[pos:pos + 8])
            chunk = blob[pos + 8:pos + 8 + n]
            if kind == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif kind == 0x004E4942:
                glb_bin = chunk
            pos += 8 + n
    else:
        doc = json.loads(blob.decode("utf-8"))
    buffers = []
    for i, b in enumerate(doc.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            if glb_bin is None:
                raise ValueError(f"buffer {i} has no data")
            buffers.append(glb_bin)
        elif uri.startswith("data:"):
            buffers.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            with open(os.path.join(base, uri), "rb") as f:
                buffers.append(f.read())
    return doc, buffers, base


def _view_bytes(doc, buffers, view_index):
    v = doc["bufferViews"][view_index]
    data = buffers[v["buffer"]]
    off = v.get("byteOffset", 0)
    return data[off:off + v["byteLength"]], v.get("byteStride")


def _accessor(doc, buffers, index):
    a = doc["accessors"][index]
    if "sparse" in a:
        raise ValueError("sparse accessors are not supported")
    dt = np.dtype(_COMPONENT[a["componentType"]]).newbyteorder("<")
    nc = _NCOMP[a["type"]]
    count = a["count"]
    if "bufferView" not in a:
        return np.zeros((count, nc), dt)
    data, stride = _view_bytes(doc, buffers, a["bufferView"])
    off = a.get("byteOffset", 0)
    elem = dt.itemsize * nc
    stride = stride or elem
    if stride == elem:
        arr = np.frombuffer(data, dt, count * nc, off).reshape(count, nc)
    else:
        rows = np.frombuffer(data, np.uint8, stride * (count - 1) + elem, off)
        arr = np.lib.stride_tricks.as_strided(rows, (count, elem), (stride, 1)).copy().view(dt).reshape(count, nc)
    if a.get("normalized") and dt.kind in "ui":
        arr = arr.astype(np.float32) / np.float32(np.iinfo(dt).max)
    return arr


# --------------------------------------------------------------------------- scene graph

def _quat_matrix(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w), 0],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w), 0],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y), 0],
                     [0, 0, 0, 1]], dtype=np.float64)


def _local_matrix(node):
    if "matrix" in node:
        return np.array(node["matrix"], dtype=np.float64).reshape(4, 4).T   # glTF stores column-major
    t = np.eye(4)
    t[:3, 3] = node.get("translation", [0, 0, 0])
    r = _quat_matrix(node.get("rotation", [0, 0, 0, 1]))
    s = np.diag(list(node.get("scale", [1, 1, 1])) + [1.0])
    return t @ r @ s


def _world_matrices(doc):
    nodes = doc.get("nodes", [])
    parent = [-1] * len(nodes)
    for i, n in enumerate(nodes):
        for c in n.get("children", []):
            parent[c] = i
    world = [None] * len(nodes)

    def get(i):
        if world[i] is None:
            local = _local_matrix(nodes[i])
            world[i] = local if parent[i] < 0 else get(parent[i]) @ local
        return world[i]

    return [get(i) for i in range(len(nodes))]


# --------------------------------------------------------------------------- loading

class BlockImage:
    """An image kept as the file stores it for wf_texture_create (a DDS's BC
    blocks or float texels): raw bytes / floats, size and format."""

    def __init__(self, raw, width, height, fmt):
        self.raw, self.width, self.height, self.format = raw, width, height, fmt


def decode_image_file(data):
    """A texture file's image as the reference's asset loader takes it
    (asset_loader.cpp:56-206), decoded by the library (wf_image_decode): 8-bit
    RGBA (PNG, JPEG, an RGBA8 DDS) as an h x w x 4 uint8 array, anything else
    (BC blocks, float texels) as a BlockImage."""
    from . import decode_image
    raw, w, h, fmt = decode_image(bytes(data))
    if fmt == TEXTURE_RGBA8:
        return raw
    return BlockImage(raw, w, h, fmt)


class GltfScene:
    """meshes: one (vertices[vertex_dtype], uint32 indices) per primitive;
    images: h x w x 4 uint8 arrays; materials: dicts of factors and image
    indices per texture slot; instances: (mesh, node_to_world 4x4, material
    index or None)."""

    def __init__(self):
        self.meshes, self.images, self.materials, self.instances = [], [], [], []


def load(path):
    doc, buffers, base = _read(path)
    scene = GltfScene()
    # images
    for i, im in enumerate(doc.get("images", [])):
        if "bufferView" in im:
            data, _ = _view_bytes(doc, buffers, im["bufferView"])
        elif im.get("uri", "").startswith("data:"):
            data = base64.b64decode(im["uri"].split(",", 1)[1])
        else:
            with open(os.path.join(base, im["uri"]), "rb") as f:
                data = f.read()
        scene.images.append(decode_image_file(data))
    textures = doc.get("textures", [])

    def image_of(info):
        if not info or "index" not in info:
            return None
        return textures[info["index"]].get("source")

    # materials (asset_loader.cpp:411-471)
    for m in doc.get("materials", []):
        mat = {"base_color_factor": [1.0, 1.0, 1.0, 1.0], "metallic_factor": 1.0, "roughness_factor": 1.0,
               "emissive_factor": [0.0, 0.0, 0.0], "emissive_strength": 0.0,
               "base_color_image": None, "normal_image": None, "metallic_roughness_image": None,
               "emissive_image": None}
        pbr = m.get("pbrMetallicRoughness")
        if pbr is not None:
            mat["base_color_factor"] = list(pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0]))
            mat["metallic_factor"] = pbr.get("metallicFactor", 1.0)
            mat["roughness_factor"] = pbr.get("roughnessFactor", 1.0)
            mat["emissive_factor"] = list(m.get("emissiveFactor", [0.0, 0.0, 0.0]))
            # cgltf leaves the strength at 0 unless the extension is present
            # (1 when it is, without a value), and the reference copies it
            ext = m.get("extensions", {}).get("KHR_materials_emissive_strength")
            mat["emissive_strength"] = ext.get("emissiveStrength", 1.0) if ext is not None else 0.0
            mat["base_color_image"] = image_of(pbr.get("baseColorTexture"))
            mat["metallic_roughness_image"] = image_of(pbr.get("metallicRoughnessTexture"))
            mat["normal_image"] = image_of(m.get("normalTexture"))
            mat["emissive_image"] = image_of(m.get("emissiveTexture"))
        scene.materials.append(mat)
    # primitives -> meshes (asset_loader.cpp:476-565)
    first_prim = []
    prim_material = []
    for mi, mesh in enumerate(doc.get("meshes", [])):
        first_prim.append(len(scene.meshes))
        for pi, prim in enumerate(mesh["primitives"]):
            if prim.get("mode", 4) != 4:
                raise ValueError(f"mesh {mi} primitive {pi}: only triangle lists are supported")
            attr = prim["attributes"]
            for name in ("POSITION", "NORMAL", "TEXCOORD_0"):
                if name not in attr:
                    raise ValueError(f"mesh {mi} primitive {pi} is missing vertex attribute {name}")
            pos = _accessor(doc, buffers, attr["POSITION"]).astype(np.float32)
            nrm = _accessor(doc, buffers, attr["NORMAL"]).astype(np.float32)
            uv = _accessor(doc, buffers, attr["TEXCOORD_0"]).astype(np.float32)
            v = np.zeros(len(pos), dtype=vertex_dtype)
            v["position"], v["normal"], v["uv"] = pos, nrm, uv
            if "TANGENT" in attr:
                v["tangent"] = _accessor(doc, buffers, attr["TANGENT"]).astype(np.float32)
            if "indices" in prim:
                idx = _accessor(doc, buffers, prim["indices"]).reshape(-1).astype(np.uint32)
            else:
                idx = np.arange(len(pos), dtype=np.uint32)
            scene.meshes.append((v, idx))
            prim_material.append(prim.get("material"))
    # nodes with a mesh -> instances (asset_loader.cpp:569-608, scene.cpp:34, 100)
    worlds = _world_matrices(doc)
    for ni, node in enumerate(doc.get("nodes", [])):
        if "mesh" not in node:
            continue
        m = node["mesh"]
        for pi in range(len(doc["meshes"][m]["primitives"])):
            g = first_prim[m] + pi
            scene.instances.append((g, worlds[ni], prim_material[g]))
    return scene


class Submitted:
    """What submit() created: mesh ids (one per primitive), texture ids by
    (image, sRGB), and the material record of every submitted instance."""

    def __init__(self, mesh_ids, texture_ids, instance_materials, transforms):
        self.mesh_ids, self.texture_ids = mesh_ids, texture_ids
        self.instance_materials, self.transforms = instance_materials, transforms


# the sRGB variant of a file's format, as colour textures load (dds.h:125-147)
def _srgb_table():
    from . import abi
    return {abi.TEXTURE_RGBA8: abi.TEXTURE_RGBA8_SRGB, abi.TEXTURE_BC1: abi.TEXTURE_BC1_SRGB,
            abi.TEXTURE_BC2: abi.TEXTURE_BC2_SRGB, abi.TEXTURE_BC3: abi.TEXTURE_BC3_SRGB,
            abi.TEXTURE_BC7: abi.TEXTURE_BC7_SRGB}


_SRGB = _srgb_table()


def submit(renderer, scene, object_transform=None, bvh=None):
    """Creates the scene's textures and meshes in `renderer` and submits its
    instances (call between begin_scene and end_scene); returns a Submitted."""
    bvh = bvh or {}
    tex_ids = {}

    def texture(image, srgb):
        if image is None:
            return 0
        key = (image, srgb)
        if key not in tex_ids:
            im = scene.images[image]
            if isinstance(im, BlockImage):
                fmt = _SRGB.get(im.format, im.format) if srgb else im.format
                tex_ids[key] = renderer.create_texture_raw(im.raw, im.width, im.height, fmt)
            else:
                tex_ids[key] = renderer.create_texture(im, TEXTURE_RGBA8_SRGB if srgb else TEXTURE_RGBA8)
        return tex_ids[key]

    mats = np.zeros(len(scene.materials) + 1, dtype=material_ext_dtype)
    default = len(scene.materials)   # primitives without a material: the renderer's default (white Lambert)
    mats[default]["base"]["base_color_factor"] = (1.0, 1.0, 1.0)
    for k, m in enumerate(scene.materials):
        b = mats[k]["base"]
        b["base_color_factor"] = m["base_color_factor"][:3]
        b["metallic_factor"] = m["metallic_factor"]
        b["roughness_factor"] = m["roughness_factor"]
        b["emissive_factor"] = m["emissive_factor"]
        b["emissive_strength"] = m["emissive_strength"]
        b["base_color_index"] = texture(m["base_color_image"], True)
        b["normal_index"] = texture(m["normal_image"], False)
        b["metallic_roughness_index"] = texture(m["metallic_roughness_image"], False)
        b["emissive_index"] = texture(m["emissive_image"], True)
        mats[k]["ior"] = 1.5
    ids = [renderer.create_render_mesh(v, i, **bvh) for v, i in scene.meshes]
    obj = np.eye(4) if object_transform is None else np.asarray(object_transform, dtype=np.float64)
    xf = np.stack([(obj @ w).astype(np.float32) for _, w, _ in scene.instances]) if scene.instances else \
        np.zeros((0, 4, 4), np.float32)
    inst_mats = mats[[default if m is None else m for _, _, m in scene.instances]]
    if scene.instances:
        renderer.submit_render_meshes([ids[g] for g, _, _ in scene.instances], xf, inst_mats)
    return Submitted(ids, tex_ids, inst_mats, xf)
