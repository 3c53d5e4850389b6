"""FBX (binary) scene ingestion in front of the C ABI.

The reference loads FBX files with ufbx (core/assets/asset_loader.cpp:613-920):
load options at asset_loader.cpp:658-684 (metres, +X right / +Y up / +Z
front, the axis and unit conversion applied by modifying the geometry,
missing normals generated, normals normalised), one render mesh per material
part of every mesh that some node instances (its faces triangulated, the
corner stream de-duplicated into an index buffer), one material per FBX
material, and one instance per (visible node, part) at the node's world
transform (scene.cpp:34, 100).  This module reads binary FBX 7.x files itself
and produces the same data, then hands it to a Renderer through the glTF
module's submit() (wf_texture_create, wf_mesh_create,
wf_instance_submit_many).

What it follows, step for step:
  * node transforms: T * Roff * Rp * Rpre * R * Rpost^-1 * Rp^-1 * Soff * Sp
    * S * Sp^-1 from the Model's Properties70 (Lcl Translation / Rotation /
    Scaling, RotationOrder, Pre/PostRotation, pivots, offsets), parents
    first; the root conversion (axis matrix times the unit scale, metres)
    goes into the vertex positions and every node's translation (its scale
    factor) and into the top-level nodes' rotation, as ufbx's geometry
    modifying conversion does; geometric transforms are ignored, as the
    reference reads raw vertex positions with node_to_world;
  * polygons: PolygonVertexIndex with negative end markers; triangles as
    they are, quads split along the shorter diagonal unless the split folds
    (the rule of ufbx_triangulate_face), larger polygons by ear clipping on
    the polygon's best-fit plane (own method: same triangle count and area
    as ufbx, not necessarily the same diagonals);
  * per-corner attributes through the layer mapping (ByPolygonVertex,
    ByVertice / ByVertex, ByPolygon, AllSame; Direct or IndexToDirect),
    the first UV set with v flipped (1 - v), normals normalised, missing
    normals generated per face when the file has none (ufbx treats every
    edge as hard without smoothing data);
  * arithmetic: the reference builds ufbx with a float real type
    (UFBX_REAL_TYPE float in its ufbx.h), so positions, normals, UVs and the
    unit factor are rounded to float when read and scaled / normalised in
    float exactly as there; node transforms are composed in double (within
    1e-6 relative of ufbx's float quaternion arithmetic);
  * material parts: faces grouped by LayerElementMaterial index into
    max(materials, 1) parts (out-of-range indices go to part 0), the
    mesh's materials being those connected to its first instance node;
  * materials: "lambert" shading keeps the reference's defaults (grey 0.8,
    metallic 0, roughness 0.5); every other shading model takes its branch
    for specular materials (white, metallic 1, roughness 1) with the
    textures connected to DiffuseColor, NormalMap, SpecularColor (as the
    metallic-roughness map) and EmissiveColor.

Where the reference is undefined this loader is defined instead: a mesh
used by several nodes gives every node its own parts (the reference's
running part counter hands later nodes other meshes' parts), parts without
triangles are skipped consistently, and a mesh without materials renders
with the default material.  ASCII FBX is not read.  Texture files are
decoded when they are PNG files next to the FBX file (by relative name);
others are left out with the texture slot empty.
"""
import os
import struct
import zlib

import numpy as np

from .abi import vertex_dtype
from .gltf import GltfScene, decode_image_file, decode_png, submit  # noqa: F401  (submit is this module's too)

_MAGIC = b"Kaydara FBX Binary  \x00"
_ARRAY = {"f": np.float32, "d": np.float64, "l": np.int64, "i": np.int32, "b": np.uint8}
_SCALAR = {"Y": "<h", "C": "<?", "I": "<i", "F": "<f", "D": "<d", "L": "<q"}


# --------------------------------------------------------------------------- binary records

class Node:
    """One FBX record: name, property values, child records."""
    __slots__ = ("name", "props", "children")

    def __init__(self, name, props, children):
        self.name, self.props, self.children = name, props, children

    def child(self, name):
        for c in self.children:
            if c.name == name:
                return c
        return None

    def all(self, name):
        return [c for c in self.children if c.name == name]


def _parse_props(data, off, count):
    props = []
    for _ in range(count):
        t = chr(data[off])
        off += 1
        if t in _SCALAR:
            fmt = _SCALAR[t]
            props.append(struct.unpack_from(fmt, data, off)[0])
            off += struct.calcsize(fmt)
        elif t in _ARRAY:
            n, enc, clen = struct.unpack_from("<III", data, off)
            off += 12
            raw = data[off:off + clen]
            off += clen
            if enc == 1:
                raw = zlib.decompress(raw)
            elif enc != 0:
                raise ValueError(f"FBX: unknown array encoding {enc}")
            arr = np.frombuffer(raw, dtype=_ARRAY[t])
            if len(arr) < n:
                raise ValueError("FBX: truncated array property")
            props.append(arr[:n].copy())
        elif t in ("S", "R"):
            (n,) = struct.unpack_from("<I", data, off)
            off += 4
            props.append(bytes(data[off:off + n]))
            off += n
        else:
            raise ValueError(f"FBX: unknown property type {t!r}")
    return props, off


def _parse_node(data, off, wide):
    if wide:
        end, nprops, _plen = struct.unpack_from("<QQQ", data, off)
        off += 24
    else:
        end, nprops, _plen = struct.unpack_from("<III", data, off)
        off += 12
    nlen = data[off]
    off += 1
    if end == 0:
        return None, off + nlen
    name = bytes(data[off:off + nlen]).decode("ascii", "replace")
    off += nlen
    props, off = _parse_props(data, off, nprops)
    children = []
    while off < end:
        child, off = _parse_node(data, off, wide)
        if child is None:
            break
        children.append(child)
    return Node(name, props, children), end


def read_records(path):
    """The top-level records of a binary FBX file and its version."""
    with open(path, "rb") as f:
        data = f.read()
    if not data.startswith(_MAGIC):
        if data[:64].lstrip().startswith(b";") or b"FBXHeaderExtension:" in data[:4096]:
            raise ValueError(f"{path}: ASCII FBX is not supported (binary FBX 7.x only)")
        raise ValueError(f"{path}: not an FBX file")
    (version,) = struct.unpack_from("<I", data, 23)
    wide = version >= 7500
    off, top = 27, []
    while off < len(data):
        node, off = _parse_node(data, off, wide)
        if node is None:
            break
        top.append(node)
    return Node("", [], top), version


def _props70(node):
    """Properties70 of a record as {name: (type, values)}."""
    out = {}
    p70 = node.child("Properties70") if node is not None else None
    if p70 is not None:
        for p in p70.all("P"):
            name = p.props[0].decode("utf-8", "replace")
            out[name] = (p.props[1].decode("utf-8", "replace"), p.props[4:])
    return out


def _vec3(props, name, default):
    v = props.get(name)
    if v is None or len(v[1]) < 3:
        return np.array(default, dtype=np.float64)
    return np.array([float(x) for x in v[1][:3]], dtype=np.float64)


def _num(props, name, default):
    v = props.get(name)
    if v is None or not v[1]:
        return default
    return v[1][0]


# --------------------------------------------------------------------------- transforms

def _rot(axis, deg):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    m = np.eye(4)
    i, j = [(1, 2), (2, 0), (0, 1)][axis]
    m[i, i], m[i, j], m[j, i], m[j, j] = c, -s, s, c
    return m


# RotationOrder enum -> axes in the order they are applied to a point
_ORDERS = {0: (0, 1, 2), 1: (0, 2, 1), 2: (1, 2, 0), 3: (1, 0, 2), 4: (2, 0, 1), 5: (2, 1, 0)}


def _euler(deg, order=0):
    m = np.eye(4)
    for ax in _ORDERS.get(int(order), (0, 1, 2)):
        m = _rot(ax, deg[ax]) @ m
    return m


def _translate(v):
    m = np.eye(4)
    m[:3, 3] = v
    return m


def _scale(v):
    return np.diag([v[0], v[1], v[2], 1.0])


def _local_matrix(props):
    t = _vec3(props, "Lcl Translation", (0, 0, 0))
    r = _vec3(props, "Lcl Rotation", (0, 0, 0))
    s = _vec3(props, "Lcl Scaling", (1, 1, 1))
    pre = _vec3(props, "PreRotation", (0, 0, 0))
    post = _vec3(props, "PostRotation", (0, 0, 0))
    rp = _vec3(props, "RotationPivot", (0, 0, 0))
    ro = _vec3(props, "RotationOffset", (0, 0, 0))
    sp = _vec3(props, "ScalingPivot", (0, 0, 0))
    so = _vec3(props, "ScalingOffset", (0, 0, 0))
    order = _num(props, "RotationOrder", 0)
    return (_translate(t) @ _translate(ro) @ _translate(rp) @ _euler(pre) @ _euler(r, order)
            @ np.linalg.inv(_euler(post)) @ _translate(-rp) @ _translate(so) @ _translate(sp) @ _scale(s)
            @ _translate(-sp))


def _axis(settings, name, sign_name):
    axis = int(_num(settings, name, 3))
    sign = int(_num(settings, sign_name, 2))
    if axis not in (0, 1, 2):
        return None
    return axis, (1.0 if sign > 0 else -1.0)


_F = np.float32


def _snap_pow10(x):
    """A single-precision value within 2^-20 relative of a power of ten
    (1e-8 .. 1e9) becomes that power of ten (single precision), as ufbx's
    unit handling does."""
    for e in range(-8, 10):
        t = float(_F(10.0 ** e))
        err = max(abs(t * 9.5367431640625e-7), 7.52316384526264005e-37)
        if t - err <= float(x) <= t + err:
            return _F(t)
    return _F(x)


def _root_conversion(settings):
    """(3x3 rotation of the axis conversion, unit scale to metres as a
    single-precision factor: the reference builds ufbx with a float real
    type, so the factor is UnitScaleFactor (rounded to float) times 0.01f,
    snapped to a power of ten)."""
    unit = _snap_pow10(_F(_num(settings, "UnitScaleFactor", 1.0)) * _F(0.01))
    unit = _snap_pow10(unit / _F(1.0))
    src = (_axis(settings, "CoordAxis", "CoordAxisSign"), _axis(settings, "UpAxis", "UpAxisSign"),
           _axis(settings, "FrontAxis", "FrontAxisSign"))
    rot = np.eye(3)
    if all(a is not None for a in src):
        dst = ((0, 1.0), (1, 1.0), (2, 1.0))   # +X right, +Y up, +Z front
        if src != dst:
            rot = np.zeros((3, 3))
            for (sa, ss), (da, ds) in zip(src, dst):
                rot[da, sa] = ss * ds
            if np.linalg.det(rot) < 0:
                raise ValueError("FBX: the file's axes are left-handed; a mirroring conversion is not supported")
    return rot, unit


# --------------------------------------------------------------------------- geometry

def _polygons(pvi):
    """Corner ranges (begin, count) of each polygon and the control point of each corner."""
    pvi = np.asarray(pvi, dtype=np.int64)
    ends = np.nonzero(pvi < 0)[0]
    verts = np.where(pvi < 0, ~pvi, pvi)
    begins = np.concatenate([[0], ends[:-1] + 1]) if len(ends) else np.zeros(0, np.int64)
    return list(zip(begins.tolist(), (ends - begins + 1).tolist())), verts


def _layer(geom, name, values_name, index_name):
    """The layer element with index 0 of a kind: (mapping, values (n x k), index array or None)."""
    cands = [c for c in geom.all(name) if (c.props[0] if c.props else 0) == 0] or geom.all(name)
    if not cands:
        return None
    el = cands[0]
    mapping = el.child("MappingInformationType")
    ref = el.child("ReferenceInformationType")
    mapping = mapping.props[0].decode() if mapping is not None else "ByPolygonVertex"
    ref = ref.props[0].decode() if ref is not None else "Direct"
    vals = el.child(values_name)
    idx = el.child(index_name) if index_name else None
    values = np.asarray(vals.props[0]) if vals is not None else np.zeros(0)
    index = np.asarray(idx.props[0], dtype=np.int64) if (idx is not None and ref != "Direct") else None
    return mapping, values, index


def _corner_values(layer, width, corners, polys, verts):
    """Per-corner values of a layer element (len(corners) x width)."""
    mapping, values, index = layer
    vals = values.reshape(-1, width)
    n = len(verts)
    if mapping in ("ByPolygonVertex",):
        key = np.arange(n)
    elif mapping in ("ByVertice", "ByVertex"):
        key = verts
    elif mapping == "ByPolygon":
        key = np.zeros(n, np.int64)
        for f, (b, c) in enumerate(polys):
            key[b:b + c] = f
    elif mapping == "AllSame":
        key = np.zeros(n, np.int64)
    else:
        return None
    if index is not None:
        key = index[key]
    return vals[key[corners]]


def _quad_split(p):
    """ufbx_triangulate_face's quad rule: the shorter diagonal unless the split folds."""
    v0, v1, v2, v3 = p

    def nrm(x):
        ln = np.sqrt(np.dot(x, x))
        return x / ln if ln > 0.0 else x
    a, b = v2 - v0, v3 - v1
    na1 = nrm(np.cross(a, v1 - v0))
    na3 = nrm(np.cross(a, v0 - v3))
    nb0 = nrm(np.cross(b, v1 - v0))
    nb2 = nrm(np.cross(b, v2 - v1))
    dot_na, dot_nb = np.dot(na1, na3), np.dot(nb0, nb2)
    split_a = np.dot(a, a) <= np.dot(b, b)
    if dot_na < 0.0 or dot_nb < 0.0:
        split_a = dot_na >= dot_nb
    return [0, 1, 2, 2, 3, 0] if split_a else [1, 2, 3, 3, 0, 1]


def _ear_clip(p):
    """Triangles of a simple polygon (indices into p) by ear clipping on its best-fit plane."""
    n = len(p)
    normal = np.zeros(3)
    for i in range(n):   # Newell's method
        a, b = p[i], p[(i + 1) % n]
        normal += np.array([(a[1] - b[1]) * (a[2] + b[2]), (a[2] - b[2]) * (a[0] + b[0]),
                            (a[0] - b[0]) * (a[1] + b[1])])
    ln = np.linalg.norm(normal)
    normal = normal / ln if ln > 0 else np.array([1.0, 0.0, 0.0])
    u = np.cross([1.0, 0.0, 0.0] if normal[0] ** 2 < 0.5 else [0.0, 1.0, 0.0], normal)
    u /= np.linalg.norm(u)
    v = np.cross(normal, u)
    q = np.stack([p @ u, p @ v], axis=1)
    idx = list(range(n))
    out = []

    def cross2(o, a, b):
        return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])

    guard = 0
    while len(idx) > 3 and guard < 4 * n * n:
        guard += 1
        m = len(idx)
        clipped = False
        for k in range(m):
            i0, i1, i2 = idx[k - 1], idx[k], idx[(k + 1) % m]
            if cross2(q[i0], q[i1], q[i2]) <= 0.0:
                continue
            inside = False
            for j in idx:
                if j in (i0, i1, i2):
                    continue
                if (cross2(q[i0], q[i1], q[j]) >= 0 and cross2(q[i1], q[i2], q[j]) >= 0
                        and cross2(q[i2], q[i0], q[j]) >= 0):
                    inside = True
                    break
            if not inside:
                out += [i0, i1, i2]
                idx.pop(k)
                clipped = True
                break
        if not clipped:   # degenerate: fan the rest
            break
    for k in range(1, len(idx) - 1):
        out += [idx[0], idx[k], idx[k + 1]]
    return out


def _triangulate(begin, count, pos_of_corner):
    if count < 3:
        return []
    corners = list(range(begin, begin + count))
    if count == 3:
        return corners
    p = np.stack([pos_of_corner(c) for c in corners])
    local = _quad_split(p) if count == 4 else _ear_clip(p)
    return [corners[i] for i in local]


def _generated_normals(polys, verts, pos):
    """Per-corner normals of a mesh without a normal layer, as ufbx makes
    them when no smoothing information is present (every edge hard): each
    corner takes its face's weighted normal (triangle: (b - a) x (c - a);
    quad: (c - a) x (d - b); larger: Newell's sum), divided by its length,
    in single precision."""
    out = np.zeros((len(verts), 3), dtype=_F)
    for b, c in polys:
        if c < 3:
            continue
        ring = pos[verts[b:b + c]]
        if c == 3:
            n = np.cross(ring[1] - ring[0], ring[2] - ring[0])
        elif c == 4:
            n = np.cross(ring[2] - ring[0], ring[3] - ring[1])
        else:
            n = np.zeros(3, dtype=_F)
            for i in range(c):
                a, bb = ring[i], ring[(i + 1) % c]
                n = n + np.array([(a[1] - bb[1]) * (a[2] + bb[2]), (a[2] - bb[2]) * (a[0] + bb[0]),
                                  (a[0] - bb[0]) * (a[1] + bb[1])], dtype=_F)
        n = n.astype(_F)
        ln = np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
        if ln > _F(0.0):
            n = n / ln
        out[b:b + c] = n
    return out


def _normalize_f32(n):
    """Each row scaled by 1 / |row| in single precision (dot product summed
    x, y, z; zero rows stay zero), as ufbx normalises normals."""
    dot = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
    ln = np.sqrt(dot)
    ok = ln > _F(1.0842021795674597e-19)
    inv = np.where(ok, _F(1.0) / np.where(ok, ln, _F(1.0)), _F(0.0)).astype(_F)
    return (n * inv[:, None]).astype(_F)


def _dedup(v):
    """Identical vertices (byte for byte) merged, first occurrence first."""
    rows = np.ascontiguousarray(v).view(np.dtype((np.void, v.dtype.itemsize)))
    _, first, inverse = np.unique(rows, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    return v[first[order]], rank[inverse.reshape(-1)].astype(np.uint32)


# --------------------------------------------------------------------------- scene

def load(path):
    """Reads a binary FBX file into a GltfScene-shaped record (meshes,
    images, materials, instances) that submit() hands to a Renderer."""
    root, _version = read_records(path)
    base = os.path.dirname(os.path.abspath(path))
    settings = _props70(root.child("GlobalSettings"))
    rot, unit = _root_conversion(settings)
    objects = root.child("Objects")
    objs = {}
    order = []
    for o in (objects.children if objects is not None else []):
        if o.props:
            objs[o.props[0]] = o
            order.append(o.props[0])
    conns = root.child("Connections")
    links = []   # (kind, child, parent, property)
    for c in (conns.all("C") if conns is not None else []):
        kind = c.props[0].decode()
        prop = c.props[3].decode("utf-8", "replace") if len(c.props) > 3 else ""
        links.append((kind, c.props[1], c.props[2], prop))

    def kind_of(i):
        o = objs.get(i)
        return o.name if o is not None else None

    # node hierarchy and transforms
    parent = {}
    for k, ch, pa, _ in links:
        if k == "OO" and kind_of(ch) == "Model" and (pa == 0 or kind_of(pa) == "Model"):
            parent.setdefault(ch, pa)
    worlds = {}

    def world(mid):
        if mid not in worlds:
            props = _props70(objs[mid])
            local = _local_matrix(props)
            p = parent.get(mid, 0)
            local[:3, 3] *= float(unit)                # translations in metres
            if p == 0:
                conv = np.eye(4)
                conv[:3, :3] = rot
                local = conv @ local                   # top-level nodes take the axis rotation
                worlds[mid] = local
            else:
                worlds[mid] = world(p) @ local
        return worlds[mid]

    def visible(mid):
        return float(_num(_props70(objs[mid]), "Visibility", 1.0)) != 0.0

    # materials in file order; textures by connected property
    scene = GltfScene()
    mat_ids = [i for i in order if objs[i].name == "Material"]
    mat_index = {m: k for k, m in enumerate(mat_ids)}
    images = {}

    def image_of(tex_id):
        tex = objs[tex_id]
        rel = tex.child("RelativeFilename")
        name = rel.props[0].decode("utf-8", "replace") if rel is not None else ""
        if not name:
            fn = tex.child("FileName")
            name = os.path.basename(fn.props[0].decode("utf-8", "replace")) if fn is not None else ""
        if name not in images:
            images[name] = None
            full = os.path.join(base, name.replace("\\", os.sep))
            if name.lower().endswith((".png", ".jpg", ".jpeg", ".dds")) and os.path.exists(full):
                with open(full, "rb") as f:
                    scene.images.append(decode_image_file(f.read()))
                images[name] = len(scene.images) - 1
        return images[name]

    texture_names = []
    for m in mat_ids:
        node = objs[m]
        sm = node.child("ShadingModel")
        shading = sm.props[0].decode("utf-8", "replace") if sm is not None else ""
        tex = {}
        for k, ch, pa, prop in links:
            if k == "OP" and pa == m and kind_of(ch) == "Texture":
                tex.setdefault(prop, ch)
        names = {}
        mat = {"base_color_image": None, "normal_image": None, "metallic_roughness_image": None,
               "emissive_image": None}
        if shading in ("lambert", "Lambert"):
            mat.update(base_color_factor=[0.8, 0.8, 0.8, 1.0], metallic_factor=0.0, roughness_factor=0.5,
                       emissive_factor=[0.0, 0.0, 0.0], emissive_strength=0.0)
        else:
            mat.update(base_color_factor=[1.0, 1.0, 1.0, 1.0], metallic_factor=1.0, roughness_factor=1.0,
                       emissive_factor=[0.0, 0.0, 0.0], emissive_strength=0.0)
            for slot, props in (("base_color_image", ("DiffuseColor", "Diffuse")), ("normal_image", ("NormalMap",)),
                                ("metallic_roughness_image", ("SpecularColor", "Specular")),
                                ("emissive_image", ("EmissiveColor", "Emissive"))):
                for p in props:
                    if p in tex:
                        mat[slot] = image_of(tex[p])
                        rel = objs[tex[p]].child("RelativeFilename")
                        names[slot] = rel.props[0].decode("utf-8", "replace") if rel is not None else ""
                        break
        scene.materials.append(mat)
        texture_names.append(names)
    scene.texture_names = texture_names

    # meshes: per geometry (file order) that some model instances, one mesh per non-empty material part
    geo_ids = [i for i in order if objs[i].name == "Geometry" and (objs[i].props[2] if len(objs[i].props) > 2
                                                                      else b"Mesh") == b"Mesh"]
    for g in geo_ids:
        inst = [pa for k, ch, pa, _ in links if k == "OO" and ch == g and kind_of(pa) == "Model"]
        if not inst:
            continue
        geom = objs[g]
        vn = geom.child("Vertices")
        pn = geom.child("PolygonVertexIndex")
        if vn is None or pn is None:
            continue
        # single precision throughout, as the reference's ufbx build: values
        # rounded to float when read, then scaled in float
        raw = np.asarray(vn.props[0], dtype=np.float64).reshape(-1, 3).astype(_F)
        pos = raw * unit if unit != _F(1.0) else raw
        polys, verts = _polygons(pn.props[0])
        nl = _layer(geom, "LayerElementNormal", "Normals", "NormalsIndex")
        ul = _layer(geom, "LayerElementUV", "UV", "UVIndex")
        if ul is None:
            raise ValueError(f"{path}: geometry {g} is missing vertex attribute tex_coord")
        all_corners = np.arange(len(verts))
        # a layer with a mapping ufbx does not read counts as absent
        normals = _corner_values(nl, 3, all_corners, polys, verts) if nl is not None else None
        uvs = _corner_values(ul, 2, all_corners, polys, verts)
        if uvs is None:
            raise ValueError(f"{path}: geometry {g} is missing vertex attribute tex_coord")
        uvs = uvs.astype(_F)
        if normals is not None:
            normals = _normalize_f32(normals.astype(_F))
        else:
            normals = _normalize_f32(_generated_normals(polys, verts, raw))
        # the mesh's materials: those connected to its first instance node, in connection order
        mats = [ch for k, ch, pa, _ in links if k == "OO" and pa == inst[0] and kind_of(ch) == "Material"]
        ml = _layer(geom, "LayerElementMaterial", "Materials", None)
        face_mat = np.zeros(len(polys), np.int64)
        if ml is not None and len(mats) > 1:
            mapping, values, _ = ml
            values = np.asarray(values, dtype=np.int64)
            if mapping == "AllSame" and len(values):
                face_mat[:] = values[0]
            elif mapping == "ByPolygon":
                face_mat[:min(len(values), len(polys))] = values[:len(polys)]
            face_mat[(face_mat < 0) | (face_mat >= len(mats))] = 0
        parts = []
        for p in range(max(len(mats), 1)):
            tri = []
            for f in np.nonzero(face_mat == p)[0]:
                b, c = polys[f]
                tri += _triangulate(b, c, lambda corner: pos[verts[corner]])
            if not tri:
                continue
            tri = np.asarray(tri, dtype=np.int64)
            v = np.zeros(len(tri), dtype=vertex_dtype)
            v["position"] = pos[verts[tri]]
            v["normal"] = normals[tri]
            v["uv"][:, 0] = uvs[tri, 0]
            v["uv"][:, 1] = _F(1.0) - uvs[tri, 1]
            uniq, idx = _dedup(v)
            scene.meshes.append((uniq, idx))
            parts.append((len(scene.meshes) - 1, mat_index.get(mats[p]) if p < len(mats) else None))
        for mid in inst:
            if not visible(mid):
                continue
            for mesh, mat in parts:
                scene.instances.append((mesh, world(mid), mat))
    return scene
