"""Binary FBX 7.x writer for the asset-ingestion tests (test side only).

Writes the record tree of a small scene: GlobalSettings (axes, unit scale),
Objects (Geometry with Vertices / PolygonVertexIndex and normal, UV and
material layers; Model with a Properties70 transform; Material with a
shading model and colours; Texture) and Connections, in either the 32-bit
(7400) or the 64-bit (7500) record layout, arrays raw or zlib-compressed.
"""
import struct
import zlib

import numpy as np

_MAGIC = b"Kaydara FBX Binary  \x00\x1a\x00"


class R:
    """A record: name, typed properties [(code, value)], children."""

    def __init__(self, name, props=(), children=()):
        self.name, self.props, self.children = name, list(props), list(children)


def S(s):
    return ("S", s.encode() if isinstance(s, str) else s)


def I(v):
    return ("I", int(v))


def L(v):
    return ("L", int(v))


def D(v):
    return ("D", float(v))


def arr(code, a, compress=False):
    return (code, (np.asarray(a), compress))


def _prop(code, value):
    out = code.encode()
    if code in ("S", "R"):
        return out + struct.pack("<I", len(value)) + value
    if code in "fdlib":
        a, compress = value
        dt = {"f": "<f4", "d": "<f8", "l": "<i8", "i": "<i4", "b": "u1"}[code]
        raw = np.ascontiguousarray(a, dtype=dt).tobytes()
        if compress:
            body = zlib.compress(raw)
            return out + struct.pack("<III", len(a), 1, len(body)) + body
        return out + struct.pack("<III", len(a), 0, len(raw)) + raw
    fmt = {"Y": "<h", "C": "<?", "I": "<i", "F": "<f", "D": "<d", "L": "<q"}[code]
    return out + struct.pack(fmt, value)


def _record(r, offset, wide):
    head = 25 if wide else 13
    props = b"".join(_prop(c, v) for c, v in r.props)
    name = r.name.encode()
    start = offset + head + len(name) + len(props)
    body = b""
    if r.children:
        pos = start
        for c in r.children:
            b = _record(c, pos, wide)
            body += b
            pos += len(b)
        body += b"\x00" * head
    end = start + len(body)
    fmt = "<QQQB" if wide else "<IIIB"
    return struct.pack(fmt, end, len(r.props), len(props), len(name)) + name + props + body


def write(path, records, version=7400):
    wide = version >= 7500
    data = _MAGIC + struct.pack("<I", version)
    for r in records:
        data += _record(r, len(data), wide)
    data += b"\x00" * (25 if wide else 13)
    data += b"\x00" * 160   # footer area (zeros)
    with open(path, "wb") as f:
        f.write(data)


def P(name, type_, label, flags, *values):
    return R("P", [S(name), S(type_), S(label), S(flags)] + list(values))


def props70(*ps):
    return R("Properties70", children=list(ps))


def global_settings(up=(1, 1), front=(2, 1), coord=(0, 1), unit=1.0):
    return R("GlobalSettings", children=[R("Version", [I(1000)]), props70(
        P("UpAxis", "int", "Integer", "", I(up[0])), P("UpAxisSign", "int", "Integer", "", I(up[1])),
        P("FrontAxis", "int", "Integer", "", I(front[0])), P("FrontAxisSign", "int", "Integer", "", I(front[1])),
        P("CoordAxis", "int", "Integer", "", I(coord[0])), P("CoordAxisSign", "int", "Integer", "", I(coord[1])),
        P("UnitScaleFactor", "double", "Number", "", D(unit)))])


def geometry(gid, name, positions, polygons, normals=None, normal_mapping="ByPolygonVertex", uvs=None,
             uv_index=None, uv_mapping="ByPolygonVertex", face_materials=None, compress=False):
    """polygons: list of control-point index lists; normals / uvs per the mapping."""
    pvi = []
    for poly in polygons:
        pvi += list(poly[:-1]) + [~poly[-1]]
    kids = [R("GeometryVersion", [I(124)]),
            R("Vertices", [arr("d", np.asarray(positions, np.float64).reshape(-1), compress)]),
            R("PolygonVertexIndex", [arr("i", pvi, compress)])]
    layer = []
    if normals is not None:
        kids.append(R("LayerElementNormal", [I(0)], [
            R("Version", [I(101)]), R("Name", [S("")]), R("MappingInformationType", [S(normal_mapping)]),
            R("ReferenceInformationType", [S("Direct")]),
            R("Normals", [arr("d", np.asarray(normals, np.float64).reshape(-1), compress)])]))
        layer.append(R("LayerElement", children=[R("Type", [S("LayerElementNormal")]), R("TypedIndex", [I(0)])]))
    if uvs is not None:
        ch = [R("Version", [I(101)]), R("Name", [S("UVMap")]), R("MappingInformationType", [S(uv_mapping)]),
              R("ReferenceInformationType", [S("IndexToDirect" if uv_index is not None else "Direct")]),
              R("UV", [arr("d", np.asarray(uvs, np.float64).reshape(-1), compress)])]
        if uv_index is not None:
            ch.append(R("UVIndex", [arr("i", uv_index, compress)]))
        kids.append(R("LayerElementUV", [I(0)], ch))
        layer.append(R("LayerElement", children=[R("Type", [S("LayerElementUV")]), R("TypedIndex", [I(0)])]))
    if face_materials is not None:
        kids.append(R("LayerElementMaterial", [I(0)], [
            R("Version", [I(101)]), R("Name", [S("")]), R("MappingInformationType", [S("ByPolygon")]),
            R("ReferenceInformationType", [S("IndexToDirect")]),
            R("Materials", [arr("i", face_materials, compress)])]))
        layer.append(R("LayerElement", children=[R("Type", [S("LayerElementMaterial")]), R("TypedIndex", [I(0)])]))
    kids.append(R("Layer", [I(0)], [R("Version", [I(100)])] + layer))
    return R("Geometry", [L(gid), S(name.encode() + b"\x00\x01Geometry"), S("Mesh")], kids)


def model(mid, name, translation=(0, 0, 0), rotation=(0, 0, 0), scaling=(1, 1, 1), rotation_order=0,
          pre_rotation=None, post_rotation=None, rotation_pivot=None, scaling_pivot=None, visible=True):
    ps = [P("Lcl Translation", "Lcl Translation", "", "A", *[D(x) for x in translation]),
          P("Lcl Rotation", "Lcl Rotation", "", "A", *[D(x) for x in rotation]),
          P("Lcl Scaling", "Lcl Scaling", "", "A", *[D(x) for x in scaling])]
    if rotation_order:
        ps.append(P("RotationOrder", "enum", "", "", I(rotation_order)))
    if pre_rotation is not None:
        ps.append(P("PreRotation", "Vector3D", "Vector", "", *[D(x) for x in pre_rotation]))
    if post_rotation is not None:
        ps.append(P("PostRotation", "Vector3D", "Vector", "", *[D(x) for x in post_rotation]))
    if rotation_pivot is not None:
        ps.append(P("RotationPivot", "Vector3D", "Vector", "", *[D(x) for x in rotation_pivot]))
    if scaling_pivot is not None:
        ps.append(P("ScalingPivot", "Vector3D", "Vector", "", *[D(x) for x in scaling_pivot]))
    if pre_rotation is not None or post_rotation is not None:
        ps.append(P("RotationActive", "bool", "", "", I(1)))
    if not visible:
        ps.append(P("Visibility", "Visibility", "", "A", D(0.0)))
    return R("Model", [L(mid), S(name.encode() + b"\x00\x01Model"), S("Mesh")],
             [R("Version", [I(232)]), props70(*ps), R("Shading", [("C", True)]), R("Culling", [S("CullingOff")])])


def material(mat_id, name, shading="phong", diffuse=(0.8, 0.8, 0.8)):
    return R("Material", [L(mat_id), S(name.encode() + b"\x00\x01Material"), S("")],
             [R("Version", [I(102)]), R("ShadingModel", [S(shading)]), R("MultiLayer", [I(0)]),
              props70(P("DiffuseColor", "Color", "", "A", *[D(x) for x in diffuse]))])


def texture(tid, name, relative):
    return R("Texture", [L(tid), S(name.encode() + b"\x00\x01Texture"), S("")],
             [R("Type", [S("TextureVideoClip")]), R("Version", [I(202)]),
              R("TextureName", [S(name.encode() + b"\x00\x01Texture")]),
              R("FileName", [S(relative)]), R("RelativeFilename", [S(relative)])])


def scene(objects, connections, settings=None):
    """Top-level records: header, settings, objects, connections (child, parent[, property])."""
    conns = []
    for c in connections:
        if len(c) == 2:
            conns.append(R("C", [S("OO"), L(c[0]), L(c[1])]))
        else:
            conns.append(R("C", [S("OP"), L(c[0]), L(c[1]), S(c[2])]))
    return [R("FBXHeaderExtension", children=[R("FBXHeaderVersion", [I(1003)]), R("FBXVersion", [I(7400)])]),
            settings or global_settings(),
            R("Documents", children=[R("Count", [I(1)])]),
            R("References"),
            R("Definitions", children=[R("Version", [I(100)]), R("Count", [I(len(objects))])]),
            R("Objects", children=list(objects)),
            R("Connections", children=conns)]
