"""Reads what oracle/ref_assets.c (the reference's scene loaders restated on
its vendored cgltf / ufbx, built into oracle/_ref/libref_assets.so) extracts
from a .gltf / .glb / .fbx file.  Test infrastructure only."""
import ctypes
import os
import struct
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_assets.so")


def available():
    return os.path.exists(LIB)


class RefScene:
    def __init__(self):
        self.materials, self.meshes, self.instances = [], [], []


def load(path):
    lib = ctypes.CDLL(LIB)
    lib.ref_asset_dump.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "dump.bin")
        rc = lib.ref_asset_dump(os.fsencode(path), os.fsencode(out))
        if rc != 0:
            raise RuntimeError(f"reference loader failed on {path}: {rc}")
        data = open(out, "rb").read()
    off = 0

    def take(fmt):
        nonlocal off
        v = struct.unpack_from(fmt, data, off)
        off += struct.calcsize(fmt)
        return v

    magic, version = take("<II")
    assert magic == 0x44414657 and version == 1
    sc = RefScene()
    (n,) = take("<I")
    for _ in range(n):
        f = take("<10f")
        m = {"base_color_factor": list(f[0:4]), "metallic_factor": f[4], "roughness_factor": f[5],
             "emissive_factor": list(f[6:9]), "emissive_strength": f[9], "images": [], "names": []}
        for _ in range(4):
            (img,) = take("<i")
            (ln,) = take("<I")
            m["images"].append(None if img < 0 else img)
            m["names"].append(data[off:off + ln].decode("utf-8", "replace"))
            off += ln
        sc.materials.append(m)
    (n,) = take("<I")
    for _ in range(n):
        (nv,) = take("<I")
        v = np.frombuffer(data, dtype=np.float32, count=8 * nv, offset=off).reshape(nv, 8).copy()
        off += 32 * nv
        (ni,) = take("<I")
        idx = np.frombuffer(data, dtype=np.uint32, count=ni, offset=off).copy()
        off += 4 * ni
        sc.meshes.append((v, idx))
    (n,) = take("<I")
    for _ in range(n):
        mesh, mat = take("<Ii")
        m = np.array(take("<16f"), dtype=np.float32).reshape(4, 4).T   # column-major -> rows
        sc.instances.append((mesh, None if mat < 0 else mat, m))
    return sc
