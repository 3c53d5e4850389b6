"""Generates tests/golden/builders.npz from the reference's own builders.

Run in a checkout where the reference sources exist (they are compiled by
oracle/build_ref.sh into oracle/_ref/libref_bvh.so):

    oracle/build_ref.sh && python tests/golden/make_golden.py

For each case the fixture stores the input (triangle positions or instance
boxes) and the reference's output blob ([header | extract()], as the renderer
uploads it).  Blobs larger than 256 KiB are stored as SHA-256 digests.
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from wavefrontpathtracing_gb300 import scenes  # noqa: E402
from wavefrontpathtracing_gb300.abi import bvh_instance_dtype, triangle_dtype  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "builders.npz")
MAX_INLINE = 256 * 1024


def tris_from_positions(pos):
    pos = np.asarray(pos, dtype=np.float32).reshape(-1, 3, 3)
    t = np.zeros(len(pos), dtype=triangle_dtype)
    t["v0"]["position"], t["v1"]["position"], t["v2"]["position"] = pos[:, 0], pos[:, 1], pos[:, 2]
    return t


def positions(tris):
    return np.stack([tris["v0"]["position"], tris["v1"]["position"], tris["v2"]["position"]], axis=1).astype(
        np.float32)


def mesh_cases():
    rng = np.random.default_rng(1234)
    cases = {}
    cases["one"] = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], dtype=np.float32)
    cases["two"] = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[2, 0, 0], [3, 0, 0], [2, 1, 0]]], np.float32)
    cases["three"] = rng.random((3, 3, 3), dtype=np.float32)
    cases["four"] = rng.random((4, 3, 3), dtype=np.float32)
    same = rng.random((1, 3, 3), dtype=np.float32)
    cases["same_centroid"] = np.repeat(same, 9, axis=0)
    g = np.stack(np.meshgrid(np.arange(8), np.arange(8), indexing="ij"), -1).reshape(-1, 2).astype(np.float32)
    quads = []
    for x, z in g:
        a, b, c, d = (x, 0, z), (x + 1, 0, z), (x, 0, z + 1), (x + 1, 0, z + 1)
        quads += [[a, c, b], [b, c, d]]
    cases["coplanar_grid"] = np.array(quads, dtype=np.float32)
    cases["icosphere_f4"] = positions(scenes.icosphere(4))
    cases["soup_1000"] = positions(scenes.triangle_soup(1000, seed=5))
    cases["soup_20000"] = positions(scenes.triangle_soup(20000, seed=6))
    box = scenes.box_scene(width=8, height=8)
    cases["box_walls"] = positions(box.meshes[0])
    cases["box_icosphere"] = positions(box.meshes[1])
    cases["box_light"] = positions(box.meshes[2])
    return cases


def tlas_cases():
    rng = np.random.default_rng(99)
    out = {}
    for n in (1, 2, 3, 7, 64, 256):
        inst = np.zeros(n, dtype=bvh_instance_dtype)
        c = rng.random((n, 3)) * 100.0
        h = rng.random((n, 3)) * 3.0 + 0.1
        inst["aabb_min"] = (c - h).astype(np.float32)
        inst["aabb_max"] = (c + h).astype(np.float32)
        inst["world_to_local"] = np.eye(4, dtype=np.float32).reshape(16)
        inst["bvh_index"] = np.arange(n) % 3
        out[f"tlas_{n}"] = inst
    return out


def main():
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libref_bvh.so missing: run oracle/build_ref.sh first")
    data = {}
    for name, pos in mesh_cases().items():
        tris = tris_from_positions(pos)
        for ic, single in ((8, 0), (16, 0), (8, 1)):
            blob = oracle.ref_bvh_build(tris, ic, bool(single))
            key = f"bvh/{name}/ic{ic}_s{single}"
            if blob.nbytes <= MAX_INLINE:
                data[key] = blob
            else:
                data[key + "/sha256"] = np.frombuffer(hashlib.sha256(blob.tobytes()).digest(), np.uint8)
                data[key + "/size"] = np.array([blob.nbytes], np.uint64)
        data[f"pos/{name}"] = pos.astype(np.float32)
    for name, inst in tlas_cases().items():
        data[f"inst/{name}"] = inst.view(np.uint8)
        data[f"tlas/{name}"] = oracle.ref_tlas_build(inst)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(data)} arrays")


if __name__ == "__main__":
    main()
