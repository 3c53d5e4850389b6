"""Test helpers: build oracle scenes from scene descriptions or from what the
GPU library reports (instances, TLAS), so both sides see identical bytes."""
import numpy as np

from wavefrontpathtracing_gb300.abi import bvh_instance_dtype, mat_f32


def inv_f32(m4):
    return mat_f32(np.linalg.inv(np.asarray(m4, dtype=np.float64)))


def single_instance_scene(orc, meshes, interval_count=16, max_leaf=4):
    """meshes: list of triangle arrays, one identity instance each."""
    built = [(t, orc.bvh_build(t, interval_count, False, max_leaf)) for t in meshes]
    inst = np.zeros(len(meshes), dtype=bvh_instance_dtype)
    oi = np.zeros(len(meshes), dtype=orc.instance_dtype)
    for i, (t, blob) in enumerate(built):
        h = blob[:12].view(np.uint32)
        root = blob[12:44].view(np.float32)
        inst[i]["world_to_local"] = np.eye(4, dtype=np.float32).reshape(16)
        inst[i]["aabb_min"] = root[0:3]
        inst[i]["aabb_max"] = root[4:7]
        inst[i]["bvh_index"] = i
        oi[i]["local_to_world"] = np.eye(4, dtype=np.float32).reshape(16)
        oi[i]["world_to_local"] = np.eye(4, dtype=np.float32).reshape(16)
        oi[i]["mesh"] = i
        oi[i]["material"]["base_color_factor"] = (0.5, 0.5, 0.5)
        del h
    return orc.Scene(built, orc.tlas_build(inst), oi)


def instance_aabb(root_min, root_max, l2w):
    """World box of a BLAS root box (renderer.cpp:1324-1336), glm pairwise mat*vec order."""
    m = np.asarray(l2w, dtype=np.float32).reshape(16)
    mn = np.full(3, np.finfo(np.float32).max, np.float32)
    mx = -mn
    for i in range(8):
        c = np.array([root_max[0] if i & 1 else root_min[0], root_max[1] if i & 2 else root_min[1],
                      root_max[2] if i & 4 else root_min[2]], np.float32)
        w = np.zeros(3, np.float32)
        for j in range(3):
            a0 = np.float32(m[j] * c[0])
            a1 = np.float32(m[4 + j] * c[1])
            a2 = np.float32(m[8 + j] * c[2])
            a3 = np.float32(m[12 + j] * np.float32(1.0))
            w[j] = np.float32(np.float32(a0 + a1) + np.float32(a2 + a3))
        mn = np.where(w < mn, w, mn)
        mx = np.where(mx < w, w, mx)
    return mn, mx


def oracle_scene_from_desc(orc, desc, blobs=None, w2l=None):
    """Oracle scene for a scenes.SceneDesc.  blobs: BLAS blobs per mesh (default:
    built by the oracle with the description's options); w2l: per-instance
    world_to_local (default: float64 inverse rounded to float32)."""
    o = desc.bvh_options
    if blobs is None:
        blobs = [orc.bvh_build(t, o["interval_count"], bool(o["subdivide_single_prim"]), o["max_leaf_prims"])
                 for t in desc.meshes]
    n = len(desc.instances)
    bi = np.zeros(n, dtype=bvh_instance_dtype)
    oi = np.zeros(n, dtype=orc.instance_dtype)
    for k, (mesh, l2w, mat) in enumerate(desc.instances):
        l2w16 = mat_f32(l2w)
        wl = inv_f32(l2w) if w2l is None else w2l[k]
        root = blobs[mesh][12:44].view(np.float32)
        mn, mx = instance_aabb(root[0:3], root[4:7], l2w16)
        bi[k]["world_to_local"] = wl
        bi[k]["aabb_min"], bi[k]["aabb_max"] = mn, mx
        bi[k]["bvh_index"] = mesh
        oi[k]["local_to_world"] = l2w16
        oi[k]["world_to_local"] = wl
        oi[k]["material"] = mat["base"]
        oi[k]["mesh"] = mesh
        oi[k]["bsdf"] = mat["bsdf"]
        oi[k]["ior"] = mat["ior"]
    meshes = list(zip(desc.meshes, blobs))
    return orc.Scene(meshes, orc.tlas_build(bi), oi)


def oracle_scene_from_renderer(orc, desc, r, mesh_ids):
    """Oracle scene built from the GPU library's own BLAS blobs, instances and
    TLAS (read back through the C ABI)."""
    blobs = [r.mesh_blas(m) for m in mesh_ids]
    bi = r.scene_instances()
    tlas = r.scene_tlas()
    n = len(desc.instances)
    oi = np.zeros(n, dtype=orc.instance_dtype)
    for k, (mesh, l2w, mat) in enumerate(desc.instances):
        oi[k]["local_to_world"] = mat_f32(l2w)
        oi[k]["world_to_local"] = bi[k]["world_to_local"]
        oi[k]["material"] = mat["base"]
        oi[k]["mesh"] = mesh
        oi[k]["bsdf"] = mat["bsdf"]
        oi[k]["ior"] = mat["ior"]
    return orc.Scene(list(zip(desc.meshes, blobs)), tlas, oi), bi


def load_scene_into(r, desc, prebuilt_blobs=None):
    """Creates the description's meshes and instances in a GPU Renderer."""
    o = desc.bvh_options
    ids = []
    for i, t in enumerate(desc.meshes):
        if prebuilt_blobs is not None:
            ids.append(r.create_mesh_prebuilt(t, prebuilt_blobs[i]))
        else:
            ids.append(r.create_mesh_from_triangles(t, interval_count=o["interval_count"],
                                                    subdivide_single_prim=bool(o["subdivide_single_prim"]),
                                                    max_leaf_prims=o["max_leaf_prims"]))
    r.begin_scene(desc.view, desc.settings["env"])
    for mesh, l2w, mat in desc.instances:
        r.submit_render_mesh(ids[mesh], l2w, mat)
    r.end_scene()
    return ids
