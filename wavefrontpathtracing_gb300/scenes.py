"""Procedural scenes for the five benchmark configurations.

The reference renders glTF/FBX assets (source/core/scene.cpp:10-12); the
benchmark configurations are procedural instead, generated here with fixed
seeds so that the GPU library and the CPU oracle see identical bytes:

  box_scene()        small box scene: 12 axis-aligned quads, an icosphere
                     (subdivision 5, radius 0.3, centre (0.5,0.3,0.5)) and an
                     emissive ceiling quad of radiance 15; Lambert albedo per
                     mesh uniform in [0.2,0.8]^3 from PCG32 seed 1.
  mixed_box_scene()  the box scene's room with one sphere of each material
                     (Lambert, GGX metal, mirror-smooth metal, dielectric).
  instanced_scene()  8 noise-displaced icospheres, 1,024 instances with random
                     rotation, scale in [0.5,2], translation in a 100^3 box,
                     60/25/15 % Lambert/metal/dielectric, one area light.
  triangle_soup()    N triangles with centroids uniform in the unit cube and
                     log-normal edge lengths (mu=-5, sigma=0.5), seed 7.

Matrices follow the reference: glm lookAtLH / perspectiveFovLH_ZO
(renderer.cpp:614-629), stored column-major.
"""
import math

import numpy as np

from .abi import (BSDF_DIELECTRIC, BSDF_LAMBERT, BSDF_METAL, View, material_dtype, material_ext_dtype,
                  mat_f32, ray_dtype, triangle_dtype)

M64 = (1 << 64) - 1


class PCG32:
    """O'Neill's PCG-XSH-RR 32-bit generator (pcg32_srandom / pcg32_random)."""

    def __init__(self, initstate, initseq=54):
        self.state = 0
        self.inc = ((initseq << 1) | 1) & M64
        self.next_u32()
        self.state = (self.state + initstate) & M64
        self.next_u32()

    def next_u32(self):
        old = self.state
        self.state = (old * 6364136223846793005 + self.inc) & M64
        xorshifted = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u32() >> 8) * (1.0 / (1 << 24)))


# --------------------------------------------------------------------------- geometry

def _tris_from_arrays(p0, p1, p2, n0=None, n1=None, n2=None):
    """Packs positions (and vertex normals; face normals if None) into triangle_t.
    Adding +0.0 turns any -0.0 coordinate into +0.0."""
    n = len(p0)
    t = np.zeros(n, dtype=triangle_dtype)
    if n0 is None:
        fn = np.cross(p1 - p0, p2 - p0)
        fn /= np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-30)
        n0 = n1 = n2 = fn
    for name, p, nn in (("v0", p0, n0), ("v1", p1, n1), ("v2", p2, n2)):
        t[name]["position"] = np.asarray(p, dtype=np.float32) + np.float32(0.0)
        t[name]["normal"] = np.asarray(nn, dtype=np.float32) + np.float32(0.0)
        t[name]["tangent"] = (1.0, 0.0, 0.0, 1.0)
    return t


def icosahedron():
    g = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, g, 0], [1, g, 0], [-1, -g, 0], [1, -g, 0], [0, -1, g], [0, 1, g], [0, -1, -g],
                  [0, 1, -g], [g, 0, -1], [g, 0, 1], [-g, 0, -1], [-g, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    return v, f


def unit_icosphere_indexed(freq):
    """Geodesic sphere as (vertices, triangles): every icosahedron face carries
    a grid of (freq+1)(freq+2)/2 points A + (B-A) i/freq + (C-A) j/freq
    projected to the unit sphere (points on shared edges repeat per face), and
    freq^2 triangles over it (20*freq^2 in all; freq = 2^k is subdivision level
    k), wound so that (p1-p0)x(p2-p0) points outward (front faces under
    back-face culling)."""
    v, faces = icosahedron()
    grid = [(i, j) for i in range(freq + 1) for j in range(freq + 1 - i)]
    gidx = {ij: k for k, ij in enumerate(grid)}
    st = np.array(grid, dtype=np.float64) / freq
    ii, jj = [], []
    for i in range(freq):
        for j in range(freq - i):
            ii.append((gidx[(i, j)], gidx[(i + 1, j)], gidx[(i, j + 1)]))
            if i + j < freq - 1:
                jj.append((gidx[(i + 1, j)], gidx[(i + 1, j + 1)], gidx[(i, j + 1)]))
    local = np.array(ii + jj, dtype=np.int64)
    ng = len(grid)
    V, F = [], []
    for f, (a, b, c) in enumerate(faces):
        A, B, C = v[a], v[b], v[c]
        V.append(A + (B - A) * st[:, 0:1] + (C - A) * st[:, 1:2])
        F.append(local + f * ng)
    V = np.concatenate(V)
    F = np.concatenate(F)
    V = V / np.linalg.norm(V, axis=1, keepdims=True)
    p0, p1, p2 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    fn = np.cross(p1 - p0, p2 - p0)
    flip = np.einsum("ij,ij->i", fn, p0 + p1 + p2) < 0
    F[flip, 1], F[flip, 2] = F[flip, 2].copy(), F[flip, 1].copy()
    return V, F


def unit_icosphere(freq):
    """unit_icosphere_indexed as float64 (p0, p1, p2) triangle corner arrays."""
    V, F = unit_icosphere_indexed(freq)
    return V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]


def icosphere(freq, center=(0.0, 0.0, 0.0), radius=1.0):
    p0, p1, p2 = unit_icosphere(freq)
    c = np.asarray(center, dtype=np.float64)
    return _tris_from_arrays(p0 * radius + c, p1 * radius + c, p2 * radius + c, p0, p1, p2)


def _value_noise(p, seed, cells=4.0):
    """Trilinear value noise with smoothstep weights on a seeded integer lattice, in [-1, 1]."""
    q = p * cells
    i0 = np.floor(q).astype(np.int64)
    f = q - i0
    w = f * f * (3.0 - 2.0 * f)

    def h(ix, iy, iz):
        x = (ix * 73856093) ^ (iy * 19349663) ^ (iz * 83492791) ^ (seed * 2654435761)
        x = (x ^ (x >> 13)) * 1274126177
        x = x ^ (x >> 16)
        return ((x & 0xFFFFFF) / float(0xFFFFFF)) * 2.0 - 1.0

    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out = out + wx * wy * wz * h(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
    return out


def displaced_icosphere(freq, seed, amplitude=0.1):
    """Unit icosphere whose radius is 1 + amplitude * value_noise(direction)."""
    V, F = unit_icosphere_indexed(freq)
    P = V * (1.0 + amplitude * _value_noise(V, seed))[:, None]
    return _tris_from_arrays(P[F[:, 0]], P[F[:, 1]], P[F[:, 2]], V[F[:, 0]], V[F[:, 1]], V[F[:, 2]])


def quad(origin, e1, e2):
    """Two triangles spanning origin + s*e1 + t*e2; front side is e1 x e2."""
    o, a, b = (np.asarray(x, dtype=np.float64) for x in (origin, e1, e2))
    p0 = np.array([o, o + a + b])
    p1 = np.array([o + a, o + b])
    p2 = np.array([o + a + b, o])
    # (o, o+a, o+a+b) and (o+a+b, o+b, o): both wound like (e1, e2)
    return _tris_from_arrays(p0, p1, p2)


# --------------------------------------------------------------------------- cameras

def look_at_lh(eye, center, up=(0.0, 1.0, 0.0)):
    eye, center, up = (np.asarray(x, dtype=np.float64) for x in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(up, f)
    s /= np.linalg.norm(s)
    u = np.cross(f, s)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, -f @ eye
    return m


def perspective_fov_lh_zo(vfov_rad, width, height, near, far):
    h = math.cos(0.5 * vfov_rad) / math.sin(0.5 * vfov_rad)
    w = h * height / width
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = w, h
    m[2, 2] = far / (far - near)
    m[2, 3] = -(far * near) / (far - near)
    m[3, 2] = 1.0
    return m


def make_view(eye, target, vfov_deg, width, height, near=0.01, far=1000.0):
    """view_t as renderer::begin_scene fills it (renderer.cpp:614-629)."""
    V = look_at_lh(eye, target)
    P = perspective_fov_lh_zo(math.radians(vfov_deg), width, height, near, far)
    v = View()
    v.world_to_view[:] = mat_f32(V).tolist()
    v.view_to_world[:] = mat_f32(np.linalg.inv(V)).tolist()
    v.view_to_clip[:] = mat_f32(P).tolist()
    v.clip_to_view[:] = mat_f32(np.linalg.inv(P)).tolist()
    v.render_dim[:] = [float(width), float(height)]
    v.near_plane, v.far_plane = near, far
    return v


# --------------------------------------------------------------------------- materials

def material(base=(0.8, 0.8, 0.8), emissive=(0.0, 0.0, 0.0), strength=0.0, bsdf=BSDF_LAMBERT, roughness=1.0,
             metallic=0.0, ior=1.5):
    m = np.zeros(1, dtype=material_ext_dtype)[0]
    m["base"]["base_color_factor"] = base
    m["base"]["metallic_factor"] = metallic
    m["base"]["roughness_factor"] = roughness
    m["base"]["emissive_factor"] = emissive
    m["base"]["emissive_strength"] = strength
    m["bsdf"] = bsdf
    m["ior"] = ior
    return m


def translate_scale(t, s=1.0, rot=None):
    m = np.eye(4)
    m[:3, :3] = (np.eye(3) if rot is None else rot) * s
    m[:3, 3] = t
    return m


def random_rotation(rng):
    """Uniform random rotation from a unit quaternion (Shoemake)."""
    u1, u2, u3 = rng.uniform(), rng.uniform(), rng.uniform()
    a, b = math.sqrt(1 - u1), math.sqrt(u1)
    x, y, z, w = (a * math.sin(2 * math.pi * u2), a * math.cos(2 * math.pi * u2),
                  b * math.sin(2 * math.pi * u3), b * math.cos(2 * math.pi * u3))
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


# --------------------------------------------------------------------------- configurations

class SceneDesc:
    """meshes: list of triangle_t arrays; instances: list of (mesh, local_to_world 4x4, material_ext)."""

    def __init__(self, name, meshes, instances, view, width, height, settings, bvh_options):
        self.name, self.meshes, self.instances, self.view = name, meshes, instances, view
        self.width, self.height, self.settings, self.bvh_options = width, height, settings, bvh_options

    @property
    def triangle_count(self):
        return sum(len(m) for m in self.meshes)

    @property
    def instanced_triangle_count(self):
        return sum(len(self.meshes[i]) for i, _, _ in self.instances)


def box_scene(width=256, height=256, subdivision=5, max_bounces=4, spp=1):
    """The small plain-method configuration (Lambert only, reference shading)."""
    rng = PCG32(1)
    walls = []
    # room [0,1]^3, six inward-facing walls
    walls.append(quad((0, 0, 0), (0, 0, 1), (1, 0, 0)))      # floor, +y
    walls.append(quad((0, 1, 0), (1, 0, 0), (0, 0, 1)))      # ceiling, -y
    walls.append(quad((0, 0, 1), (0, 1, 0), (1, 0, 0)))      # back, -z
    walls.append(quad((0, 0, 0), (1, 0, 0), (0, 1, 0)))      # front, +z (culled from the camera)
    walls.append(quad((0, 0, 0), (0, 1, 0), (0, 0, 1)))      # left, +x
    walls.append(quad((1, 0, 0), (0, 0, 1), (0, 1, 0)))      # right, -x
    # an outward-facing block
    x0, x1, y0, y1, z0, z1 = 0.82, 0.98, 0.0, 0.4, 0.1, 0.3
    dx, dy, dz = (x1 - x0, 0, 0), (0, y1 - y0, 0), (0, 0, z1 - z0)
    walls.append(quad((x0, y1, z0), dz, dx))                  # top, +y
    walls.append(quad((x0, y0, z0), dx, dz))                  # bottom, -y
    walls.append(quad((x0, y0, z0), dy, dx))                  # front, -z
    walls.append(quad((x0, y0, z1), dx, dy))                  # back, +z
    walls.append(quad((x0, y0, z0), dz, dy))                  # left, -x
    walls.append(quad((x1, y0, z0), dy, dz))                  # right, +x
    box = np.concatenate(walls)
    sphere = icosphere(2 ** subdivision, center=(0.5, 0.3, 0.5), radius=0.3)
    light = quad((0.35, 0.998, 0.35), (0.3, 0, 0), (0, 0, 0.3))   # faces -y
    albedo = [tuple(rng.uniform(0.2, 0.8) for _ in range(3)) for _ in range(3)]
    instances = [
        (0, np.eye(4), material(base=albedo[0])),
        (1, np.eye(4), material(base=albedo[1])),
        (2, np.eye(4), material(base=albedo[2], emissive=(1.0, 1.0, 1.0), strength=15.0)),
    ]
    view = make_view((0.5, 0.5, -1.2), (0.5, 0.45, 0.5), 45.0, width, height)
    settings = dict(max_bounces=max_bounces, spp=spp, nee=0, rr_start_depth=0xFFFFFFFF, env=(0.0, 0.0, 0.0),
                    env_strength=1.0, cosine=1)
    return SceneDesc("box", [box, sphere, light], instances, view, width, height, settings,
                     dict(interval_count=16, subdivide_single_prim=0, max_leaf_prims=4))


def mixed_box_scene(width=80, height=60, subdivision=3, max_bounces=8, spp=1):
    """The box scene's room (walls and block, Lambert) with one sphere of each
    of the instanced configuration's materials standing on the floor —
    Lambert, GGX metal at roughness 0.3 and 0.1, a metal smooth enough to be a
    mirror (roughness 0.005, alpha below 1e-4) and a dielectric of IOR 1.5 —
    under a 0.5 x 0.5 ceiling light of radiance 6; next-event estimation and
    Russian roulette from depth 3, as the instanced configuration renders."""
    box = box_scene(width, height, subdivision=1).meshes[0]
    sphere = icosphere(2 ** subdivision)
    light = quad((0.25, 0.998, 0.25), (0.5, 0, 0), (0, 0, 0.5))   # faces -y
    rng = PCG32(4)
    wall = tuple(rng.uniform(0.3, 0.8) for _ in range(3))
    instances = [
        (0, np.eye(4), material(base=wall)),
        (2, np.eye(4), material(base=(0.8, 0.8, 0.8), emissive=(1.0, 0.95, 0.9), strength=6.0)),
        (1, translate_scale((0.22, 0.13, 0.62), 0.13), material(base=(0.75, 0.3, 0.25))),
        (1, translate_scale((0.50, 0.14, 0.68), 0.14),
         material(base=(0.9, 0.7, 0.4), bsdf=BSDF_METAL, roughness=0.3, metallic=1.0)),
        (1, translate_scale((0.72, 0.11, 0.48), 0.11),
         material(base=(0.6, 0.8, 0.9), bsdf=BSDF_METAL, roughness=0.1, metallic=1.0)),
        (1, translate_scale((0.35, 0.12, 0.30), 0.12),
         material(base=(0.95, 0.95, 0.95), bsdf=BSDF_METAL, roughness=0.005, metallic=1.0)),
        (1, translate_scale((0.60, 0.14, 0.20), 0.14), material(base=(1.0, 1.0, 1.0), bsdf=BSDF_DIELECTRIC, ior=1.5)),
    ]
    view = make_view((0.5, 0.38, -0.55), (0.48, 0.16, 0.45), 45.0, width, height)   # the spheres fill the frame
    settings = dict(max_bounces=max_bounces, spp=spp, nee=1, rr_start_depth=3, env=(0.0, 0.0, 0.0),
                    env_strength=1.0, cosine=1)
    return SceneDesc("mixed_box", [box, sphere, light], instances, view, width, height, settings,
                     dict(interval_count=16, subdivide_single_prim=0, max_leaf_prims=4))


# Geodesic frequencies whose 20*f^2 triangle counts come closest to 50k/100k/200k/500k.
INSTANCED_FREQS = (50, 71, 100, 158)


def instanced_scene(width=1920, height=1080, instances=1024, freqs=INSTANCED_FREQS, spp=16, max_bounces=8,
                    seed=3):
    """The instanced configuration: 8 displaced icospheres (two noise seeds per
    frequency), `instances` random instances, mixed materials, one area light."""
    rng = PCG32(seed)
    meshes = []
    for k, f in enumerate(list(freqs) * 2):
        meshes.append(displaced_icosphere(f, seed=11 + k, amplitude=0.1))
    light_mesh = len(meshes)
    meshes.append(quad((30.0, 110.0, 30.0), (40.0, 0, 0), (0, 0, 40.0)))   # faces -y
    inst = []
    nblas = len(freqs) * 2
    for i in range(instances):
        mesh = i % nblas
        rot = random_rotation(rng)
        s = rng.uniform(0.5, 2.0)
        t = (rng.uniform(0, 100), rng.uniform(0, 100), rng.uniform(0, 100))
        u = rng.uniform()
        base = (rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9))
        rough = rng.uniform(0.0, 0.5)
        if u < 0.60:
            m = material(base=base)
        elif u < 0.85:
            m = material(base=base, bsdf=BSDF_METAL, roughness=rough, metallic=1.0)
        else:
            m = material(base=(1.0, 1.0, 1.0), bsdf=BSDF_DIELECTRIC, ior=1.5)
        inst.append((mesh, translate_scale(t, s, rot), m))
    inst.append((light_mesh, np.eye(4), material(base=(0.8, 0.8, 0.8), emissive=(1.0, 0.95, 0.9), strength=60.0)))
    view = make_view((50.0, 55.0, -75.0), (50.0, 45.0, 50.0), 55.0, width, height)
    settings = dict(max_bounces=max_bounces, spp=spp, nee=1, rr_start_depth=3, env=(0.0, 0.0, 0.0),
                    env_strength=1.0, cosine=1)
    return SceneDesc("instanced", meshes, inst, view, width, height, settings,
                     dict(interval_count=16, subdivide_single_prim=0, max_leaf_prims=4))


class BatchSceneDesc:
    """One scene of a batch: instances = list of (mesh index into the batch's
    mesh list, local_to_world 4x4, material_ext)."""

    def __init__(self, width, height, spp, view, instances, env, sphere_triangles):
        self.width, self.height, self.spp, self.view = width, height, spp, view
        self.instances, self.env, self.sphere_triangles = instances, env, sphere_triangles

    @property
    def paths(self):
        return self.width * self.height * self.spp


def batch_scenes(count=64, seed=5, tri_range=(1_000, 2_000_000), resolutions=(64, 128, 256, 512, 1024),
                 spps=(1, 4, 16)):
    """The batched configuration: `count` scenes, each a seeded displaced
    icosphere soup whose triangle count is log-uniform in tri_range (geodesic
    frequency round(sqrt(n / 20)), so 20 * freq^2 triangles), a square image
    with its side drawn from `resolutions`, spp drawn from `spps`, and a
    material from the 60/25/15 Lambert / metal / dielectric mix.  Every scene
    also holds a ground quad and an emissive quad light (two meshes shared by
    all scenes).  Returns (meshes, scenes): meshes[0] ground, meshes[1] light,
    meshes[2 + k] scene k's soup."""
    rng = PCG32(seed)
    ground = quad((-6.0, -1.25, 6.0), (12.0, 0.0, 0.0), (0.0, 0.0, -12.0))   # faces +y
    light = quad((-0.75, 3.0, -0.75), (1.5, 0.0, 0.0), (0.0, 0.0, 1.5))     # faces -y
    meshes = [ground, light]
    scenes = []
    lo, hi = math.log(tri_range[0]), math.log(tri_range[1])
    for k in range(count):
        n = math.exp(rng.uniform(lo, hi))
        freq = max(1, int(round(math.sqrt(n / 20.0))))
        meshes.append(displaced_icosphere(freq, seed=1000 + k, amplitude=0.1))
        side = resolutions[rng.next_u32() % len(resolutions)]
        spp = spps[rng.next_u32() % len(spps)]
        u = rng.uniform()
        base = (rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9))
        rough = rng.uniform(0.0, 0.5)
        if u < 0.60:
            m = material(base=base)
        elif u < 0.85:
            m = material(base=base, bsdf=BSDF_METAL, roughness=rough, metallic=1.0)
        else:
            m = material(base=(1.0, 1.0, 1.0), bsdf=BSDF_DIELECTRIC, ior=1.5)
        az = rng.uniform(0.0, 2.0 * math.pi)
        el = rng.uniform(0.15, 0.6)
        eye = (3.6 * math.cos(el) * math.sin(az), 3.6 * math.sin(el), -3.6 * math.cos(el) * math.cos(az))
        view = make_view(eye, (0.0, 0.0, 0.0), 45.0, side, side)
        inst = [(2 + k, np.eye(4), m),
                (0, np.eye(4), material(base=(0.6, 0.6, 0.6))),
                (1, np.eye(4), material(base=(0.8, 0.8, 0.8), emissive=(1.0, 0.95, 0.9), strength=25.0))]
        scenes.append(BatchSceneDesc(side, side, spp, view, inst, (0.05, 0.06, 0.08), len(meshes[-1])))
    return meshes, scenes


def triangle_soup(n, seed=7, mu=-5.0, sigma=0.5):
    """n triangles: centroid uniform in [0,1]^3, three vertices at centroid +
    L * (random unit vector), L log-normal(mu, sigma).  The random draws are
    made in one stream; the per-triangle arithmetic runs on row blocks in
    threads (the same operations on every row, so the result does not depend
    on the split)."""
    import concurrent.futures
    import os
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3), dtype=np.float64)
    L = rng.lognormal(mu, sigma, size=(n, 1))
    dirs = rng.normal(size=(n, 3, 3))
    out = np.zeros(n, dtype=triangle_dtype)

    def block(lo, hi):
        d = dirs[lo:hi]
        d /= np.linalg.norm(d, axis=2, keepdims=True)
        p = c[lo:hi, None, :] + L[lo:hi, None, :] * d
        p -= p.mean(axis=1, keepdims=True) - c[lo:hi, None, :]
        out[lo:hi] = _tris_from_arrays(p[:, 0], p[:, 1], p[:, 2])

    step = 1 << 18
    with concurrent.futures.ThreadPoolExecutor(min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(lambda lo: block(lo, min(n, lo + step)), range(0, n, step)))
    return out


def soup_rays(n_side, seed=7, kind="coherent"):
    """Rays for the traversal micro-benchmark.  coherent: pinhole camera at
    (0.5, 0.5, -0.5) looking down +z with a 90-degree field of view, so the
    n_side^2 rays enter the unit cube through its z = 0 face (at distance 0.5
    .. 0.87) and an any-hit query with tmax U[0, 1] ends on either side of the
    first triangle; incoherent: origins uniform in the cube, directions
    uniform on the sphere."""
    n = n_side * n_side
    r = np.zeros(n, dtype=ray_dtype)
    if kind == "coherent":
        ys, xs = np.divmod(np.arange(n, dtype=np.int64), n_side)
        u = (xs + 0.5) / n_side * 2.0 - 1.0
        v = 1.0 - (ys + 0.5) / n_side * 2.0
        half = math.tan(math.radians(45.0))
        d = np.stack([u * half, v * half, np.ones_like(u)], axis=1)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        r["origin"] = (0.5, 0.5, -0.5)
        r["dir"] = d
    else:
        rng = np.random.default_rng(seed + 1)
        r["origin"] = rng.random((n, 3))
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        r["dir"] = d
    r["origin"] += np.float32(0.0)
    r["dir"] += np.float32(0.0)
    r["tmin"] = 1e-8
    r["tmax"] = np.finfo(np.float32).max
    return r
