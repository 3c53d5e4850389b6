"""An independently written FP64 path tracer for the mixed-material scenes.

Test infrastructure only.  It shares nothing with the oracle's shading code:
its own random numbers (numpy's PCG64), its own orthonormal bases, its own
samplers written from the formulas (cosine-weighted hemisphere; GGX half
vectors from the inverse CDF tan^2 = a2 u / (1 - u); Fresnel's equations and
Snell's law for the dielectric), BSDF sampling only — no next-event
estimation, no multiple importance sampling, no Russian roulette — so it
converges to the same image as the oracle's estimator by a different route.
Only the ray cast is shared: the oracle's FP64 query, which is pinned to the
reference's traversal text (tests/test_ref_hlsl.py).

The scene model it implements (the one the oracle and the GPU library
render): camera rays without jitter (the reference's make_primary_ray);
back faces culled except for rays travelling inside a dielectric; an
emitter's emission ends the path; a miss adds the environment; opaque
surfaces met from inside glass are shaded from the side the ray arrives on;
metal alpha = roughness^2, a mirror below alpha 1e-4, Schlick F with
F0 = base colour; path length up to max_bounces + 1 segments.
"""
import math

import numpy as np

from wavefrontpathtracing_gb300.abi import hit_dtype, ray_dtype

ANY_HIT, NO_CULL = 1, 2


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _frame(n):
    """An orthonormal basis (t, b) around each normal (Duff et al. 2017)."""
    s = np.where(n[:, 2] >= 0.0, 1.0, -1.0)
    a = -1.0 / (s + n[:, 2])
    b = n[:, 0] * n[:, 1] * a
    t = np.stack([1.0 + s * n[:, 0] ** 2 * a, s * b, -s * n[:, 0]], axis=1)
    bt = np.stack([b, s + n[:, 1] ** 2 * a, -n[:, 1]], axis=1)
    return t, bt


def _dot(a, b):
    return np.sum(a * b, axis=1)


class IndependentTracer:
    def __init__(self, orc_scene, desc):
        self.sc = orc_scene
        inst = orc_scene._inst
        self.l2w = np.array([np.asarray(m, np.float64).reshape(4, 4).T for m in inst["local_to_world"]])  # row-major
        mat = inst["material"]
        self.base = np.asarray(mat["base_color_factor"], np.float64)
        self.le = np.asarray(mat["emissive_factor"], np.float64) * np.asarray(mat["emissive_strength"], np.float64)[:, None]
        self.rough = np.asarray(mat["roughness_factor"], np.float64)
        self.bsdf = np.asarray(inst["bsdf"])
        self.ior = np.asarray(inst["ior"], np.float64)
        self.mesh = np.asarray(inst["mesh"])
        self.tris = orc_scene._tris
        self.env = np.asarray(desc.settings["env"], np.float64) * desc.settings["env_strength"]
        self.max_bounces = desc.settings["max_bounces"]

    def _surface(self, hit):
        """World position and shading normal at each hit."""
        inst, prim = hit["instance"].astype(np.int64), hit["primitive"].astype(np.int64)
        u = hit["bary"][:, 0].astype(np.float64)[:, None]
        v = hit["bary"][:, 1].astype(np.float64)[:, None]
        p = np.zeros((len(hit), 3))
        nrm = np.zeros((len(hit), 3))
        for m in np.unique(self.mesh[inst]):
            sel = self.mesh[inst] == m
            t = self.tris[m][prim[sel]]
            P = [t[k]["position"].astype(np.float64) for k in ("v0", "v1", "v2")]
            Nn = [t[k]["normal"].astype(np.float64) for k in ("v0", "v1", "v2")]
            p[sel] = (1.0 - u[sel] - v[sel]) * P[0] + u[sel] * P[1] + v[sel] * P[2]
            nrm[sel] = (1.0 - u[sel] - v[sel]) * Nn[0] + u[sel] * Nn[1] + v[sel] * Nn[2]
        M = self.l2w[inst]
        pw = np.einsum("nij,nj->ni", M[:, :3, :3], p) + M[:, :3, 3]
        nw = _unit(np.einsum("nij,nj->ni", M[:, :3, :3], nrm))
        return pw, nw

    def render(self, view_rays, spp, seed, threads=8):
        """view_rays: the camera ray of each pixel (ray_dtype, row-major).
        Returns (mean radiance per pixel, per-sample radiance [spp, pixels, 3])."""
        rng = np.random.default_rng(seed)
        npx = len(view_rays)
        M = npx * spp
        o = np.repeat(view_rays["origin"].astype(np.float64)[None], spp, 0).reshape(M, 3)
        d = np.repeat(view_rays["dir"].astype(np.float64)[None], spp, 0).reshape(M, 3)
        T = np.ones((M, 3))
        Lsum = np.zeros((M, 3))
        alive = np.ones(M, bool)
        inside = np.zeros(M, bool)
        for depth in range(self.max_bounces + 1):
            idx = np.nonzero(alive)[0]
            if len(idx) == 0:
                break
            hit = np.zeros(len(idx), dtype=hit_dtype)
            for flags, sel in ((0, ~inside[idx]), (NO_CULL, inside[idx])):
                if not sel.any():
                    continue
                rays = np.zeros(int(sel.sum()), ray_dtype)
                rays["origin"] = o[idx[sel]]
                rays["dir"] = d[idx[sel]]
                rays["tmin"] = 1e-8
                rays["tmax"] = np.finfo(np.float32).max
                h, _, _ = self.sc.trace(rays, flags=flags, threads=threads, f64=True)
                hit[sel] = h
            miss = hit["instance"] == 0xFFFFFFFF
            Lsum[idx[miss]] += T[idx[miss]] * self.env
            alive[idx[miss]] = False
            idx, hit = idx[~miss], hit[~miss]
            if len(idx) == 0:
                break
            inst = hit["instance"].astype(np.int64)
            le = self.le[inst]
            emit = np.any(le != 0.0, axis=1)
            Lsum[idx[emit]] += T[idx[emit]] * le[emit]
            alive[idx[emit]] = False
            idx, hit, inst = idx[~emit], hit[~emit], inst[~emit]
            if len(idx) == 0 or depth == self.max_bounces:
                alive[idx] = False
                break
            p, n = self._surface(hit)
            V = -_unit(d[idx])
            kind = self.bsdf[inst].copy()
            alpha = self.rough[inst] ** 2
            kind[(kind == 1) & (alpha < 1e-4)] = 3
            flip = inside[idx] & (kind != 2) & (_dot(n, V) < 0.0)
            n[flip] = -n[flip]
            base = self.base[inst]
            u1, u2 = rng.random(len(idx)), rng.random(len(idx))
            newd = np.zeros((len(idx), 3))
            w = np.zeros((len(idx), 3))
            ok = np.ones(len(idx), bool)
            neworg = p.copy()
            toggle = np.zeros(len(idx), bool)
            tb, bb = _frame(n)
            # Lambert: cosine-weighted hemisphere, weight = albedo
            s = kind == 0
            if s.any():
                r = np.sqrt(u1[s])
                ph = 2.0 * math.pi * u2[s]
                loc = np.stack([r * np.cos(ph), r * np.sin(ph), np.sqrt(np.maximum(0.0, 1.0 - u1[s]))], 1)
                newd[s] = loc[:, :1] * tb[s] + loc[:, 1:2] * bb[s] + loc[:, 2:] * n[s]
                w[s] = base[s]
                ok[s] = _dot(newd[s], n[s]) > 0.0
            # GGX metal: half vector from D(h)(n.h), weight f cos / pdf
            s = kind == 1
            if s.any():
                a2 = alpha[s] ** 2
                t2 = a2 * u1[s] / (1.0 - u1[s])
                ch = 1.0 / np.sqrt(1.0 + t2)
                sh = np.sqrt(np.maximum(0.0, 1.0 - ch * ch))
                ph = 2.0 * math.pi * u2[s]
                h = (sh * np.cos(ph))[:, None] * tb[s] + (sh * np.sin(ph))[:, None] * bb[s] + ch[:, None] * n[s]
                vh = _dot(V[s], h)
                Ld = 2.0 * vh[:, None] * h - V[s]
                nl, nv, nh = _dot(n[s], Ld), _dot(n[s], V[s]), _dot(n[s], h)
                good = (nl > 0) & (nv > 0) & (vh > 0) & (nh > 0)
                q = nh * nh * (a2 - 1.0) + 1.0
                D = a2 / (math.pi * q * q)
                g1 = lambda x: 2.0 * x / (x + np.sqrt(a2 + (1.0 - a2) * x * x))
                F = base[s] + (1.0 - base[s]) * ((1.0 - vh) ** 5)[:, None]
                with np.errstate(all="ignore"):
                    f = F * (D * g1(nl) * g1(nv) / (4.0 * nv * nl))[:, None]
                    pdf = D * nh / (4.0 * vh)
                    ww = f * (nl / pdf)[:, None]
                newd[s] = Ld
                w[s] = np.where(good[:, None], ww, 0.0)
                ok[s] = good
            # mirror: perfect reflection, Schlick F at n.v
            s = kind == 3
            if s.any():
                nv = _dot(n[s], V[s])
                newd[s] = 2.0 * nv[:, None] * n[s] - V[s]
                w[s] = base[s] + (1.0 - base[s]) * ((1.0 - nv) ** 5)[:, None]
                ok[s] = nv > 0
            # smooth dielectric: Fresnel's equations choose reflection, Snell refracts
            s = kind == 2
            if s.any():
                ior = self.ior[inst][s]
                cn = _dot(V[s], n[s])
                ent = cn > 0
                n1, n2 = np.where(ent, 1.0, ior), np.where(ent, ior, 1.0)
                nn = np.where(ent[:, None], n[s], -n[s])
                ci = np.abs(cn)
                eta = n1 / n2
                s2t = eta * eta * (1.0 - ci * ci)
                tir = s2t >= 1.0
                ct = np.sqrt(np.maximum(0.0, 1.0 - s2t))
                with np.errstate(all="ignore"):
                    rs = (n1 * ci - n2 * ct) / (n1 * ci + n2 * ct)
                    rp = (n1 * ct - n2 * ci) / (n1 * ct + n2 * ci)
                Fr = np.where(tir, 1.0, 0.5 * (rs * rs + rp * rp))
                refl = u1[s] < Fr
                din = -V[s]
                rdir = din + 2.0 * ci[:, None] * nn
                tdir = _unit(eta[:, None] * din + (eta * ci - ct)[:, None] * nn)
                newd[s] = np.where(refl[:, None], rdir, tdir)
                w[s] = 1.0
                toggle[s] = ~refl
                pp = p[s]
                neworg[s] = pp + newd[s] * (1e-4 * (1.0 + np.max(np.abs(pp), axis=1)))[:, None]
            T[idx] *= w
            alive[idx[~ok]] = False
            inside[idx[toggle]] = ~inside[idx[toggle]]
            o[idx] = neworg
            d[idx] = newd
        per_sample = Lsum.reshape(spp, npx, 3)
        return per_sample.mean(0), per_sample
