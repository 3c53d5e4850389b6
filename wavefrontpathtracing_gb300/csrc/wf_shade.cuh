// wf_shade.cuh — per-path shading arithmetic shared by the single-scene
// wavefront (wf_shade.cu) and the batched multi-scene pipeline (wf_batch.cu),
// so both perform the same operations in the same order as the CPU oracle
// (oracle/orc_impl.h); every translation unit is compiled without fused
// multiply-add.
#pragma once
#include "wf_kernels.h"

namespace wf {

// Slot allocation for a warp: one atomicAdd per warp on the queue tail (the
// reference issues one InterlockedAdd per surviving ray, shade.hlsl:164).
__device__ __forceinline__ uint32_t warp_append(uint32_t* tail, bool want) {
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    if (mask == 0u) return 0u;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(tail, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

// make_primary_ray (common.hlsl:182-195).
template <class Cam>
__device__ __forceinline__ void primary_ray(const Cam& W, uint32_t px, uint32_t py, V3& o, V3& d) {
    float uvx = ((float)px + 0.5f) / W.dim_x;
    float uvy = ((float)py + 0.5f) / W.dim_y;
    uvy = 1.0f - uvy;
    float cx = 2.0f * uvx - 1.0f, cy = 2.0f * uvy - 1.0f;
    V3 pv = xform(mk(cx, cy, 1.0f), 1.0f, W.clip_to_view[0], W.clip_to_view[1], W.clip_to_view[2],
                  W.clip_to_view[3]);
    V3 dv = normalize(pv);
    d = xform(dv, 0.0f, W.view_to_world[0], W.view_to_world[1], W.view_to_world[2], W.view_to_world[3]);
    o = xform(mk(0.0f, 0.0f, 0.0f), 1.0f, W.view_to_world[0], W.view_to_world[1], W.view_to_world[2],
              W.view_to_world[3]);
}

// create_orthonormal_basis (sample.hlsl:13-27).
__device__ __forceinline__ void basis(V3 n, V3& tg, V3& bt) {
    if (fabsf(n.x) > fabsf(n.z)) tg = normalize(mk(-n.y, n.x, 0.0f));
    else tg = normalize(mk(0.0f, -n.z, n.y));
    bt = cross(n, tg);
}
__device__ __forceinline__ V3 to_world(V3 v, V3 tg, V3 n, V3 bt) {
    return mk(v.x * tg.x + v.y * n.x + v.z * bt.x, v.x * tg.y + v.y * n.y + v.z * bt.y,
              v.x * tg.z + v.y * n.z + v.z * bt.z);
}
__device__ __forceinline__ V3 schlick(V3 f0, float c) {
    float m = 1.0f - c;
    float m2 = m * m;
    float m5 = (m2 * m2) * m;
    return mk(f0.x + (1.0f - f0.x) * m5, f0.y + (1.0f - f0.y) * m5, f0.z + (1.0f - f0.z) * m5);
}
__device__ __forceinline__ float g1(float x, float a2) { return (2.0f * x) / (x + sqrtf(a2 + (1.0f - a2) * (x * x))); }
__device__ __forceinline__ float ggx_d(float noh, float a2) {
    float q = (noh * noh) * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * (q * q));
}
__device__ __forceinline__ float offset_eps(V3 p) {
    return 1e-5f * (1.0f + fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
}

constexpr float kMetalDeltaAlpha = 1e-4f;
constexpr float kShadowTmaxScale = 0.999f;

__device__ __forceinline__ uint32_t pick_light(const LightTri* L, uint32_t count, float total, float r) {
    float x = r * total;
    uint32_t lo = 0, hi = count - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (x < L[mid].e1.w) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// Everything one shading event needs (one queue entry).
struct ShadeIn {
    V3 rd;             // ray direction
    float4 tuvp;       // hit {t, bary u, bary v, primitive}
    uint32_t inst;     // instance index into ShadeRefs.sinst, kInvalid for a miss
    V3 T;              // throughput
    float last_pdf;    // pdf of the BSDF sample that produced the ray
    uint32_t flags;    // path flags
    uint32_t pixel, sample, depth;   // keys of the path's random numbers
    V3 Lb, Lb_lo;      // adjoint replay only: the path's radiance before this event (and its rounding errors)
};

// Per-wave (or per-scene) constants of shading.
struct ShadeCtl {
    uint32_t frame_seed, max_bounces, nee, rr_start, cosine;
    float env_strength, env0, env1, env2;
    const LightTri* lights;
    uint32_t light_count;
    float light_total;
    TexRef env_tex;         // equirect environment (texels null: constant env0..2)
    uint32_t view_mode;     // RENDER_VIEW_MODE_* (0 = path tracing)
    float far_plane;        // view_t.far_plane, for the depth view
};

__device__ __forceinline__ V3 abs3(V3 a) { return mk(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }

// Material texture of a slot (id 0: the slot's default texture).
__device__ __forceinline__ float4 mat_tex(const ShadeRefs& SH, uint32_t id, uint32_t slot, float u, float v) {
    if (id == 0u || !in_bounds(id, SH.texture_count + 1ull, SH.status)) return tex_default(slot);
    return tex_bilinear(SH.textures[id], u, v);
}

struct ShadeOut {
    V3 add;            // radiance this event adds to the path
    bool has_add;
    bool enqueue;      // continue the path with (org, dir), throughput T, pdf, flags
    V3 org, dir, T;
    float pdf;
    uint32_t flags;
    bool shadow;       // a next-event shadow ray (spos, sdir, stmax) carrying contrib
    V3 spos, sdir, contrib;
    float stmax;
    uint32_t light_inst;   // the shadow ray's emitter instance (the adjoint's key)
    uint32_t em_key;   // adjoint: emitter reached (kInvalid if none) and its gradient
    float em_val;
};

// One shading event: shade.hlsl:42-174 (miss -> environment, emission ->
// terminate, Lambert bounce) plus GGX metal, smooth dielectric, next-event
// estimation with power-heuristic MIS, and Russian roulette.  The same
// operations, in the same order, as the oracle (oracle/orc_impl.h path()).
// adj_path / adj_pixel index the adjoint buffers when A is active.
__device__ __forceinline__ void shade_one(const ShadeRefs& SH, const ShadeCtl& K, const ShadeIn& in,
                                          const AdjointRefs& A, uint32_t adj_path, uint32_t adj_pixel,
                                          ShadeOut& o) {
    o.has_add = false; o.enqueue = false; o.shadow = false; o.em_key = kInvalid; o.em_val = 0.0f;
    V3 T = in.T;
    const V3 rd = in.rd;
    uint32_t flags = in.flags;
    if (in.inst == kInvalid) {
        if (K.view_mode != 0u) {
            // debug views of a miss (shade.hlsl:140-153): the hit record's
            // ids, barycentrics and t; views of the surface read zero (the
            // reference loads the surface of instance UINT_MAX out of bounds)
            const uint32_t vm = K.view_mode;
            V3 val = mk(0.0f, 0.0f, 0.0f);
            if (vm == 1u) val = int_to_color(kInvalid);
            else if (vm == 2u) val = int_to_color(__float_as_uint(in.tuvp.w));
            else if (vm == 3u) val = mk(in.tuvp.y, in.tuvp.z, 0.0f);
            else if (vm == 11u) { const float q = in.tuvp.x / K.far_plane; val = mk(q, q, q); }
            o.add = val;
            o.has_add = true;
            return;
        }
        // miss: energy += throughput * strength * env (shade.hlsl:60-65)
        const V3 env = K.env_tex.texels ? env_texel(K.env_tex, rd) : mk(K.env0, K.env1, K.env2);
        o.add = mk((T.x * K.env_strength) * env.x, (T.y * K.env_strength) * env.y, (T.z * K.env_strength) * env.z);
        o.has_add = true;
        return;
    }
    const uint32_t inst = in.inst;
    if (!in_bounds(inst, SH.inst_count, SH.status)) return;   // checked builds: the path ends
    const float4* ip = SH.sinst + (size_t)kInstRows * inst;
    const float4 c0 = ip[0], c1 = ip[1], c2 = ip[2], c3 = ip[3], mb = ip[4], me = ip[5], tx = ip[6];
    const uint32_t mesh = __float_as_uint(c0.w);
    const uint32_t prim = __float_as_uint(in.tuvp.w);
    if (!in_bounds(mesh, SH.mesh_count, SH.status) || !in_bounds(prim, SH.blas[mesh].tri_count, SH.status)) return;
    const float4* tp = SH.stri[mesh] + 6ull * prim;
    const V3 p0 = xyz(tp[0]), p1 = xyz(tp[1]), p2 = xyz(tp[2]);
    const V3 n0 = xyz(tp[3]), n1 = xyz(tp[4]), n2 = xyz(tp[5]);
    const float hu = in.tuvp.y, hv = in.tuvp.z;
    // get_hit_surface (common.hlsl:228-245)
    const V3 pl = add(add(p0, scl(sub(p1, p0), hu)), scl(sub(p2, p0), hv));
    const V3 pos = xform(pl, 1.0f, c0, c1, c2, c3);
    const V3 nl = add(add(n0, scl(sub(n1, n0), hu)), scl(sub(n2, n0), hv));
    V3 N = normalize(xform(nl, 0.0f, c0, c1, c2, c3));
    // sample_material (material.hlsl:15-39): factors times textures at the
    // interpolated uv (default textures when a slot has none)
    const uint32_t t_base = __float_as_uint(tx.x), t_nrm = __float_as_uint(tx.y);
    const uint32_t t_mr = __float_as_uint(tx.z), t_em = __float_as_uint(tx.w);
    float tu = 0.0f, tv = 0.0f;
    if ((t_base | t_nrm | t_mr | t_em) != 0u || K.view_mode == 5u) {
        tu = (tp[0].w + hu * (tp[2].w - tp[0].w)) + hv * (tp[4].w - tp[0].w);
        tv = (tp[1].w + hu * (tp[3].w - tp[1].w)) + hv * (tp[5].w - tp[1].w);
    }
    const float4 tbase = mat_tex(SH, t_base, TEX_BASE, tu, tv);
    const float4 mr = mat_tex(SH, t_mr, TEX_METAL_ROUGH, tu, tv);
    const float4 et = mat_tex(SH, t_em, TEX_EMISSIVE, tu, tv);
    V3 base_c = mk(mb.x * tbase.x, mb.y * tbase.y, mb.z * tbase.z);
    uint32_t stri = 0;
    if (SH.tri_albedo) {
        stri = SH.inst_tri_offset[inst] + prim;
        if (!in_bounds(stri, SH.albedo_count, SH.status)) return;
        base_c = xyz(SH.tri_albedo[stri]);
    }
    const V3 le = mk(me.x * et.x, me.y * et.y, me.z * et.z);
    if (K.view_mode != 0u) {
        // debug views (shade.hlsl:140-153), written instead of the radiance
        const uint32_t vm = K.view_mode;
        V3 val = mk(0.0f, 0.0f, 0.0f);
        if (vm == 1u) val = int_to_color(inst);
        else if (vm == 2u) val = int_to_color(prim);
        else if (vm == 3u) val = mk(hu, hv, 0.0f);
        else if (vm == 4u) val = abs3(nl);
        else if (vm == 5u) val = mk(tu, tv, 0.0f);
        else if (vm == 6u) val = base_c;
        else if (vm == 7u) val = abs3(xyz(mat_tex(SH, t_nrm, TEX_NORMAL, tu, tv)));
        else if (vm == 8u) val = mk(0.0f, mr.y, mr.z);
        else if (vm == 9u) val = le;
        else if (vm == 10u) val = abs3(N);
        else if (vm == 11u) { const float q = in.tuvp.x / K.far_plane; val = mk(q, q, q); }
        o.add = val;
        o.has_add = true;
        return;
    }
    if (le.x != 0.0f || le.y != 0.0f || le.z != 0.0f) {
        float w = 1.0f;
        if (K.nee && !(flags & kFlagSpecular) && K.light_count > 0) {
            V3 ng = normalize(xform(cross(sub(p1, p0), sub(p2, p0)), 0.0f, c0, c1, c2, c3));
            float cos_l = -dot(ng, rd);
            if (cos_l > 0.0f) {
                float d2 = (in.tuvp.x * in.tuvp.x) * dot(rd, rd);
                float pdf_l = d2 / (cos_l * K.light_total);
                // power heuristic in ratio form: 1 / (1 + (pdf_l / pdf_bsdf)^2)
                float q = pdf_l / in.last_pdf;
                w = (q == q) ? 1.0f / (1.0f + q * q) : 0.0f;
            }
        }
        o.add = mk((T.x * le.x) * w, (T.y * le.y) * w, (T.z * le.z) * w);
        o.has_add = true;
        if (A.g_emission && me.w != 0.0f) {
            // the contribution is linear in this emitter's strength
            const float4 g = A.dimage[adj_pixel];
            const float gl = (g.x * A.inv_spp) * o.add.x + (g.y * A.inv_spp) * o.add.y + (g.z * A.inv_spp) * o.add.z;
            o.em_key = inst;
            o.em_val = gl / me.w;
        }
        return;
    }
    const uint32_t depth = in.depth;
    uint32_t seed = path_seed(K.frame_seed, in.pixel, in.sample, depth);
    (void)rand_float(seed);  // r_path (shade.hlsl:81), drawn and unused
    const float r1 = rand_float(seed);
    const float r2 = rand_float(seed);
    const V3 V = neg(rd);
    V3 L = mk(0, 0, 0), wgt = mk(0, 0, 0);
    float pdf = 0.0f;
    bool delta = false, valid = true, toggle_inside = false;
    V3 org = pos;
    const float rough = c3.w * mr.y;   // roughness factor x texture green
    const float alpha = rough * rough;
    uint32_t bsdf = __float_as_uint(c1.w);
    if (bsdf == 1u && alpha < kMetalDeltaAlpha) bsdf = 3u;
    if ((flags & kFlagInside) && bsdf != 2u && dot(N, V) < 0.0f) N = neg(N);
    V3 tg, bt;
    basis(N, tg, bt);
    if (bsdf == 0u && A.g_albedo && SH.tri_albedo) {
        // everything the path gathers from here on (this vertex's shadow ray
        // and the rest of the path) is linear in this albedo: the final
        // radiance less what was gathered before (both sums carry their
        // rounding errors, so the difference keeps its precision when the
        // rest of the path adds little)
        const float4 Lf = A.L_final[adj_path], Lo = A.L_final_lo[adj_path], g = A.dimage[adj_pixel];
        const V3 Ld = mk((Lf.x - in.Lb.x) + (Lo.x - in.Lb_lo.x), (Lf.y - in.Lb.y) + (Lo.y - in.Lb_lo.y),
                         (Lf.z - in.Lb.z) + (Lo.z - in.Lb_lo.z));
        const uint32_t rep = (blockIdx.x ^ (threadIdx.x >> 5)) & (A.replicas - 1u);
        float* ga = reinterpret_cast<float*>(A.g_albedo + (size_t)rep * A.triangles + stri);
        if (base_c.x != 0.0f) atomicAdd(ga, ((g.x * A.inv_spp) * Ld.x) / base_c.x);
        if (base_c.y != 0.0f) atomicAdd(ga + 1, ((g.y * A.inv_spp) * Ld.y) / base_c.y);
        if (base_c.z != 0.0f) atomicAdd(ga + 2, ((g.z * A.inv_spp) * Ld.z) / base_c.z);
    }
    if (bsdf == 0u) {
        V3 loc;
        float sn, cs;
        if (K.cosine) {
            float st = sqrtf(r1);
            sincos_2pi(r2, sn, cs);
            loc = mk(st * cs, sqrtf(1.0f - r1), st * sn);
        } else {
            float st = sqrtf(1.0f - r1 * r1);
            sincos_2pi(r2, sn, cs);
            loc = mk(st * cs, r1, st * sn);
        }
        L = to_world(normalize(loc), tg, N, bt);
        const float nol = fmaxf(0.0f, dot(N, L));
        pdf = K.cosine ? nol * kInvPi : kInvTwoPi;
        const float ipdf = 1.0f / pdf;
        if (ipdf <= FLT_MAX) {
            wgt = mk((nol * (base_c.x * kInvPi)) * ipdf, (nol * (base_c.y * kInvPi)) * ipdf,
                     (nol * (base_c.z * kInvPi)) * ipdf);
        } else {
            // A cosine sample in the tangent plane (rand_float rounds to 1.0f, so
            // sqrt(1 - r1) = 0, or the dot product rounds to 0): the reference's
            // weight is 0 * inf = NaN (shade.hlsl:123-135) and its pixel turns
            // NaN.  The path ends here instead.
            valid = false;
        }
    } else if (bsdf == 1u) {
        const float a2 = alpha * alpha;
        const float cth = sqrtf((1.0f - r1) / (1.0f + (a2 - 1.0f) * r1));
        const float sth = sqrtf(fmaxf(0.0f, 1.0f - cth * cth));
        float sn, cs;
        sincos_2pi(r2, sn, cs);
        const V3 H = to_world(mk(sth * cs, cth, sth * sn), tg, N, bt);
        const float voh = dot(V, H);
        L = sub(scl(H, 2.0f * voh), V);
        const float nol = dot(N, L), nov = dot(N, V), noh = dot(N, H);
        if (nol <= 0.0f || nov <= 0.0f || voh <= 0.0f || noh <= 0.0f) {
            valid = false;
        } else {
            const V3 F = schlick(base_c, voh);
            const float G = g1(nol, a2) * g1(nov, a2);
            const float gw = (G * voh) / (nov * noh);
            wgt = scl(F, gw);
            pdf = (ggx_d(noh, a2) * noh) / (4.0f * voh);
        }
    } else if (bsdf == 3u) {
        const float nov = dot(N, V);
        delta = true;
        if (nov <= 0.0f) {
            valid = false;
        } else {
            L = sub(scl(N, 2.0f * nov), V);
            wgt = schlick(base_c, nov);
        }
    } else {
        float ci = dot(V, N);
        const bool entering = ci > 0.0f;
        const float ior = c2.w;
        const float n1 = entering ? 1.0f : ior, n2 = entering ? ior : 1.0f;
        const V3 nn = entering ? N : neg(N);
        ci = fabsf(ci);
        const float eta = n1 / n2;
        const float s2t = (eta * eta) * (1.0f - ci * ci);
        float F = 1.0f, ct = 0.0f;
        if (s2t < 1.0f) {
            ct = sqrtf(1.0f - s2t);
            const float rs = (n1 * ci - n2 * ct) / (n1 * ci + n2 * ct);
            const float rp = (n1 * ct - n2 * ci) / (n1 * ct + n2 * ci);
            F = 0.5f * (rs * rs + rp * rp);
        }
        if (r1 < F) {
            L = add(rd, scl(nn, 2.0f * ci));
        } else {
            L = normalize(add(scl(rd, eta), scl(nn, eta * ci - ct)));
            toggle_inside = true;
        }
        wgt = mk(1.0f, 1.0f, 1.0f);
        delta = true;
        org = add(pos, scl(L, offset_eps(pos)));
    }

    // next-event estimation: the shadow ray for the connect stage
    if (K.nee && !delta && depth < K.max_bounces && K.light_count > 0) {
        const float rl0 = rand_float(seed);
        const float rl1 = rand_float(seed);
        const float rl2 = rand_float(seed);
        const LightTri lt = K.lights[pick_light(K.lights, K.light_count, K.light_total, rl0)];
        const float su = sqrtf(rl1);
        const float b1 = su * (1.0f - rl2), b2 = su * rl2;
        const V3 y = add(add(xyz(lt.p0), scl(xyz(lt.e1), b1)), scl(xyz(lt.e2), b2));
        const V3 wv = sub(y, pos);
        const float dd2 = dot(wv, wv);
        const float dist = sqrtf(dd2);
        const V3 wl = scl(wv, 1.0f / dist);
        const float cos_l = -dot(xyz(lt.n), wl);
        const float cos_x = dot(N, wl);
        if (cos_l > 0.0f && cos_x > 0.0f) {
            const float pdf_l = dd2 / (cos_l * K.light_total);
            V3 f = mk(0, 0, 0);
            float pdf_b = 0.0f;
            bool ok = true;
            if (bsdf == 0u) {
                f = scl(base_c, kInvPi);
                pdf_b = K.cosine ? cos_x * kInvPi : kInvTwoPi;
            } else {
                const V3 H = normalize(add(V, wl));
                const float nov = dot(N, V), noh = dot(N, H), voh = dot(V, H);
                if (nov <= 0.0f || voh <= 0.0f) {
                    ok = false;
                } else {
                    const float a2 = alpha * alpha;
                    const float D = ggx_d(noh, a2);
                    const float G = g1(cos_x, a2) * g1(nov, a2);
                    const V3 F = schlick(base_c, voh);
                    f = scl(F, (D * G) / ((4.0f * cos_x) * nov));
                    pdf_b = (D * noh) / (4.0f * voh);
                    if (!(D <= FLT_MAX)) ok = false;
                }
            }
            if (ok) {
                const float q = pdf_b / pdf_l;
                const float w = (q == q) ? 1.0f / (1.0f + q * q) : 0.0f;
                const float sc = (cos_x * w) / pdf_l;
                V3 ltle = xyz(lt.le);
                const uint32_t lt_tex = __float_as_uint(lt.le.w);
                if (lt_tex != 0u && in_bounds(lt_tex, SH.texture_count + 1ull, SH.status)) {
                    // textured emitter: its emission texture at the sampled point
                    const float lu = (lt.uv01.x + b1 * (lt.uv01.z - lt.uv01.x)) + b2 * (lt.uv2.x - lt.uv01.x);
                    const float lv = (lt.uv01.y + b1 * (lt.uv01.w - lt.uv01.y)) + b2 * (lt.uv2.y - lt.uv01.y);
                    const float4 t = tex_bilinear(SH.textures[lt_tex], lu, lv);
                    ltle = mk(ltle.x * t.x, ltle.y * t.y, ltle.z * t.z);
                }
                o.contrib = mk(((T.x * f.x) * sc) * ltle.x, ((T.y * f.y) * sc) * ltle.y, ((T.z * f.z) * sc) * ltle.z);
                o.spos = pos;
                o.sdir = wl;
                o.stmax = dist * kShadowTmaxScale;
                o.light_inst = __float_as_uint(lt.n.w);
                o.shadow = true;
            }
        }
    }
    if (valid) {
        T = mul(T, wgt);
        if (depth < K.max_bounces) {
            bool survive = true;
            if (depth >= K.rr_start) {
                const float rr = rand_float(seed);
                const float q = fminf(fmaxf(fmaxf(T.x, T.y), T.z), 1.0f);
                if (rr >= q) survive = false;
                else T = mk(T.x / q, T.y / q, T.z / q);
            }
            if (survive) {
                if (toggle_inside) flags ^= kFlagInside;
                flags = delta ? (flags | kFlagSpecular) : (flags & ~kFlagSpecular);
                o.flags = flags;
                o.pdf = pdf;
                o.org = org;
                o.dir = L;
                o.T = T;
                o.enqueue = true;
            }
        }
    }
}

// Warp-aggregated atomic add of v to g[key] (one atomic per distinct key in the warp).
__device__ __forceinline__ void warp_add_by_key(float* g, uint32_t key, float v) {
    bool pending = key != kInvalid;
    for (;;) {
        const unsigned rem = __ballot_sync(0xffffffffu, pending);
        if (!rem) break;
        const int leader = __ffs(rem) - 1;
        const uint32_t k = __shfl_sync(0xffffffffu, key, leader);
        const bool mine = pending && key == k;
        float s = mine ? v : 0.0f;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if ((int)(threadIdx.x & 31) == leader) atomicAdd(&g[k], s);
        if (mine) pending = false;
    }
}

}  // namespace wf
