// wf_shade.cu — generate (clear_buffers.hlsl + generate.hlsl), shade
// (shade.hlsl:42-174 plus the added metal / dielectric / next-event /
// Russian-roulette steps) and post-process (post_process.hlsl:25-72).
//
// The per-path arithmetic is the CPU oracle's (oracle/orc_impl.h) operation
// for operation; both are compiled without fused multiply-add.
#include "wf_kernels.h"

namespace wf {

namespace {

constexpr int kBlock = 256;

unsigned grid_for(uint32_t n) {
    unsigned blocks = (n + kBlock - 1) / kBlock;
    unsigned cap = (unsigned)sm_count() * 8u;
    if (blocks > cap) blocks = cap;
    return blocks ? blocks : 1u;
}

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
__device__ __forceinline__ void primary_ray(const WaveParams& W, uint32_t px, uint32_t py, V3& o, V3& d) {
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

__global__ void __launch_bounds__(kBlock) k_generate(RenderBuffers B, WaveParams W) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < W.npaths; p += stride) {
        const uint32_t pixel = W.pix0 + p % W.np;
        V3 o, d;
        primary_ray(W, pixel % W.width, pixel / W.width, o, d);
        B.q_o[0][p] = make_float4(o.x, o.y, o.z, __uint_as_float(0u));
        B.q_d[0][p] = make_float4(d.x, d.y, d.z, FLT_MAX);
        B.q_path[0][p] = p;
        B.ps_T[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        B.ps_flags[p] = kFlagSpecular;
        B.ps_L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) B.counts[0] = W.npaths;
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

__global__ void __launch_bounds__(kBlock) k_shade(ShadeRefs SH, RenderBuffers B, WaveParams W, uint32_t depth,
                                                  AdjointRefs A) {
    const uint32_t n = B.counts[depth];
    const int cur = depth & 1, nxt = cur ^ 1;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool enqueue = false, shadow = false;
        uint32_t path = 0, pixel = 0, nflags = 0;
        V3 T = mk(0, 0, 0), norg = mk(0, 0, 0), ndir = mk(0, 0, 0), sdir = mk(0, 0, 0), contrib = mk(0, 0, 0);
        float npdf = 0.0f, stmax = 0.0f;
        V3 spos = mk(0, 0, 0);
        uint32_t em_key = kInvalid;   // adjoint: emitter instance reached by this path
        float em_val = 0.0f;
        if (i < n) {
            const float4 d4 = B.q_d[cur][i];
            path = B.q_path[cur][i];
            pixel = W.pix0 + path % W.np;
            const uint32_t sample = W.s0 + path / W.np;
            const float4 tuvp = B.h_tuvp[i];
            const uint32_t inst = B.h_inst[i];
            const float4 T4 = B.ps_T[path];
            uint32_t flags = B.ps_flags[path];
            T = xyz(T4);
            const float last_pdf = T4.w;
            const V3 rd = xyz(d4);
            if (inst == kInvalid) {
                // miss: energy += throughput * strength * env (shade.hlsl:60-65)
                float4 acc = B.ps_L[path];
                acc.x = acc.x + (T.x * W.env_strength) * W.env[0];
                acc.y = acc.y + (T.y * W.env_strength) * W.env[1];
                acc.z = acc.z + (T.z * W.env_strength) * W.env[2];
                B.ps_L[path] = acc;
            } else {
                const float4* ip = SH.sinst + 6ull * inst;
                const float4 c0 = ip[0], c1 = ip[1], c2 = ip[2], c3 = ip[3], mb = ip[4], me = ip[5];
                const uint32_t mesh = __float_as_uint(c0.w);
                const uint32_t prim = __float_as_uint(tuvp.w);
                const float4* tp = SH.stri[mesh] + 6ull * prim;
                const V3 p0 = xyz(tp[0]), p1 = xyz(tp[1]), p2 = xyz(tp[2]);
                const V3 n0 = xyz(tp[3]), n1 = xyz(tp[4]), n2 = xyz(tp[5]);
                const float hu = tuvp.y, hv = tuvp.z;
                // get_hit_surface (common.hlsl:228-245)
                const V3 pl = add(add(p0, scl(sub(p1, p0), hu)), scl(sub(p2, p0), hv));
                const V3 pos = xform(pl, 1.0f, c0, c1, c2, c3);
                const V3 nl = add(add(n0, scl(sub(n1, n0), hu)), scl(sub(n2, n0), hv));
                V3 N = normalize(xform(nl, 0.0f, c0, c1, c2, c3));
                V3 base_c = mk(mb.x * 1.0f, mb.y * 1.0f, mb.z * 1.0f);
                uint32_t stri = 0;
                if (SH.tri_albedo) {
                    stri = SH.inst_tri_offset[inst] + prim;
                    base_c = xyz(SH.tri_albedo[stri]);
                }
                const V3 le = mk(me.x * 1.0f, me.y * 1.0f, me.z * 1.0f);
                if (le.x != 0.0f || le.y != 0.0f || le.z != 0.0f) {
                    float w = 1.0f;
                    if (W.nee && !(flags & kFlagSpecular) && SH.light_count > 0) {
                        V3 ng = normalize(xform(cross(sub(p1, p0), sub(p2, p0)), 0.0f, c0, c1, c2, c3));
                        float cos_l = -dot(ng, rd);
                        if (cos_l > 0.0f) {
                            float d2 = (tuvp.x * tuvp.x) * dot(rd, rd);
                            float pdf_l = d2 / (cos_l * SH.light_total);
                            // power heuristic in ratio form: 1 / (1 + (pdf_l / pdf_bsdf)^2)
                            float q = pdf_l / last_pdf;
                            w = (q == q) ? 1.0f / (1.0f + q * q) : 0.0f;
                        }
                    }
                    float4 acc = B.ps_L[path];
                    acc.x = acc.x + (T.x * le.x) * w;
                    acc.y = acc.y + (T.y * le.y) * w;
                    acc.z = acc.z + (T.z * le.z) * w;
                    B.ps_L[path] = acc;
                    if (A.g_emission && me.w != 0.0f) {
                        const float4 L = A.L_final[path], g = A.dimage[pixel];
                        const float gl = (g.x * A.inv_spp) * L.x + (g.y * A.inv_spp) * L.y + (g.z * A.inv_spp) * L.z;
                        em_key = inst;
                        em_val = gl / me.w;
                    }
                } else {
                    uint32_t seed = path_seed(W.frame_seed, pixel, sample, depth);
                    (void)rand_float(seed);  // r_path (shade.hlsl:81), drawn and unused
                    const float r1 = rand_float(seed);
                    const float r2 = rand_float(seed);
                    const V3 V = neg(rd);
                    V3 L = mk(0, 0, 0), wgt = mk(0, 0, 0);
                    float pdf = 0.0f;
                    bool delta = false, valid = true, toggle_inside = false;
                    V3 org = pos;
                    const float alpha = c3.w * c3.w;
                    uint32_t bsdf = __float_as_uint(c1.w);
                    if (bsdf == 1u && alpha < kMetalDeltaAlpha) bsdf = 3u;
                    if ((flags & kFlagInside) && bsdf != 2u && dot(N, V) < 0.0f) N = neg(N);
                    V3 tg, bt;
                    basis(N, tg, bt);
                    if (bsdf == 0u && A.g_albedo && SH.tri_albedo) {
                        const float4 L = A.L_final[path], g = A.dimage[pixel];
                        const uint32_t rep = (blockIdx.x ^ (threadIdx.x >> 5)) & (A.replicas - 1u);
                        float* ga = reinterpret_cast<float*>(A.g_albedo + (size_t)rep * A.triangles + stri);
                        if (base_c.x != 0.0f) atomicAdd(ga, ((g.x * A.inv_spp) * L.x) / base_c.x);
                        if (base_c.y != 0.0f) atomicAdd(ga + 1, ((g.y * A.inv_spp) * L.y) / base_c.y);
                        if (base_c.z != 0.0f) atomicAdd(ga + 2, ((g.z * A.inv_spp) * L.z) / base_c.z);
                    }
                    if (bsdf == 0u) {
                        V3 loc;
                        float sn, cs;
                        if (W.cosine) {
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
                        pdf = W.cosine ? nol * kInvPi : kInvTwoPi;
                        const float ipdf = 1.0f / pdf;
                        wgt = mk((nol * (base_c.x * kInvPi)) * ipdf, (nol * (base_c.y * kInvPi)) * ipdf,
                                 (nol * (base_c.z * kInvPi)) * ipdf);
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
                    if (W.nee && !delta && depth < W.max_bounces && SH.light_count > 0) {
                        const float rl0 = rand_float(seed);
                        const float rl1 = rand_float(seed);
                        const float rl2 = rand_float(seed);
                        const LightTri lt = SH.lights[pick_light(SH.lights, SH.light_count, SH.light_total, rl0)];
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
                            const float pdf_l = dd2 / (cos_l * SH.light_total);
                            V3 f = mk(0, 0, 0);
                            float pdf_b = 0.0f;
                            bool ok = true;
                            if (bsdf == 0u) {
                                f = scl(base_c, kInvPi);
                                pdf_b = W.cosine ? cos_x * kInvPi : kInvTwoPi;
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
                                const V3 ltle = xyz(lt.le);
                                contrib = mk(((T.x * f.x) * sc) * ltle.x, ((T.y * f.y) * sc) * ltle.y,
                                             ((T.z * f.z) * sc) * ltle.z);
                                spos = pos;
                                sdir = wl;
                                stmax = dist * kShadowTmaxScale;
                                shadow = true;
                            }
                        }
                    }
                    if (valid) {
                        T = mul(T, wgt);
                        if (depth < W.max_bounces) {
                            bool survive = true;
                            if (depth >= W.rr_start) {
                                const float rr = rand_float(seed);
                                const float q = fminf(fmaxf(fmaxf(T.x, T.y), T.z), 1.0f);
                                if (rr >= q) survive = false;
                                else T = mk(T.x / q, T.y / q, T.z / q);
                            }
                            if (survive) {
                                if (toggle_inside) flags ^= kFlagInside;
                                flags = delta ? (flags | kFlagSpecular) : (flags & ~kFlagSpecular);
                                nflags = flags;
                                npdf = pdf;
                                norg = org;
                                ndir = L;
                                enqueue = true;
                            }
                        }
                    }
                }
            }
        }
        if (A.g_emission) {
            // one atomic per distinct emitter in the warp (usually one)
            bool pending = em_key != kInvalid;
            for (;;) {
                const unsigned rem = __ballot_sync(0xffffffffu, pending);
                if (!rem) break;
                const int leader = __ffs(rem) - 1;
                const uint32_t k = __shfl_sync(0xffffffffu, em_key, leader);
                const bool mine = pending && em_key == k;
                float v = mine ? em_val : 0.0f;
                for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
                if ((int)(threadIdx.x & 31) == leader) atomicAdd(&A.g_emission[k], v);
                if (mine) pending = false;
            }
        }
        const uint32_t slot = warp_append(&B.counts[depth + 1], enqueue);
        if (enqueue) {
            B.q_o[nxt][slot] = make_float4(norg.x, norg.y, norg.z, __uint_as_float(nflags & kFlagInside));
            B.q_d[nxt][slot] = make_float4(ndir.x, ndir.y, ndir.z, FLT_MAX);
            B.q_path[nxt][slot] = path;
            B.ps_T[path] = make_float4(T.x, T.y, T.z, npdf);
            B.ps_flags[path] = nflags;
        }
        const uint32_t sslot = warp_append(&B.counts[kMaxDepth + depth], shadow);
        if (shadow) {
            B.s_o[sslot] = make_float4(spos.x, spos.y, spos.z, stmax);
            B.s_d[sslot] = make_float4(sdir.x, sdir.y, sdir.z, __uint_as_float(path));
            B.s_c[sslot] = make_float4(contrib.x, contrib.y, contrib.z, 0.0f);
        }
    }
}

// post_process.hlsl:25-72 with accumulate on: average, NaN/Inf -> magenta,
// Reinhard, linear -> sRGB, RGBA8.
__device__ __forceinline__ float srgb(float c) {
    float x = fminf(fmaxf(c, 0.0f), 1.0f);
    return (x <= 0.0031308f) ? x * 12.92f : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ unsigned char unorm8(float c) {
    return (unsigned char)(fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f + 0.5f);
}
__device__ __forceinline__ bool bad(float x) { return isnan(x) || isinf(x); }

__global__ void k_post(const float4* __restrict__ accum, uint32_t npix, uint32_t tonemap, uchar4* __restrict__ out) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += stride) {
        float4 a = accum[i];
        float inv = a.w > 0.0f ? 1.0f / a.w : 0.0f;
        float r = a.x * inv, g = a.y * inv, b = a.z * inv;
        if (bad(r) || bad(g) || bad(b)) { r = 1.0f; g = 0.0f; b = 1.0f; }
        if (tonemap) { r = r / (1.0f + r); g = g / (1.0f + g); b = b / (1.0f + b); }
        out[i] = make_uchar4(unorm8(srgb(r)), unorm8(srgb(g)), unorm8(srgb(b)), 255);
    }
}

__global__ void k_wave_resolve(RenderBuffers B, WaveParams W) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < W.np; p += stride) {
        float4 acc = B.accum[W.pix0 + p];
        for (uint32_t s = 0; s < W.nsamples; ++s) {
            const float4 L = B.ps_L[(size_t)s * W.np + p];
            acc.x = acc.x + L.x;
            acc.y = acc.y + L.y;
            acc.z = acc.z + L.z;
            acc.w = acc.w + 1.0f;
        }
        B.accum[W.pix0 + p] = acc;
    }
}

__global__ void k_resolve(const float4* __restrict__ accum, uint32_t npix, float4* __restrict__ out) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += stride) {
        float4 a = accum[i];
        out[i] = a.w > 0.0f ? make_float4(a.x / a.w, a.y / a.w, a.z / a.w, a.w) : make_float4(0, 0, 0, 0);
    }
}

__global__ void k_reduce_replicas(float4* g, uint32_t triangles, uint32_t replicas) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < triangles; t += stride) {
        float4 a = g[t];
        for (uint32_t r = 1; r < replicas; ++r) {
            const float4 b = g[(size_t)r * triangles + t];
            a.x += b.x; a.y += b.y; a.z += b.z;
        }
        g[t] = a;
    }
}

}  // namespace

cudaError_t launch_generate(const RenderBuffers& B, const WaveParams& W, cudaStream_t stream) {
    k_generate<<<grid_for(W.npaths), kBlock, 0, stream>>>(B, W);
    return cudaGetLastError();
}

cudaError_t launch_shade(const ShadeRefs& SH, const RenderBuffers& B, const WaveParams& W, uint32_t depth,
                         uint32_t max_rays, const AdjointRefs& A, cudaStream_t stream) {
    k_shade<<<grid_for(max_rays), kBlock, 0, stream>>>(SH, B, W, depth, A);
    return cudaGetLastError();
}

cudaError_t launch_reduce_replicas(float4* g, uint32_t triangles, uint32_t replicas, cudaStream_t stream) {
    k_reduce_replicas<<<grid_for(triangles), kBlock, 0, stream>>>(g, triangles, replicas);
    return cudaGetLastError();
}

cudaError_t launch_wave_resolve(const RenderBuffers& B, const WaveParams& W, cudaStream_t stream) {
    k_wave_resolve<<<grid_for(W.np), kBlock, 0, stream>>>(B, W);
    return cudaGetLastError();
}

cudaError_t launch_post(const float4* accum, uint32_t npix, uint32_t tonemap, uchar4* out, cudaStream_t stream) {
    k_post<<<grid_for(npix), kBlock, 0, stream>>>(accum, npix, tonemap, out);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const float4* accum, uint32_t npix, float4* out, cudaStream_t stream) {
    k_resolve<<<grid_for(npix), kBlock, 0, stream>>>(accum, npix, out);
    return cudaGetLastError();
}

}  // namespace wf
