/*
 * orc_impl.h — oracle traversal and shading, written once for a real type R
 * and included twice by orc_trace.c (R = float, suffix _f32; R = double,
 * suffix _f64).  TEST INFRASTRUCTURE ONLY (see wf_oracle.h).
 *
 * Required macros: R, FN(name), K(literal) (appends f for float), SQRT, FABS,
 * FMIN, FMAX, SINCOS2PI(r, &s, &c), MAXT (the miss sentinel, FLT_MAX).
 *
 * Every expression below is evaluated in the order written, with no fused
 * multiply-add.  The FP32 instance is the GPU library's contract: the CUDA
 * kernels (compiled with --fmad=false) perform the same operations in the
 * same order and must agree bit for bit.
 */

typedef struct { R x, y, z; } FN(v3);

static inline FN(v3) FN(mk)(R x, R y, R z) { FN(v3) r; r.x = x; r.y = y; r.z = z; return r; }
static inline FN(v3) FN(ld)(const float* p) { return FN(mk)((R)p[0], (R)p[1], (R)p[2]); }
static inline FN(v3) FN(add)(FN(v3) a, FN(v3) b) { return FN(mk)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline FN(v3) FN(sub)(FN(v3) a, FN(v3) b) { return FN(mk)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline FN(v3) FN(mul)(FN(v3) a, FN(v3) b) { return FN(mk)(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline FN(v3) FN(scl)(FN(v3) a, R s) { return FN(mk)(a.x * s, a.y * s, a.z * s); }
static inline FN(v3) FN(neg)(FN(v3) a) { return FN(mk)(-a.x, -a.y, -a.z); }
/* dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z */
static inline R FN(dot)(FN(v3) a, FN(v3) b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline FN(v3) FN(cross)(FN(v3) a, FN(v3) b) {
    return FN(mk)(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* normalize(v) = v * (1 / sqrt(dot(v, v))) */
static inline FN(v3) FN(normalize)(FN(v3) v) { R s = K(1.0) / SQRT(FN(dot)(v, v)); return FN(scl)(v, s); }

/* HLSL mul(float4(v, w), M) with row-major packing == glm M * v:
 * out_j = ((v.x*m[j] + v.y*m[4+j]) + v.z*m[8+j]) + w*m[12+j]. */
static inline FN(v3) FN(xform)(FN(v3) v, R w, const float* m) {
    R o[3];
    for (int j = 0; j < 3; ++j)
        o[j] = v.x * (R)m[j] + v.y * (R)m[4 + j] + v.z * (R)m[8 + j] + w * (R)m[12 + j];
    return FN(mk)(o[0], o[1], o[2]);
}

/* intersect_ray_aabb (intersect.hlsl:53-76); min/max are IEEE minNum/maxNum
 * like HLSL's. */
static inline R FN(slab_cmp)(const float* bmn, const float* bmx, FN(v3) o, FN(v3) inv, R t, int tie) {
    R tx1 = ((R)bmn[0] - o.x) * inv.x, tx2 = ((R)bmx[0] - o.x) * inv.x;
    R tmin = FMIN(tx1, tx2), tmax = FMAX(tx1, tx2);
    R ty1 = ((R)bmn[1] - o.y) * inv.y, ty2 = ((R)bmx[1] - o.y) * inv.y;
    tmin = FMAX(tmin, FMIN(ty1, ty2));
    tmax = FMIN(tmax, FMAX(ty1, ty2));
    R tz1 = ((R)bmn[2] - o.z) * inv.z, tz2 = ((R)bmx[2] - o.z) * inv.z;
    tmin = FMAX(tmin, FMIN(tz1, tz2));
    tmax = FMIN(tmax, FMAX(tz1, tz2));
    if (tmax >= tmin && (tie ? tmin <= t : tmin < t) && tmax > K(0.0)) return tmin;
    return MAXT;
}
static inline R FN(slab)(const float* bmn, const float* bmx, FN(v3) o, FN(v3) inv, R t) {
    return FN(slab_cmp)(bmn, bmx, o, inv, t, 0);
}

/* intersect_ray_triangle (intersect.hlsl:7-51), Moeller-Trumbore with the
 * back-face test det < 1e-8 (|det| < 1e-8 without culling). */
static inline int FN(tri_cmp)(FN(v3) v0, FN(v3) v1, FN(v3) v2, FN(v3) o, FN(v3) d, R* t_io, R* bu, R* bv,
                              int no_cull, int tie_wins) {
    FN(v3) e1 = FN(sub)(v1, v0), e2 = FN(sub)(v2, v0);
    FN(v3) pvec = FN(cross)(d, e2);
    R det = FN(dot)(e1, pvec);
    if (no_cull ? (FABS(det) < K(1e-8)) : (det < K(1e-8))) return 0;
    R inv_det = K(1.0) / det;
    FN(v3) tvec = FN(sub)(o, v0);
    R v = FN(dot)(tvec, pvec) * inv_det;
    if (v < K(0.0) || v > K(1.0)) return 0;
    FN(v3) qvec = FN(cross)(tvec, e1);
    R w = FN(dot)(d, qvec) * inv_det;
    if (w < K(0.0) || v + w > K(1.0)) return 0;
    R t = FN(dot)(e2, qvec) * inv_det;
    if (t < K(0.0) || t > *t_io || (t == *t_io && !tie_wins)) return 0;
    *t_io = t; *bu = v; *bv = w;
    return 1;
}
static inline int FN(tri)(FN(v3) v0, FN(v3) v1, FN(v3) v2, FN(v3) o, FN(v3) d, R* t_io, R* bu, R* bv,
                          int no_cull) {
    return FN(tri_cmp)(v0, v1, v2, o, d, t_io, bu, bv, no_cull, 0);
}

typedef struct {
    uint32_t inst, prim;
    R t, u, v;
} FN(hit);

#define ORC_STACK 64

/* trace_ray_bvh_local (accelstruct.hlsl:58-131).  Returns 1 on a hit, 0 on
 * none, -1 when the 64-entry stack overflowed.  With ORC_TIE_RULE (closest
 * hit only) a triangle at exactly the current t wins when its (instance,
 * primitive) is smaller than the current hit's, and boxes entered at exactly
 * the current t are visited: the result is then the smallest (t, instance,
 * primitive) whatever the visiting order (the order the reference's strict
 * "t < ray.t" makes matter only on exact ties). */
static int FN(trace_blas)(const uint8_t* blas, FN(v3) o, FN(v3) d, FN(v3) inv, R* t, FN(hit)* h,
                          uint32_t flags, orc_counters* c, uint32_t inst) {
    const int tie = (flags & ORC_TIE_RULE) && !(flags & ORC_ANY_HIT);
    bvh_header_t hd;
    memcpy(&hd, blas, sizeof(hd));
    const uint8_t* nodes = blas + hd.nodes_offset;
    const uint8_t* tris = blas + hd.triangles_offset;
    const uint8_t* idx = blas + hd.indices_offset;
    bvh_node_t node, stack[ORC_STACK];
    int sp = 0, has_hit = 0;
    memcpy(&node, nodes, 32);
    c->blas_node_loads++;
    for (;;) {
        if (node.prim_count > 0) {
            for (uint32_t i = node.left_first; i < node.left_first + node.prim_count; ++i) {
                uint32_t ti;
                bvh_triangle_t tr;
                memcpy(&ti, idx + 4ull * i, 4);
                memcpy(&tr, tris + 36ull * ti, 36);
                c->triangle_tests++;
                R bu, bv;
                int wins = 0;
                if (tie) {
                    /* the current hit: this instance once it has one here, else the outer one */
                    const uint32_t bi = has_hit ? inst : h->inst;
                    wins = inst < bi || (inst == bi && ti < h->prim);
                }
                if (FN(tri_cmp)(FN(ld)(tr.p0), FN(ld)(tr.p1), FN(ld)(tr.p2), o, d, t, &bu, &bv,
                                (flags & ORC_NO_CULL) != 0, wins)) {
                    h->prim = ti; h->u = bu; h->v = bv;
                    has_hit = 1;
                    if (flags & ORC_ANY_HIT) return 1;
                }
            }
            if (sp == 0) break;
            node = stack[--sp];
            continue;
        }
        bvh_node_t l, r;
        memcpy(&l, nodes + 32ull * node.left_first, 32);
        memcpy(&r, nodes + 32ull * (node.left_first + 1), 32);
        c->blas_node_loads += 2;
        R dl = FN(slab_cmp)(l.aabb_min, l.aabb_max, o, inv, *t, tie);
        R dr = FN(slab_cmp)(r.aabb_min, r.aabb_max, o, inv, *t, tie);
        if (dl > dr) { R td = dl; dl = dr; dr = td; bvh_node_t tn = l; l = r; r = tn; }
        if (dl == MAXT) {
            if (sp == 0) break;
            node = stack[--sp];
        } else {
            node = l;
            if (dr != MAXT) {
                if (sp == ORC_STACK) return -1;
                stack[sp++] = r;
            }
        }
    }
    return has_hit;
}

/* trace_ray_tlas (accelstruct.hlsl:151-218) with trace_ray_bvh_instance
 * (:133-149): the ray goes to object space through world_to_local without
 * renormalising, so t is shared by both spaces.  Returns -1 on overflow. */
static int FN(trace_one)(const orc_scene* s, FN(v3) o, FN(v3) d, R tmax, uint32_t flags, FN(hit)* h,
                         orc_counters* c) {
    h->inst = WF_INVALID_INDEX; h->prim = WF_INVALID_INDEX; h->t = MAXT; h->u = 0; h->v = 0;
    tlas_header_t th;
    memcpy(&th, s->tlas, sizeof(th));
    const uint8_t* nodes = s->tlas + th.nodes_offset;
    const uint8_t* insts = s->tlas + th.instances_offset;
    FN(v3) inv = FN(mk)(K(1.0) / d.x, K(1.0) / d.y, K(1.0) / d.z);
    R t = tmax;
    tlas_node_t node, stack[ORC_STACK];
    int sp = 0;
    memcpy(&node, nodes, 32);
    c->tlas_node_loads++;
    const int tie = (flags & ORC_TIE_RULE) && !(flags & ORC_ANY_HIT);
    if (s->inst_count == 0) return 0;
    if (FN(slab_cmp)(node.aabb_min, node.aabb_max, o, inv, t, tie) == MAXT) return 0;
    for (;;) {
        if (node.left_right == 0) {
            bvh_instance_t in;
            memcpy(&in, insts + 92ull * node.instance_idx, 92);
            c->instance_loads++;
            FN(v3) lo = FN(xform)(o, K(1.0), in.world_to_local);
            FN(v3) ld = FN(xform)(d, K(0.0), in.world_to_local);
            FN(v3) linv = FN(mk)(K(1.0) / ld.x, K(1.0) / ld.y, K(1.0) / ld.z);
            R lt = t;
            int r = FN(trace_blas)(s->meshes[in.bvh_index].blas, lo, ld, linv, &lt, h, flags, c, node.instance_idx);
            if (r < 0) {
                h->inst = WF_INVALID_INDEX; h->prim = WF_INVALID_INDEX; h->t = MAXT; h->u = 0; h->v = 0;
                return -1;
            }
            t = lt;
            if (r) {
                h->inst = node.instance_idx;
                h->t = t;
                if (flags & ORC_ANY_HIT) return 1;
            }
            if (sp == 0) break;
            node = stack[--sp];
            continue;
        }
        tlas_node_t l, r;
        memcpy(&l, nodes + 32ull * (node.left_right >> 16), 32);
        memcpy(&r, nodes + 32ull * (node.left_right & 0xFFFFu), 32);
        c->tlas_node_loads += 2;
        R dl = FN(slab_cmp)(l.aabb_min, l.aabb_max, o, inv, t, tie);
        R dr = FN(slab_cmp)(r.aabb_min, r.aabb_max, o, inv, t, tie);
        if (dl > dr) { R td = dl; dl = dr; dr = td; tlas_node_t tn = l; l = r; r = tn; }
        if (dl == MAXT) {
            if (sp == 0) break;
            node = stack[--sp];
        } else {
            node = l;
            if (dr != MAXT) {
                if (sp == ORC_STACK) {
                    h->inst = WF_INVALID_INDEX; h->prim = WF_INVALID_INDEX; h->t = MAXT; h->u = 0; h->v = 0;
                    return -1;
                }
                stack[sp++] = r;
            }
        }
    }
    return h->inst != WF_INVALID_INDEX;
}

/* ---------------------------------------------------------------------------
 * Textures (material.hlsl:15-39 sampling, shade.hlsl:36-40 environment)
 * ------------------------------------------------------------------------- */

/* Bilinear, wrap addressing, texel centres at (i + 0.5) / w; weights in R. */
static void FN(tex_sample)(const orc_texture* t, R u, R v, R out[4]) {
    R x = u * (R)t->w - K(0.5), y = v * (R)t->h - K(0.5);
    R x0 = FLOOR(x), y0 = FLOOR(y);
    R ax = x - x0, ay = y - y0;
    uint32_t i0 = wrap_texel((double)x0, t->w), i1 = wrap_texel((double)(x0 + K(1.0)), t->w);
    uint32_t j0 = wrap_texel((double)y0, t->h), j1 = wrap_texel((double)(y0 + K(1.0)), t->h);
    const float* a = t->texels + 4 * ((size_t)j0 * t->w + i0);
    const float* b = t->texels + 4 * ((size_t)j0 * t->w + i1);
    const float* c = t->texels + 4 * ((size_t)j1 * t->w + i0);
    const float* d = t->texels + 4 * ((size_t)j1 * t->w + i1);
    for (int k = 0; k < 4; ++k) {
        R top = (R)a[k] + ((R)b[k] - (R)a[k]) * ax;
        R bot = (R)c[k] + ((R)d[k] - (R)c[k]) * ax;
        out[k] = top + (bot - top) * ay;
    }
}

/* The texture of a material slot; id 0 = the reference's default texture
 * (renderer.cpp:244-272): white base colour / emission, normal
 * (127, 127, 255)/255, metallic-roughness RG8 (255, 255) = (1, 1, 0, 1). */
static void FN(mat_tex)(const orc_scene* s, uint32_t id, int slot, R u, R v, R out[4]) {
    if (id == 0) {
        out[0] = out[1] = out[2] = out[3] = K(1.0);
        if (slot == 1) { out[0] = K(127.0) / K(255.0); out[1] = K(127.0) / K(255.0); }
        if (slot == 2) out[2] = K(0.0);
        return;
    }
    FN(tex_sample)(&s->textures[id - 1], u, v, out);
}

/* sample_hdr_env: direction_to_equirect_uv (sample.hlsl:4-11, INV_ATAN =
 * (0.1591, 0.3183)) times the texture size, truncated; out of range = 0. */
static FN(v3) FN(env_texel)(const orc_texture* e, FN(v3) d) {
    R u = ATAN2(d.z, d.x) * K(0.1591) + K(0.5);
    R v = ASIN(-d.y) * K(0.3183) + K(0.5);
    R fx = u * (R)e->w, fy = v * (R)e->h;
    if (!(fx >= K(0.0) && fx < (R)e->w && fy >= K(0.0) && fy < (R)e->h)) return FN(mk)(0, 0, 0);
    const float* p = e->texels + 4 * ((size_t)(uint32_t)fy * e->w + (uint32_t)fx);
    return FN(mk)((R)p[0], (R)p[1], (R)p[2]);
}

/* int_to_color (common.hlsl:276-295). */
static FN(v3) FN(int_to_color)(uint32_t v) {
    uint32_t h = murmur_mix(v);
    R k = K(1.0) / K(255.0);
    return FN(mk)((R)(h & 255u) * k, (R)((h >> 8) & 255u) * k, (R)((h >> 16) & 255u) * k);
}

static inline FN(v3) FN(abs3)(FN(v3) a) { return FN(mk)(FABS(a.x), FABS(a.y), FABS(a.z)); }

/* ---------------------------------------------------------------------------
 * Shading
 * ------------------------------------------------------------------------- */

#define ORC_PI K(3.14159265)
#define ORC_INV_PI K(0.31830988)
#define ORC_INV_TWO_PI K(0.15915494)

/* create_orthonormal_basis (sample.hlsl:13-27): rows tangent, normal, bitangent. */
static inline void FN(basis)(FN(v3) n, FN(v3)* tg, FN(v3)* bt) {
    if (FABS(n.x) > FABS(n.z)) *tg = FN(normalize)(FN(mk)(-n.y, n.x, K(0.0)));
    else *tg = FN(normalize)(FN(mk)(K(0.0), -n.z, n.y));
    *bt = FN(cross)(n, *tg);
}
/* mul(v, float3x3(T, N, B)) = (v.x*T + v.y*N) + v.z*B per component. */
static inline FN(v3) FN(to_world)(FN(v3) v, FN(v3) tg, FN(v3) n, FN(v3) bt) {
    return FN(mk)(v.x * tg.x + v.y * n.x + v.z * bt.x,
                  v.x * tg.y + v.y * n.y + v.z * bt.y,
                  v.x * tg.z + v.y * n.z + v.z * bt.z);
}

/* cosine_weighted_hemisphere_sample / uniform_hemisphere_sample
 * (sample.hlsl:29-54): phi = 2 pi r2 (SINCOS2PI), the local direction
 * normalised, then mul(local, basis). */
static inline FN(v3) FN(hemisphere)(FN(v3) n, FN(v3) tg, FN(v3) bt, R r1, R r2, int cosine) {
    FN(v3) loc;
    R sn, cs;
    if (cosine) {
        R st_ = SQRT(r1);
        SINCOS2PI(r2, &sn, &cs);
        loc = FN(mk)(st_ * cs, SQRT(K(1.0) - r1), st_ * sn);
    } else {
        R st_ = SQRT(K(1.0) - r1 * r1);
        SINCOS2PI(r2, &sn, &cs);
        loc = FN(mk)(st_ * cs, r1, st_ * sn);
    }
    return FN(to_world)(FN(normalize)(loc), tg, n, bt);
}

typedef struct {
    FN(v3) p0, e1, e2, n, le;
    R area;
    R uv[6];                  /* vertex uv (u0, v0, u1, v1, u2, v2) */
    uint32_t tex;             /* emissive texture id (0 = none) */
    uint32_t inst;            /* the instance it belongs to (the adjoint's emitter key) */
    R strength;               /* that instance's emissive strength */
} FN(light);

typedef struct {
    FN(light)* tri;
    R* cdf;
    uint32_t count;
    R total;
} FN(lights);

/* Emitter table: every triangle of every instance whose emissive colour has a
 * non-zero component, in instance order then triangle order.  Vertices go to
 * world space with xform(p, 1, local_to_world); area = 0.5*|e1 x e2|; the CDF
 * is a running sum of areas in that order. */
static void FN(build_lights)(const orc_scene* s, FN(lights)* L) {
    uint32_t cnt = 0;
    for (uint32_t i = 0; i < s->inst_count; ++i) {
        const material_t* m = &s->inst[i].material;
        R le0 = (R)m->emissive_strength * (R)m->emissive_factor[0];
        R le1 = (R)m->emissive_strength * (R)m->emissive_factor[1];
        R le2 = (R)m->emissive_strength * (R)m->emissive_factor[2];
        if (le0 != K(0.0) || le1 != K(0.0) || le2 != K(0.0)) cnt += s->meshes[s->inst[i].mesh].tri_count;
    }
    L->count = cnt;
    L->total = K(0.0);
    L->tri = (FN(light)*)malloc(sizeof(FN(light)) * (cnt ? cnt : 1));
    L->cdf = (R*)malloc(sizeof(R) * (cnt ? cnt : 1));
    uint32_t k = 0;
    R run = K(0.0);
    for (uint32_t i = 0; i < s->inst_count; ++i) {
        const orc_instance* in = &s->inst[i];
        const material_t* m = &in->material;
        FN(v3) le = FN(mk)((R)m->emissive_strength * (R)m->emissive_factor[0],
                           (R)m->emissive_strength * (R)m->emissive_factor[1],
                           (R)m->emissive_strength * (R)m->emissive_factor[2]);
        if (!(le.x != K(0.0) || le.y != K(0.0) || le.z != K(0.0))) continue;
        const orc_mesh* me = &s->meshes[in->mesh];
        for (uint32_t t = 0; t < me->tri_count; ++t) {
            FN(v3) p0 = FN(xform)(FN(ld)(me->tris[t].v0.position), K(1.0), in->local_to_world);
            FN(v3) p1 = FN(xform)(FN(ld)(me->tris[t].v1.position), K(1.0), in->local_to_world);
            FN(v3) p2 = FN(xform)(FN(ld)(me->tris[t].v2.position), K(1.0), in->local_to_world);
            FN(light)* lt = &L->tri[k];
            lt->p0 = p0;
            lt->e1 = FN(sub)(p1, p0);
            lt->e2 = FN(sub)(p2, p0);
            FN(v3) c = FN(cross)(lt->e1, lt->e2);
            R len = SQRT(FN(dot)(c, c));
            lt->area = K(0.5) * len;
            lt->n = FN(scl)(c, K(1.0) / len);
            lt->le = le;
            lt->uv[0] = (R)me->tris[t].v0.uv[0]; lt->uv[1] = (R)me->tris[t].v0.uv[1];
            lt->uv[2] = (R)me->tris[t].v1.uv[0]; lt->uv[3] = (R)me->tris[t].v1.uv[1];
            lt->uv[4] = (R)me->tris[t].v2.uv[0]; lt->uv[5] = (R)me->tris[t].v2.uv[1];
            lt->tex = m->emissive_index;
            lt->inst = i;
            lt->strength = (R)m->emissive_strength;
            run = run + lt->area;
            L->cdf[k] = run;
            k++;
        }
    }
    L->total = run;
}

/* First entry whose running area exceeds r*total (the last entry if none). */
static uint32_t FN(pick_light)(const FN(lights)* L, R r) {
    R x = r * L->total;
    uint32_t lo = 0, hi = L->count - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (x < L->cdf[mid]) hi = mid; else lo = mid + 1;
    }
    return lo;
}

/* Schlick Fresnel per channel: F0 + (1 - F0) * (1 - c)^5, (m^2 * m^2) * m. */
static inline FN(v3) FN(schlick)(FN(v3) f0, R c) {
    R m = K(1.0) - c;
    R m2 = m * m;
    R m5 = (m2 * m2) * m;
    return FN(mk)(f0.x + (K(1.0) - f0.x) * m5, f0.y + (K(1.0) - f0.y) * m5, f0.z + (K(1.0) - f0.z) * m5);
}
/* Smith G1 for GGX: 2x / (x + sqrt(a2 + (1 - a2) * x^2)). */
static inline R FN(g1)(R x, R a2) { return (K(2.0) * x) / (x + SQRT(a2 + (K(1.0) - a2) * (x * x))); }
/* GGX D: a2 / (pi * q^2), q = NoH^2 * (a2 - 1) + 1. */
static inline R FN(ggx_d)(R noh, R a2) { R q = (noh * noh) * (a2 - K(1.0)) + K(1.0); return a2 / (ORC_PI * (q * q)); }

#define ORC_F_INSIDE 1u
#define ORC_F_SPECULAR 2u
#define ORC_METAL_DELTA_ALPHA K(1e-4)
#define ORC_SHADOW_TMAX_SCALE K(0.999)

static inline R FN(offset_eps)(FN(v3) p) {
    return K(1e-5) * (K(1.0) + FMAX(FABS(p.x), FMAX(FABS(p.y), FABS(p.z))));
}

typedef struct {
    FN(v3) L, wgt, org;     /* next direction, throughput factor, next origin */
    R pdf;                  /* solid-angle pdf of L (0 for delta lobes) */
    int delta, valid, toggle_inside;
} FN(scatter);

/* The shade stage's scattering step at a surface point with shading normal N
 * (basis tg, bt) for a ray arriving along rd: bsdf 0 = Lambert
 * (shade.hlsl:107-135: cosine-weighted or uniform hemisphere, weight
 * NoL * base/pi / pdf), 1 = GGX metal (alpha = roughness^2; half vector from
 * the GGX normal distribution, weight F * G1(L) G1(V) * VoH / (NoV * NoH),
 * Schlick F with F0 = base), 3 = mirror (metal with alpha < 1e-4: weight
 * Schlick F at NoV), 2 = smooth dielectric (exact Fresnel reflectance chooses
 * reflection or refraction, weight 1, origin offset along L). */
static FN(scatter) FN(sample_bsdf)(uint32_t bsdf, FN(v3) base, R alpha, R ior, FN(v3) N, FN(v3) tg, FN(v3) bt,
                                   FN(v3) rd, FN(v3) pos, R r1, R r2, int cosine) {
    FN(scatter) o;
    FN(v3) V = FN(neg)(rd);
    FN(v3) L = FN(mk)(0, 0, 0), wgt = FN(mk)(0, 0, 0);
    R pdf = K(0.0);
    int delta = 0, valid = 1, toggle_inside = 0;
    FN(v3) org = pos;
    if (bsdf == 0) {
        /* shade.hlsl:107-135 */
        L = FN(hemisphere)(N, tg, bt, r1, r2, cosine);
        R nol = FMAX(K(0.0), FN(dot)(N, L));
        pdf = cosine ? nol * ORC_INV_PI : ORC_INV_TWO_PI;
        R ip = K(1.0) / pdf;
        /* shade.hlsl:135 multiplies by 1 / pdf unguarded: a sample in the
         * tangent plane (r1 == 1, or NoL rounding to 0) gives 0 * inf = NaN
         * there.  Here the path ends (the GPU kernels do the same). */
        if (ip <= MAXT)
            wgt = FN(mk)((nol * (base.x * ORC_INV_PI)) * ip, (nol * (base.y * ORC_INV_PI)) * ip,
                         (nol * (base.z * ORC_INV_PI)) * ip);
        else
            valid = 0;
    } else if (bsdf == 1) {
        R a2 = alpha * alpha;
        R cth = SQRT((K(1.0) - r1) / (K(1.0) + (a2 - K(1.0)) * r1));
        R sth = SQRT(FMAX(K(0.0), K(1.0) - cth * cth));
        R sn, cs;
        SINCOS2PI(r2, &sn, &cs);
        FN(v3) H = FN(to_world)(FN(mk)(sth * cs, cth, sth * sn), tg, N, bt);
        R voh = FN(dot)(V, H);
        L = FN(sub)(FN(scl)(H, K(2.0) * voh), V);
        R nol = FN(dot)(N, L), nov = FN(dot)(N, V), noh = FN(dot)(N, H);
        if (nol <= K(0.0) || nov <= K(0.0) || voh <= K(0.0) || noh <= K(0.0)) {
            valid = 0;
        } else {
            FN(v3) F = FN(schlick)(base, voh);
            R G = FN(g1)(nol, a2) * FN(g1)(nov, a2);
            R gw = (G * voh) / (nov * noh);
            wgt = FN(scl)(F, gw);
            pdf = (FN(ggx_d)(noh, a2) * noh) / (K(4.0) * voh);
        }
    } else if (bsdf == 3) {
        R nov = FN(dot)(N, V);
        delta = 1;
        if (nov <= K(0.0)) valid = 0;
        else {
            L = FN(sub)(FN(scl)(N, K(2.0) * nov), V);
            wgt = FN(schlick)(base, nov);
        }
    } else {
        /* smooth dielectric */
        R ci = FN(dot)(V, N);
        int entering = ci > K(0.0);
        R n1 = entering ? K(1.0) : ior, n2 = entering ? ior : K(1.0);
        FN(v3) nn = entering ? N : FN(neg)(N);
        ci = FABS(ci);
        R eta = n1 / n2;
        R s2t = (eta * eta) * (K(1.0) - ci * ci);
        R F = K(1.0), ct = K(0.0);
        if (s2t < K(1.0)) {
            ct = SQRT(K(1.0) - s2t);
            R rs = (n1 * ci - n2 * ct) / (n1 * ci + n2 * ct);
            R rp = (n1 * ct - n2 * ci) / (n1 * ct + n2 * ci);
            F = K(0.5) * (rs * rs + rp * rp);
        }
        if (r1 < F) {
            L = FN(add)(rd, FN(scl)(nn, K(2.0) * ci));
        } else {
            L = FN(normalize)(FN(add)(FN(scl)(rd, eta), FN(scl)(nn, eta * ci - ct)));
            toggle_inside = 1;
        }
        wgt = FN(mk)(K(1.0), K(1.0), K(1.0));
        delta = 1;
        org = FN(add)(pos, FN(scl)(L, FN(offset_eps)(pos)));
    }

    o.L = L; o.wgt = wgt; o.org = org; o.pdf = pdf;
    o.delta = delta; o.valid = valid; o.toggle_inside = toggle_inside;
    return o;
}

/* The BSDF value f toward wl and the pdf with which sample_bsdf would have
 * drawn wl (the connect stage's multiple importance sampling): Lambert
 * base/pi, GGX metal F D G / (4 cos_x NoV) with pdf D NoH / (4 VoH).  Returns
 * 0 where the metal's half vector faces away or D is not finite. */
static int FN(eval_bsdf)(uint32_t bsdf, FN(v3) base, R alpha, FN(v3) N, FN(v3) V, FN(v3) wl, R cos_x, int cosine,
                         FN(v3)* f_out, R* pdf_out) {
    FN(v3) f = FN(mk)(0, 0, 0);
    R pdf_b = K(0.0);
    int ok = 1;
    if (bsdf == 0) {
        f = FN(scl)(base, ORC_INV_PI);
        pdf_b = cosine ? cos_x * ORC_INV_PI : ORC_INV_TWO_PI;
    } else {
        FN(v3) H = FN(normalize)(FN(add)(V, wl));
        R nov = FN(dot)(N, V), noh = FN(dot)(N, H), voh = FN(dot)(V, H);
        if (nov <= K(0.0) || voh <= K(0.0)) ok = 0;
        else {
            R a2 = alpha * alpha;
            R D = FN(ggx_d)(noh, a2);
            R G = FN(g1)(cos_x, a2) * FN(g1)(nov, a2);
            FN(v3) F = FN(schlick)(base, voh);
            f = FN(scl)(F, (D * G) / ((K(4.0) * cos_x) * nov));
            pdf_b = (D * noh) / (K(4.0) * voh);
            if (!(D <= MAXT)) ok = 0;
        }
    }
    *f_out = f;
    *pdf_out = pdf_b;
    return ok;
}

typedef struct {
    const orc_scene* s;
    const view_t* view;
    const orc_render_params* p;
    FN(lights) lights;
    uint32_t width, height, pix0, pix1;
    void* accum;
    volatile uint32_t next_row;
} FN(job);

typedef struct {
    orc_render_stats st;
} FN(tstate);

/* What the adjoint needs of one path: every Lambert vertex (its scene
 * triangle, albedo, and the path radiance gathered before it: the part that
 * does not depend on that albedo), and every emitted contribution (an
 * emission hit or an unoccluded shadow ray) with its emitter and strength. */
typedef struct {
    uint32_t n;
    uint32_t tri[32];       /* scene triangle of each Lambert vertex */
    R rho[32][3];           /* its albedo */
    R before[32][3];        /* path radiance before the vertex */
    uint32_t ne;
    uint32_t em_inst[32];   /* emitter instance of each emitted contribution */
    R em_strength[32];
    R em_c[32][3];          /* the contribution */
} FN(record);

/* One camera path of the wavefront loop (generate.hlsl, extend.hlsl,
 * shade.hlsl:42-174 and the added connect stage).  acc is the path's own
 * radiance, which receives the contributions in the order the GPU stages add
 * them (shade at depth d, then connect at depth d, then depth d+1). */
static void FN(path)(FN(job)* J, uint32_t pixel, uint32_t sample, R acc[3], orc_render_stats* st,
                     FN(record)* rec) {
    if (rec) { rec->n = 0; rec->ne = 0; }
    const orc_scene* s = J->s;
    const orc_render_params* P = J->p;
    uint32_t px = pixel % J->width, py = pixel / J->width;
    RayDesc2 pr;
    orc_primary_ray(J->view, px, py, &pr);
    FN(v3) ro = FN(mk)((R)pr.Origin[0], (R)pr.Origin[1], (R)pr.Origin[2]);
    FN(v3) rd = FN(mk)((R)pr.Direction[0], (R)pr.Direction[1], (R)pr.Direction[2]);
    FN(v3) T = FN(mk)(K(1.0), K(1.0), K(1.0));
    uint32_t flags = ORC_F_SPECULAR;
    R last_pdf = K(0.0);
    FN(v3) env = FN(mk)((R)P->env_color[0], (R)P->env_color[1], (R)P->env_color[2]);
    R env_strength = (R)P->hdr_env_strength;

    for (uint32_t d = 0; d <= P->max_bounces; ++d) {
        st->extend_rays[d < 16 ? d : 15]++;
        FN(hit) h;
        int tr = FN(trace_one)(s, ro, rd, MAXT,
                               ((flags & ORC_F_INSIDE) ? ORC_NO_CULL : 0) | (P->tie_rule ? ORC_TIE_RULE : 0), &h,
                               &st->extend_traffic);
        if (tr < 0) { st->stack_overflows++; }
        if (h.inst == WF_INVALID_INDEX) {
            if (P->view_mode != 0) {
                /* debug views of a miss: the hit record's ids, barycentrics and
                 * t; views of the surface read zero */
                FN(v3) val = FN(mk)(0, 0, 0);
                if (P->view_mode == 1 || P->view_mode == 2) val = FN(int_to_color)(WF_INVALID_INDEX);
                else if (P->view_mode == 3) val = FN(mk)(h.u, h.v, K(0.0));
                else if (P->view_mode == 11) { R q = h.t / (R)J->view->far_plane; val = FN(mk)(q, q, q); }
                acc[0] = acc[0] + val.x; acc[1] = acc[1] + val.y; acc[2] = acc[2] + val.z;
                return;
            }
            if (s->env_texture) env = FN(env_texel)(&s->textures[s->env_texture - 1], rd);
            /* miss: energy += throughput * strength * env (shade.hlsl:60-65) */
            acc[0] = acc[0] + (T.x * env_strength) * env.x;
            acc[1] = acc[1] + (T.y * env_strength) * env.y;
            acc[2] = acc[2] + (T.z * env_strength) * env.z;
            return;
        }
        const orc_instance* in = &s->inst[h.inst];
        const triangle_t* tri = &s->meshes[in->mesh].tris[h.prim];
        /* get_hit_surface (common.hlsl:228-245) */
        FN(v3) p0 = FN(ld)(tri->v0.position), p1 = FN(ld)(tri->v1.position), p2 = FN(ld)(tri->v2.position);
        FN(v3) pl = FN(add)(FN(add)(p0, FN(scl)(FN(sub)(p1, p0), h.u)), FN(scl)(FN(sub)(p2, p0), h.v));
        FN(v3) pos = FN(xform)(pl, K(1.0), in->local_to_world);
        FN(v3) n0 = FN(ld)(tri->v0.normal), n1 = FN(ld)(tri->v1.normal), n2 = FN(ld)(tri->v2.normal);
        FN(v3) nl = FN(add)(FN(add)(n0, FN(scl)(FN(sub)(n1, n0), h.u)), FN(scl)(FN(sub)(n2, n0), h.v));
        FN(v3) N = FN(normalize)(FN(xform)(nl, K(0.0), in->local_to_world));
        /* sample_material (material.hlsl:15-39): factors x textures at the uv */
        const material_t* m = &in->material;
        R tu = K(0.0), tv = K(0.0);
        if ((m->base_color_index | m->normal_index | m->metallic_roughness_index | m->emissive_index) != 0u ||
            P->view_mode == 5) {
            tu = ((R)tri->v0.uv[0] + h.u * ((R)tri->v1.uv[0] - (R)tri->v0.uv[0])) +
                 h.v * ((R)tri->v2.uv[0] - (R)tri->v0.uv[0]);
            tv = ((R)tri->v0.uv[1] + h.u * ((R)tri->v1.uv[1] - (R)tri->v0.uv[1])) +
                 h.v * ((R)tri->v2.uv[1] - (R)tri->v0.uv[1]);
        }
        R tb[4], tmr[4], tem[4];
        FN(mat_tex)(s, m->base_color_index, 0, tu, tv, tb);
        FN(mat_tex)(s, m->metallic_roughness_index, 2, tu, tv, tmr);
        FN(mat_tex)(s, m->emissive_index, 3, tu, tv, tem);
        FN(v3) base = FN(mk)((R)m->base_color_factor[0] * tb[0], (R)m->base_color_factor[1] * tb[1],
                             (R)m->base_color_factor[2] * tb[2]);
        uint32_t stri = 0;
        if (s->tri_albedo) {
            stri = s->inst_tri_offset[h.inst] + h.prim;
            base = FN(mk)((R)s->tri_albedo[3ull * stri], (R)s->tri_albedo[3ull * stri + 1],
                          (R)s->tri_albedo[3ull * stri + 2]);
        }
        FN(v3) le = FN(mk)(((R)m->emissive_strength * (R)m->emissive_factor[0]) * tem[0],
                           ((R)m->emissive_strength * (R)m->emissive_factor[1]) * tem[1],
                           ((R)m->emissive_strength * (R)m->emissive_factor[2]) * tem[2]);
        if (P->view_mode != 0) {
            /* debug views (shade.hlsl:140-153) */
            FN(v3) val = FN(mk)(0, 0, 0);
            uint32_t vm = P->view_mode;
            if (vm == 1) val = FN(int_to_color)(h.inst);
            else if (vm == 2) val = FN(int_to_color)(h.prim);
            else if (vm == 3) val = FN(mk)(h.u, h.v, K(0.0));
            else if (vm == 4) val = FN(abs3)(nl);
            else if (vm == 5) val = FN(mk)(tu, tv, K(0.0));
            else if (vm == 6) val = base;
            else if (vm == 7) { R tn[4]; FN(mat_tex)(s, m->normal_index, 1, tu, tv, tn); val = FN(abs3)(FN(mk)(tn[0], tn[1], tn[2])); }
            else if (vm == 8) val = FN(mk)(K(0.0), tmr[1], tmr[2]);
            else if (vm == 9) val = le;
            else if (vm == 10) val = FN(abs3)(N);
            else if (vm == 11) { R q = h.t / (R)J->view->far_plane; val = FN(mk)(q, q, q); }
            acc[0] = acc[0] + val.x; acc[1] = acc[1] + val.y; acc[2] = acc[2] + val.z;
            return;
        }
        if (le.x != K(0.0) || le.y != K(0.0) || le.z != K(0.0)) {
            R w = K(1.0);
            if (P->nee && !(flags & ORC_F_SPECULAR) && J->lights.count > 0) {
                FN(v3) ng = FN(normalize)(FN(xform)(FN(cross)(FN(sub)(p1, p0), FN(sub)(p2, p0)), K(0.0),
                                                     in->local_to_world));
                R cos_l = -FN(dot)(ng, rd);
                if (cos_l > K(0.0)) {
                    R d2 = (h.t * h.t) * FN(dot)(rd, rd);
                    R pdf_l = d2 / (cos_l * J->lights.total);
                    /* power heuristic in ratio form: 1 / (1 + (pdf_l / pdf_bsdf)^2) */
                    R q = pdf_l / last_pdf;
                    w = (q == q) ? K(1.0) / (K(1.0) + q * q) : K(0.0);
                }
            }
            acc[0] = acc[0] + (T.x * le.x) * w;
            acc[1] = acc[1] + (T.y * le.y) * w;
            acc[2] = acc[2] + (T.z * le.z) * w;
            if (rec && rec->ne < 32) {
                rec->em_inst[rec->ne] = h.inst;
                rec->em_strength[rec->ne] = (R)m->emissive_strength;
                rec->em_c[rec->ne][0] = (T.x * le.x) * w;
                rec->em_c[rec->ne][1] = (T.y * le.y) * w;
                rec->em_c[rec->ne][2] = (T.z * le.z) * w;
                rec->ne++;
            }
            return;
        }
        uint32_t seed = orc_path_seed(P->frame_seed, pixel, sample, d);
        (void)orc_rand_float(&seed); /* r_path: drawn as in shade.hlsl:81, unused */
        R r1 = (R)orc_rand_float(&seed);
        R r2 = (R)orc_rand_float(&seed);
        FN(v3) V = FN(neg)(rd);
        FN(v3) L = FN(mk)(0, 0, 0), wgt = FN(mk)(0, 0, 0);
        R pdf = K(0.0);
        int delta = 0, valid = 1, toggle_inside = 0;
        FN(v3) org = pos;
        R rough = (R)m->roughness_factor * tmr[1];   /* roughness factor x texture green */
        R alpha = rough * rough;
        uint32_t bsdf = in->bsdf;
        if (bsdf == 1 && alpha < ORC_METAL_DELTA_ALPHA) bsdf = 3; /* mirror */
        /* a ray travelling inside glass may reach an opaque surface from behind */
        if ((flags & ORC_F_INSIDE) && bsdf != 2 && FN(dot)(N, V) < K(0.0)) N = FN(neg)(N);
        FN(v3) tg, bt;
        FN(basis)(N, &tg, &bt);
        if (bsdf == 0 && rec && s->tri_albedo && rec->n < 32) {
            rec->tri[rec->n] = stri;
            rec->rho[rec->n][0] = base.x; rec->rho[rec->n][1] = base.y; rec->rho[rec->n][2] = base.z;
            rec->before[rec->n][0] = acc[0]; rec->before[rec->n][1] = acc[1]; rec->before[rec->n][2] = acc[2];
            rec->n++;
        }
        FN(scatter) sc_ = FN(sample_bsdf)(bsdf, base, alpha, (R)in->ior, N, tg, bt, rd, pos, r1, r2,
                                          (int)P->cosine_weighted_diffuse);
        L = sc_.L; wgt = sc_.wgt; org = sc_.org; pdf = sc_.pdf;
        delta = sc_.delta; valid = sc_.valid; toggle_inside = sc_.toggle_inside;

        /* connect: next-event estimation towards the emitter table */
        if (P->nee && !delta && d < P->max_bounces && J->lights.count > 0) {
            R rl0 = (R)orc_rand_float(&seed);
            R rl1 = (R)orc_rand_float(&seed);
            R rl2 = (R)orc_rand_float(&seed);
            const FN(light)* lt = &J->lights.tri[FN(pick_light)(&J->lights, rl0)];
            R su = SQRT(rl1);
            R b1 = su * (K(1.0) - rl2), b2 = su * rl2;
            FN(v3) y = FN(add)(FN(add)(lt->p0, FN(scl)(lt->e1, b1)), FN(scl)(lt->e2, b2));
            FN(v3) wv = FN(sub)(y, pos);
            R dd2 = FN(dot)(wv, wv);
            R dist = SQRT(dd2);
            FN(v3) wl = FN(scl)(wv, K(1.0) / dist);
            R cos_l = -FN(dot)(lt->n, wl);
            R cos_x = FN(dot)(N, wl);
            if (cos_l > K(0.0) && cos_x > K(0.0)) {
                R pdf_l = dd2 / (cos_l * J->lights.total);
                FN(v3) f;
                R pdf_b;
                int ok = FN(eval_bsdf)(bsdf, base, alpha, N, V, wl, cos_x, (int)P->cosine_weighted_diffuse, &f, &pdf_b);
                if (ok) {
                    R q = pdf_b / pdf_l;
                    R w = (q == q) ? K(1.0) / (K(1.0) + q * q) : K(0.0);
                    R sc = (cos_x * w) / pdf_l;
                    FN(v3) ltle = lt->le;
                    if (lt->tex) {
                        /* textured emitter: its emission texture at the sampled point */
                        R lu = (lt->uv[0] + b1 * (lt->uv[2] - lt->uv[0])) + b2 * (lt->uv[4] - lt->uv[0]);
                        R lv = (lt->uv[1] + b1 * (lt->uv[3] - lt->uv[1])) + b2 * (lt->uv[5] - lt->uv[1]);
                        R te[4];
                        FN(tex_sample)(&s->textures[lt->tex - 1], lu, lv, te);
                        ltle = FN(mk)(ltle.x * te[0], ltle.y * te[1], ltle.z * te[2]);
                    }
                    FN(v3) contrib = FN(mk)(((T.x * f.x) * sc) * ltle.x, ((T.y * f.y) * sc) * ltle.y,
                                            ((T.z * f.z) * sc) * ltle.z);
                    st->shadow_rays[d < 16 ? d : 15]++;
                    FN(hit) sh;
                    int r = FN(trace_one)(s, pos, wl, dist * ORC_SHADOW_TMAX_SCALE, ORC_ANY_HIT, &sh,
                                          &st->shadow_traffic);
                    if (r < 0) st->stack_overflows++;
                    if (sh.inst == WF_INVALID_INDEX && r >= 0) {
                        acc[0] = acc[0] + contrib.x;
                        acc[1] = acc[1] + contrib.y;
                        acc[2] = acc[2] + contrib.z;
                        if (rec && rec->ne < 32) {
                            rec->em_inst[rec->ne] = lt->inst;
                            rec->em_strength[rec->ne] = lt->strength;
                            rec->em_c[rec->ne][0] = contrib.x;
                            rec->em_c[rec->ne][1] = contrib.y;
                            rec->em_c[rec->ne][2] = contrib.z;
                            rec->ne++;
                        }
                    }
                }
            }
        }
        if (!valid) return;
        T = FN(mul)(T, wgt);
        if (d >= P->max_bounces) return;
        if (d >= P->rr_start_depth) {
            R rr = (R)orc_rand_float(&seed);
            R q = FMIN(FMAX(FMAX(T.x, T.y), T.z), K(1.0));
            if (rr >= q) return;
            T = FN(mk)(T.x / q, T.y / q, T.z / q);
        }
        if (toggle_inside) flags ^= ORC_F_INSIDE;
        flags = delta ? (flags | ORC_F_SPECULAR) : (flags & ~ORC_F_SPECULAR);
        last_pdf = pdf;
        ro = org;
        rd = L;
    }
}
