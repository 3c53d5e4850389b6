/*
 * orc_trace.c — oracle traversal, shading and rendering entry points.
 * TEST INFRASTRUCTURE ONLY (see wf_oracle.h).  Instantiates orc_impl.h for
 * float (the GPU's bit-exact contract) and double (the image oracle).
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include "wf_oracle.h"

/* ---- random numbers (common.hlsl:79-97, core/random.h:7-24) ----------- */
uint32_t orc_wang_hash(uint32_t seed) {
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed;
}

/* rand_float: float(wang_hash(seed)) * 2.3283064365387e-10f; the result can
 * round up to exactly 1.0f. */
float orc_rand_float(uint32_t* seed) {
    *seed = orc_wang_hash(*seed);
    return (float)(*seed) * 2.3283064365387e-10f;
}

/* Per-path seed.  The reference seeds by frame_seed + compacted queue index
 * (shade.hlsl:80), which changes with the order in which an atomic hands out
 * slots; this build keys the stream by (pixel, sample, depth) so that a path
 * can be replayed and the GPU and CPU draw the same numbers. */
uint32_t orc_path_seed(uint32_t frame_seed, uint32_t pixel, uint32_t sample, uint32_t depth) {
    uint32_t s = frame_seed + pixel;
    s = orc_wang_hash(s) ^ (sample * 0x9E3779B9u);
    s = orc_wang_hash(s) ^ (depth * 0x85EBCA6Bu);
    return s;
}

/* sin(phi), cos(phi): Cody-Waite reduction by pi/2 with a three-part
 * constant (1.5703125 + 4.838268e-4 + 2.563344e-12; the first two parts have
 * 8 and 22 significant bits, so k times them is exact while |k| <= 4, i.e.
 * for |phi| up to about 7), k = rint(phi * 2/pi), x = phi - k*pi/2 in about
 * [-pi/4, pi/4]; then truncated Taylor series (sin to x^9, cos to x^10,
 * truncation error below 2e-9) in Horner form, and a quarter-turn rotation by
 * k mod 4.  Absolute error against sin/cos of the same float phi < 1e-7 on
 * [0, 2*pi].  Written out operation by operation so the CUDA kernels can
 * evaluate the identical sequence.  This is this project's definition of the
 * HLSL sin / cos intrinsics, whose precision nothing in the reference pins. */
void orc_sincos(float phi, float* s_out, float* c_out) {
    float k = rintf(phi * 0.636619747f);
    float x = phi - k * 1.5703125f;
    x = x - k * 4.83826792e-4f;
    x = x - k * 2.56334415e-12f;
    float x2 = x * x;
    float sp = -1.98412698e-4f + x2 * 2.75573192e-6f;
    sp = 8.33333377e-3f + x2 * sp;
    sp = -1.66666672e-1f + x2 * sp;
    float sn = x + (x * x2) * sp;
    float cp = 2.48015876e-5f + x2 * -2.75573188e-7f;
    cp = -1.38888892e-3f + x2 * cp;
    cp = 4.16666679e-2f + x2 * cp;
    cp = -0.5f + x2 * cp;
    float cs = 1.0f + x2 * cp;
    int q = ((int)k) & 3;
    float s, c;
    if (q == 0) { s = sn; c = cs; }
    else if (q == 1) { s = cs; c = -sn; }
    else if (q == 2) { s = -sn; c = -cs; }
    else { s = -cs; c = sn; }
    *s_out = s;
    *c_out = c;
}

/* The hemisphere samplers' angle (sample.hlsl:29-54): phi = 2.0 * PI * r.y
 * with PI = 3.14159265, i.e. the float 6.28318548 times r, rounded to float,
 * then sin(phi) and cos(phi). */
void orc_sincos_2pi(float r, float* s_out, float* c_out) { orc_sincos(6.28318548f * r, s_out, c_out); }

static void sincos_2pi_f64(double r, double* s, double* c) {
    double a = 6.283185307179586 * r;
    *s = sin(a);
    *c = cos(a);
}

/* ---- instantiations ------------------------------------------------------ */
/* ---- FP32 inverse trigonometry (the GPU library's own, same operations) ----
 * On [0, 1] arguments above tan(pi/8) are reduced by atan z = pi/4 +
 * atan((z - 1) / (z + 1)); on |z| <= tan(pi/8) the Taylor series of atan
 * through z^17 in Horner form. */
static float atan_unit_f(float z) {
    float off = 0.0f;
    if (z > 0.41421357f) {
        z = (z - 1.0f) / (z + 1.0f);
        off = 0.78539819f;
    }
    const float t2 = z * z;
    float p = 0.05882353f;
    p = 0.06666667f - t2 * p;
    p = 0.07692308f - t2 * p;
    p = 0.09090909f - t2 * p;
    p = 0.11111111f - t2 * p;
    p = 0.14285715f - t2 * p;
    p = 0.2f - t2 * p;
    p = 0.33333334f - t2 * p;
    p = 1.0f - t2 * p;
    return off + z * p;
}
float orc_atan2(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f) return 0.0f;
    float a = (ay <= ax) ? atan_unit_f(ay / ax) : 1.57079637f - atan_unit_f(ax / ay);
    if (x < 0.0f) a = 3.14159274f - a;
    return (y < 0.0f) ? -a : a;
}
float orc_asin(float y) { return orc_atan2(y, sqrtf(fmaxf(0.0f, (1.0f - y) * (1.0f + y)))); }

static uint32_t murmur_mix(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

/* Wrap addressing of an integral coordinate; out-of-range or non-finite
 * coordinates read texel 0 (as the GPU library). */
static uint32_t wrap_texel(double f, uint32_t n) {
    if (!(f > -16777216.0 && f < 16777216.0)) return 0u;
    int m = ((int)f) % (int)n;
    if (m < 0) m += (int)n;
    return (uint32_t)m;
}

#define R float
#define FN(x) x##_f32
#define ATAN2 orc_atan2
#define ASIN orc_asin
#define FLOOR floorf
#define K(x) x##f
#define SQRT sqrtf
#define FABS fabsf
#define FMIN fminf
#define FMAX fmaxf
#define SINCOS2PI(r, s, c) orc_sincos_2pi((r), (s), (c))
#define MAXT FLT_MAX
#include "orc_impl.h"
#undef R
#undef FN
#undef K
#undef SQRT
#undef FABS
#undef FMIN
#undef FMAX
#undef SINCOS2PI
#undef MAXT

void orc_int_to_color(uint32_t v, float out[3]) {
    v3_f32 c = int_to_color_f32(v);
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}
void orc_tex_sample(const orc_texture* t, float u, float v, float out[4]) { tex_sample_f32(t, u, v, out); }
void orc_env_texel(const orc_texture* t, const float dir[3], float out[3]) {
    v3_f32 c = env_texel_f32(t, mk_f32(dir[0], dir[1], dir[2]));
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}
void orc_hemisphere_sample(const float n[3], float r1, float r2, int cosine, float out[3]) {
    v3_f32 N = mk_f32(n[0], n[1], n[2]), tg, bt;
    basis_f32(N, &tg, &bt);
    v3_f32 L = hemisphere_f32(N, tg, bt, r1, r2, cosine);
    out[0] = L.x; out[1] = L.y; out[2] = L.z;
}

#undef ATAN2
#undef ASIN
#undef FLOOR
#define R double
#define FN(x) x##_f64
#define ATAN2 atan2
#define ASIN asin
#define FLOOR floor
#define K(x) x
#define SQRT sqrt
#define FABS fabs
#define FMIN fmin
#define FMAX fmax
#define SINCOS2PI(r, s, c) sincos_2pi_f64((r), (s), (c))
#define MAXT ((double)FLT_MAX)
#include "orc_impl.h"

/* ---- the scattering models on their own (physics tests) ------------------- */
/* Draws one scattering direction at a surface with shading normal n for a ray
 * arriving along rd, as the shade stage does (in = bsdf, base[3], alpha, ior,
 * r1, r2, cosine; out = L[3], weight[3], pdf, flags bit 0 delta, bit 1 valid,
 * bit 2 toggles inside).  f64 selects the double instance. */
int orc_sample_bsdf(int f64, uint32_t bsdf, const double base[3], double alpha, double ior, const double n[3],
                    const double rd[3], double r1, double r2, int cosine, double L[3], double wgt[3], double* pdf) {
    scatter_f64 o;
    if (f64) {
        v3_f64 N = mk_f64(n[0], n[1], n[2]), tg, bt;
        basis_f64(N, &tg, &bt);
        o = sample_bsdf_f64(bsdf, mk_f64(base[0], base[1], base[2]), alpha, ior, N, tg, bt,
                            mk_f64(rd[0], rd[1], rd[2]), mk_f64(0, 0, 0), r1, r2, cosine);
    } else {
        v3_f32 N = mk_f32((float)n[0], (float)n[1], (float)n[2]), tg, bt;
        basis_f32(N, &tg, &bt);
        scatter_f32 q = sample_bsdf_f32(bsdf, mk_f32((float)base[0], (float)base[1], (float)base[2]), (float)alpha,
                                        (float)ior, N, tg, bt, mk_f32((float)rd[0], (float)rd[1], (float)rd[2]),
                                        mk_f32(0, 0, 0), (float)r1, (float)r2, cosine);
        o.L = mk_f64(q.L.x, q.L.y, q.L.z);
        o.wgt = mk_f64(q.wgt.x, q.wgt.y, q.wgt.z);
        o.pdf = q.pdf;
        o.delta = q.delta; o.valid = q.valid; o.toggle_inside = q.toggle_inside;
    }
    L[0] = o.L.x; L[1] = o.L.y; L[2] = o.L.z;
    wgt[0] = o.wgt.x; wgt[1] = o.wgt.y; wgt[2] = o.wgt.z;
    *pdf = o.pdf;
    return (o.delta ? 1 : 0) | (o.valid ? 2 : 0) | (o.toggle_inside ? 4 : 0);
}

/* orc_sample_bsdf for m random pairs r[2m] at one surface configuration. */
void orc_sample_bsdf_batch(int f64, uint32_t bsdf, const double base[3], double alpha, double ior, const double n[3],
                           const double rd[3], const double* r, uint32_t m, int cosine, double* L, double* wgt,
                           double* pdf, int* flags) {
    for (uint32_t i = 0; i < m; ++i)
        flags[i] = orc_sample_bsdf(f64, bsdf, base, alpha, ior, n, rd, r[2 * i], r[2 * i + 1], cosine, L + 3 * i,
                                   wgt + 3 * i, pdf + i);
}

/* The BSDF value toward wl and its sampling pdf, as the connect stage
 * evaluates them (v = the direction back to the viewer).  Returns 1 if
 * valid. */
int orc_eval_bsdf(uint32_t bsdf, const double base[3], double alpha, const double n[3], const double v[3],
                  const double wl[3], int cosine, double f[3], double* pdf) {
    v3_f64 N = mk_f64(n[0], n[1], n[2]), W = mk_f64(wl[0], wl[1], wl[2]), fo;
    int ok = eval_bsdf_f64(bsdf, mk_f64(base[0], base[1], base[2]), alpha, N, mk_f64(v[0], v[1], v[2]), W,
                           dot_f64(N, W), cosine, &fo, pdf);
    f[0] = fo.x; f[1] = fo.y; f[2] = fo.z;
    return ok;
}

/* orc_eval_bsdf toward m directions wl[3m]. */
void orc_eval_bsdf_batch(uint32_t bsdf, const double base[3], double alpha, const double n[3], const double v[3],
                         const double* wl, uint32_t m, int cosine, double* f, double* pdf, int* ok) {
    for (uint32_t i = 0; i < m; ++i) ok[i] = orc_eval_bsdf(bsdf, base, alpha, n, v, wl + 3 * i, cosine, f + 3 * i, pdf + i);
}

/* ---- exported known-answer helpers ---------------------------------------- */
int orc_intersect_triangle(const float v0[3], const float v1[3], const float v2[3], const float org[3],
                           const float dir[3], float* t_inout, float bary[2], int no_cull) {
    return tri_f32(ld_f32(v0), ld_f32(v1), ld_f32(v2), ld_f32(org), ld_f32(dir), t_inout, &bary[0], &bary[1],
                   no_cull);
}

float orc_intersect_aabb(const float bmin[3], const float bmax[3], const float org[3], const float inv_dir[3],
                         float t) {
    return slab_f32(bmin, bmax, ld_f32(org), ld_f32(inv_dir), t);
}

/* make_primary_ray (hardware-ray variant, common.hlsl:182-195): no origin
 * nudge, TMin = 1e-8, TMax = FLT_MAX. */
void orc_primary_ray(const view_t* view, uint32_t px, uint32_t py, RayDesc2* out) {
    float uvx = ((float)px + 0.5f) / view->render_dim[0];
    float uvy = ((float)py + 0.5f) / view->render_dim[1];
    uvy = 1.0f - uvy;
    float cx = 2.0f * uvx - 1.0f, cy = 2.0f * uvy - 1.0f;
    v3_f32 pv = xform_f32(mk_f32(cx, cy, 1.0f), 1.0f, view->clip_to_view);
    v3_f32 dv = normalize_f32(pv);
    v3_f32 dw = xform_f32(dv, 0.0f, view->view_to_world);
    v3_f32 ow = xform_f32(mk_f32(0.0f, 0.0f, 0.0f), 1.0f, view->view_to_world);
    out->Origin[0] = ow.x; out->Origin[1] = ow.y; out->Origin[2] = ow.z;
    out->TMin = 1e-8f;
    out->Direction[0] = dw.x; out->Direction[1] = dw.y; out->Direction[2] = dw.z;
    out->TMax = FLT_MAX;
}

/* ---- multithreaded ray queries -------------------------------------------- */
typedef struct {
    const orc_scene* s;
    const RayDesc2* rays;
    hit_result_t* hits;
    uint32_t n, flags;
    int f64;
    volatile uint32_t next;
    pthread_mutex_t mu;
    orc_counters total;
    uint32_t overflows;
} trace_job;

static void* trace_worker(void* arg) {
    trace_job* J = (trace_job*)arg;
    orc_counters c = {0, 0, 0, 0};
    uint32_t ovf = 0;
    for (;;) {
        uint32_t begin = __atomic_fetch_add(&J->next, 4096u, __ATOMIC_RELAXED);
        if (begin >= J->n) break;
        uint32_t end = begin + 4096u < J->n ? begin + 4096u : J->n;
        for (uint32_t i = begin; i < end; ++i) {
            const RayDesc2* r = &J->rays[i];
            hit_result_t* o = &J->hits[i];
            if (!J->f64) {
                hit_f32 h;
                int rc = trace_one_f32(J->s, ld_f32(r->Origin), ld_f32(r->Direction), r->TMax, J->flags, &h, &c);
                if (rc < 0) ovf++;
                o->instance_idx = h.inst; o->primitive_idx = h.prim; o->t = h.t;
                o->bary[0] = h.u; o->bary[1] = h.v;
            } else {
                hit_f64 h;
                int rc = trace_one_f64(J->s, ld_f64(r->Origin), ld_f64(r->Direction), (double)r->TMax, J->flags,
                                       &h, &c);
                if (rc < 0) ovf++;
                o->instance_idx = h.inst; o->primitive_idx = h.prim; o->t = (float)h.t;
                o->bary[0] = (float)h.u; o->bary[1] = (float)h.v;
            }
        }
    }
    pthread_mutex_lock(&J->mu);
    J->total.tlas_node_loads += c.tlas_node_loads;
    J->total.instance_loads += c.instance_loads;
    J->total.blas_node_loads += c.blas_node_loads;
    J->total.triangle_tests += c.triangle_tests;
    J->overflows += ovf;
    pthread_mutex_unlock(&J->mu);
    return NULL;
}

static uint32_t run_trace(const orc_scene* s, const RayDesc2* rays, uint32_t n, hit_result_t* hits, uint32_t flags,
                          orc_counters* counters, int threads, int f64) {
    trace_job J;
    memset(&J, 0, sizeof(J));
    J.s = s; J.rays = rays; J.hits = hits; J.n = n; J.flags = flags; J.f64 = f64;
    pthread_mutex_init(&J.mu, NULL);
    if (threads <= 1) {
        trace_worker(&J);
    } else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
        for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, trace_worker, &J);
        for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    if (counters) *counters = J.total;
    return J.overflows;
}

uint32_t orc_trace(const orc_scene* s, const RayDesc2* rays, uint32_t n, hit_result_t* hits, uint32_t flags,
                   orc_counters* counters, int threads) {
    return run_trace(s, rays, n, hits, flags, counters, threads, 0);
}

uint32_t orc_trace_f64(const orc_scene* s, const RayDesc2* rays, uint32_t n, hit_result_t* hits, uint32_t flags,
                       int threads) {
    return run_trace(s, rays, n, hits, flags, NULL, threads, 1);
}

/* ---- rendering ----------------------------------------------------------- */
typedef struct {
    const orc_scene* s;
    const view_t* view;
    const orc_render_params* p;
    lights_f32 l32;
    lights_f64 l64;
    int f64;
    uint32_t width, pix0, pix1;
    float* acc32;
    double* acc64;
    volatile uint32_t next;
    pthread_mutex_t mu;
    orc_render_stats total;
} render_job;

static void merge_counters(orc_counters* a, const orc_counters* b) {
    a->tlas_node_loads += b->tlas_node_loads;
    a->instance_loads += b->instance_loads;
    a->blas_node_loads += b->blas_node_loads;
    a->triangle_tests += b->triangle_tests;
}

static void* render_worker(void* arg) {
    render_job* J = (render_job*)arg;
    orc_render_stats st;
    memset(&st, 0, sizeof(st));
    job_f32 j32;
    job_f64 j64;
    memset(&j32, 0, sizeof(j32));
    memset(&j64, 0, sizeof(j64));
    j32.s = J->s; j32.view = J->view; j32.p = J->p; j32.lights = J->l32; j32.width = J->width;
    j64.s = J->s; j64.view = J->view; j64.p = J->p; j64.lights = J->l64; j64.width = J->width;
    const uint32_t chunk = 256;
    for (;;) {
        uint32_t begin = __atomic_fetch_add(&J->next, chunk, __ATOMIC_RELAXED);
        uint32_t b = J->pix0 + begin;
        if (b >= J->pix1) break;
        uint32_t e = b + chunk < J->pix1 ? b + chunk : J->pix1;
        for (uint32_t px = b; px < e; ++px) {
            for (uint32_t sidx = 0; sidx < J->p->spp; ++sidx) {
                uint32_t sample = J->p->sample_offset + sidx;
                /* a path sums its own contributions from zero; the pixel then
                 * adds whole paths in sample order */
                if (!J->f64) {
                    float L[3] = {0.0f, 0.0f, 0.0f};
                    path_f32(&j32, px, sample, L, &st, NULL);
                    J->acc32[4ull * px] = J->acc32[4ull * px] + L[0];
                    J->acc32[4ull * px + 1] = J->acc32[4ull * px + 1] + L[1];
                    J->acc32[4ull * px + 2] = J->acc32[4ull * px + 2] + L[2];
                    J->acc32[4ull * px + 3] += 1.0f;
                } else {
                    double L[3] = {0.0, 0.0, 0.0};
                    path_f64(&j64, px, sample, L, &st, NULL);
                    J->acc64[4ull * px] = J->acc64[4ull * px] + L[0];
                    J->acc64[4ull * px + 1] = J->acc64[4ull * px + 1] + L[1];
                    J->acc64[4ull * px + 2] = J->acc64[4ull * px + 2] + L[2];
                    J->acc64[4ull * px + 3] += 1.0;
                }
            }
        }
    }
    pthread_mutex_lock(&J->mu);
    for (int d = 0; d < 16; ++d) {
        J->total.extend_rays[d] += st.extend_rays[d];
        J->total.shadow_rays[d] += st.shadow_rays[d];
    }
    J->total.stack_overflows += st.stack_overflows;
    merge_counters(&J->total.extend_traffic, &st.extend_traffic);
    merge_counters(&J->total.shadow_traffic, &st.shadow_traffic);
    pthread_mutex_unlock(&J->mu);
    return NULL;
}

static int run_render(const orc_scene* s, const view_t* view, const orc_render_params* p, float* acc32,
                      double* acc64, orc_render_stats* stats, int threads) {
    if (!s || !view || !p || p->max_bounces > 15) return -1;
    render_job J;
    memset(&J, 0, sizeof(J));
    J.s = s; J.view = view; J.p = p; J.acc32 = acc32; J.acc64 = acc64; J.f64 = acc64 != NULL;
    J.width = (uint32_t)view->render_dim[0];
    uint32_t npix = J.width * (uint32_t)view->render_dim[1];
    J.pix0 = p->pixel_begin;
    J.pix1 = p->pixel_end ? p->pixel_end : npix;
    if (J.pix1 > npix || J.pix0 > J.pix1) return -1;
    if (J.f64) build_lights_f64(s, &J.l64);
    else build_lights_f32(s, &J.l32);
    pthread_mutex_init(&J.mu, NULL);
    if (threads <= 1) {
        render_worker(&J);
    } else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
        for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, render_worker, &J);
        for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    if (J.f64) { free(J.l64.tri); free(J.l64.cdf); }
    else { free(J.l32.tri); free(J.l32.cdf); }
    if (stats) *stats = J.total;
    return 0;
}

int orc_render(const orc_scene* s, const view_t* view, const orc_render_params* p, float* accum,
               orc_render_stats* stats, int threads) {
    if (!accum) return -1;
    return run_render(s, view, p, accum, NULL, stats, threads);
}

int orc_render_f64(const orc_scene* s, const view_t* view, const orc_render_params* p, double* accum,
                   int threads) {
    if (!accum) return -1;
    return run_render(s, view, p, NULL, accum, NULL, threads);
}

/* The adjoint of one precision: each path traced as path_<R> traces it, the
 * gradient accumulated in double. */
#define ORC_ADJOINT_BODY(SUF)                                                                                 \
    job_##SUF J;                                                                                              \
    memset(&J, 0, sizeof(J));                                                                                 \
    J.s = s; J.view = view; J.p = p; J.width = (uint32_t)view->render_dim[0];                                 \
    build_lights_##SUF(s, &J.lights);                                                                         \
    const uint32_t npix = J.width * (uint32_t)view->render_dim[1];                                            \
    const double inv_spp = 1.0 / (double)p->spp;                                                              \
    orc_render_stats st;                                                                                      \
    memset(&st, 0, sizeof(st));                                                                               \
    record_##SUF rec;                                                                                         \
    for (uint32_t px = 0; px < npix; ++px) {                                                                  \
        for (uint32_t si = 0; si < p->spp; ++si) {                                                            \
            R_##SUF L[3] = {0, 0, 0};                                                                         \
            path_##SUF(&J, px, p->sample_offset + si, L, &st, &rec);                                          \
            const double w[3] = {dimg[3ull * px] * inv_spp, dimg[3ull * px + 1] * inv_spp,                   \
                                 dimg[3ull * px + 2] * inv_spp};                                              \
            /* a Lambert vertex scales everything gathered after it */                                        \
            for (uint32_t v = 0; v < rec.n; ++v)                                                              \
                for (int c = 0; c < 3; ++c)                                                                   \
                    if (rec.rho[v][c] != 0)                                                                   \
                        g_albedo[3ull * rec.tri[v] + c] +=                                                    \
                            w[c] * ((double)L[c] - (double)rec.before[v][c]) / (double)rec.rho[v][c];         \
            /* an emitted contribution is linear in its emitter's strength */                                 \
            for (uint32_t e = 0; e < rec.ne; ++e)                                                             \
                if (rec.em_strength[e] != 0)                                                                  \
                    g_emission[rec.em_inst[e]] += (w[0] * rec.em_c[e][0] + w[1] * rec.em_c[e][1] +            \
                                                   w[2] * rec.em_c[e][2]) / (double)rec.em_strength[e];       \
        }                                                                                                     \
    }                                                                                                         \
    free(J.lights.tri);                                                                                       \
    free(J.lights.cdf);

typedef float R_f32;
typedef double R_f64;

int orc_adjoint_f64(const orc_scene* s, const view_t* view, const orc_render_params* p, const double* dimg,
                    double* g_albedo, double* g_emission) {
    if (!s || !view || !p || !dimg || !g_albedo || !g_emission || !s->tri_albedo || p->max_bounces > 15) return -1;
    ORC_ADJOINT_BODY(f64)
    return 0;
}

int orc_adjoint_f32(const orc_scene* s, const view_t* view, const orc_render_params* p, const double* dimg,
                    double* g_albedo, double* g_emission) {
    if (!s || !view || !p || !dimg || !g_albedo || !g_emission || !s->tri_albedo || p->max_bounces > 15) return -1;
    ORC_ADJOINT_BODY(f32)
    return 0;
}
