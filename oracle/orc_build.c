/*
 * orc_build.c — oracle restatement of the reference's CPU acceleration-
 * structure builders.  TEST INFRASTRUCTURE ONLY (see wf_oracle.h).
 *
 * BLAS: binned-SAH builder, bvh_builder.cpp:6-264 with as_util.h:7-23.
 * TLAS: agglomerative builder, tlas_builder.cpp:6-110.
 *
 * min/max follow glm 1.0.0 (extern/glm/detail/func_common.inl:17-35):
 * min(x, y) = (y < x) ? y : x and max(x, y) = (x < y) ? y : x, folded in the
 * same order as the reference so that even the sign of a zero bound matches.
 */
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include "wf_oracle.h"

static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline float gmax(float x, float y) { return (x < y) ? y : x; }

typedef struct { float v[3]; } f3;

/* as_util::get_aabb_volume (as_util.h:7-11): the half surface area. */
static inline float half_area(const float* mn, const float* mx) {
    float ex = mx[0] - mn[0], ey = mx[1] - mn[1], ez = mx[2] - mn[2];
    return ex * ey + ey * ez + ez * ex;
}

typedef struct {
    uint32_t interval_count, subdivide_single_prim, max_leaf_prims;
    uint32_t n;
    bvh_triangle_t* tris;
    uint32_t* idx;
    f3* centroid;
    bvh_node_t* nodes;
    uint32_t node_at;
    /* per-call bin scratch */
    float* bmin; float* bmax; uint32_t* bcnt; float* larea; float* rarea;
} builder;

/* get_triangle_centroid (bvh_builder.cpp:252-255): (p0 + p1 + p2) * 0.3333f. */
static f3 centroid_of(const bvh_triangle_t* t) {
    f3 c;
    for (int a = 0; a < 3; ++a) c.v[a] = ((t->p0[a] + t->p1[a]) + t->p2[a]) * 0.3333f;
    return c;
}

/* calc_node_min_max (bvh_builder.cpp:71-93). */
static void node_bounds(builder* b, bvh_node_t* node, float* cmin, float* cmax) {
    for (int a = 0; a < 3; ++a) {
        node->aabb_min[a] = FLT_MAX; node->aabb_max[a] = -FLT_MAX;
        cmin[a] = FLT_MAX; cmax[a] = -FLT_MAX;
    }
    for (uint32_t i = node->left_first; i < node->left_first + node->prim_count; ++i) {
        const bvh_triangle_t* t = &b->tris[b->idx[i]];
        const f3* c = &b->centroid[b->idx[i]];
        for (int a = 0; a < 3; ++a) {
            float tmn = gmin(gmin(t->p0[a], t->p1[a]), t->p2[a]);
            float tmx = gmax(gmax(t->p0[a], t->p1[a]), t->p2[a]);
            node->aabb_min[a] = gmin(node->aabb_min[a], tmn);
            node->aabb_max[a] = gmax(node->aabb_max[a], tmx);
            cmin[a] = gmin(cmin[a], c->v[a]);
            cmax[a] = gmax(cmax[a], c->v[a]);
        }
    }
}

/* find_best_split_plane (bvh_builder.cpp:170-250). */
static float best_split(builder* b, const bvh_node_t* node, const float* cmin, const float* cmax,
                        uint32_t* out_axis, uint32_t* out_pos) {
    float cheapest = FLT_MAX;
    const uint32_t nb = b->interval_count;
    for (uint32_t axis = 0; axis < 3; ++axis) {
        float lo = cmin[axis], hi = cmax[axis];
        if (lo == hi) continue;
        for (uint32_t i = 0; i < nb; ++i) {
            b->bcnt[i] = 0;
            for (int a = 0; a < 3; ++a) { b->bmin[i * 3 + a] = FLT_MAX; b->bmax[i * 3 + a] = -FLT_MAX; }
        }
        float scale = (float)nb / (hi - lo);
        for (uint32_t i = node->left_first; i < node->left_first + node->prim_count; ++i) {
            const bvh_triangle_t* t = &b->tris[b->idx[i]];
            int32_t bin = (int32_t)((b->centroid[b->idx[i]].v[axis] - lo) * scale);
            if ((int32_t)nb - 1 < bin) bin = (int32_t)nb - 1;
            b->bcnt[bin]++;
            const float* p[3] = {t->p0, t->p1, t->p2};
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) {
                    b->bmin[bin * 3 + a] = gmin(b->bmin[bin * 3 + a], p[k][a]);
                    b->bmax[bin * 3 + a] = gmax(b->bmax[bin * 3 + a], p[k][a]);
                }
        }
        float lmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        float rmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t lsum = 0, rsum = 0;
        for (uint32_t i = 0; i < nb - 1; ++i) {
            lsum += b->bcnt[i];
            for (int a = 0; a < 3; ++a) {
                lmn[a] = gmin(lmn[a], b->bmin[i * 3 + a]);
                lmx[a] = gmax(lmx[a], b->bmax[i * 3 + a]);
            }
            b->larea[i] = (float)lsum * half_area(lmn, lmx);
            uint32_t r = nb - 1 - i;
            rsum += b->bcnt[r];
            for (int a = 0; a < 3; ++a) {
                rmn[a] = gmin(rmn[a], b->bmin[r * 3 + a]);
                rmx[a] = gmax(rmx[a], b->bmax[r * 3 + a]);
            }
            b->rarea[nb - 2 - i] = (float)rsum * half_area(rmn, rmx);
        }
        for (uint32_t i = 0; i < nb - 1; ++i) {
            float cost = b->larea[i] + b->rarea[i];
            if (cost < cheapest) { *out_axis = axis; *out_pos = i + 1; cheapest = cost; }
        }
    }
    return cheapest;
}

/* subdivide_node (bvh_builder.cpp:100-168), with the recursion unrolled onto an
 * explicit stack that still visits left before right (pre-order), so child
 * pairs are numbered exactly as the recursive version numbers them. */
static void subdivide(builder* b) {
    typedef struct { uint32_t node; float cmin[3], cmax[3]; } item;
    uint32_t cap = 128, top = 0;
    item* st = (item*)malloc(sizeof(item) * cap);
    st[top].node = 0;
    node_bounds(b, &b->nodes[0], st[top].cmin, st[top].cmax);
    top++;
    while (top > 0) {
        item it = st[--top];
        bvh_node_t* node = &b->nodes[it.node];
        uint32_t axis = 0, pos = 0;
        float cost = best_split(b, node, it.cmin, it.cmax, &axis, &pos);
        if (b->subdivide_single_prim) {
            if (node->prim_count == 1) continue;
        } else {
            int force = b->max_leaf_prims > 0 && node->prim_count > b->max_leaf_prims;
            float parent = (float)node->prim_count * half_area(node->aabb_min, node->aabb_max);
            if (!force && cost >= parent) continue;
        }
        /* Two-pointer partition (bvh_builder.cpp:121-137).  With pos == 0
         * (no plane found: every centroid axis degenerate) the comparison
         * "bin < 0u" is false for every triangle, so the loop still runs and
         * rotates the index range left by one before the node stays a leaf;
         * the bin itself (0 * inf = NaN cast to int) is never needed then. */
        int32_t i = (int32_t)node->left_first;
        int32_t j = i + (int32_t)node->prim_count - 1;
        float scale = pos > 0 ? (float)b->interval_count / (it.cmax[axis] - it.cmin[axis]) : 0.0f;
        while (i <= j) {
            int left = 0;
            if (pos > 0) {
                float c = b->centroid[b->idx[i]].v[axis];
                int32_t bin = (int32_t)((c - it.cmin[axis]) * scale);
                if ((int32_t)b->interval_count - 1 < bin) bin = (int32_t)b->interval_count - 1;
                left = (uint32_t)bin < pos;
            }
            if (left) i++;
            else { uint32_t tmp = b->idx[i]; b->idx[i] = b->idx[j]; b->idx[j] = tmp; j--; }
        }
        uint32_t nleft = (uint32_t)i - node->left_first;
        if (nleft == 0 || nleft == node->prim_count) continue;
        uint32_t l = b->node_at++, r = b->node_at++;
        b->nodes[l].left_first = node->left_first;
        b->nodes[l].prim_count = nleft;
        b->nodes[r].left_first = (uint32_t)i;
        b->nodes[r].prim_count = node->prim_count - nleft;
        node->left_first = l;
        node->prim_count = 0;
        if (top + 2 > cap) { cap *= 2; st = (item*)realloc(st, sizeof(item) * cap); }
        st[top].node = r; node_bounds(b, &b->nodes[r], st[top].cmin, st[top].cmax); top++;
        st[top].node = l; node_bounds(b, &b->nodes[l], st[top].cmin, st[top].cmax); top++;
    }
    free(st);
}

int orc_bvh_build(const triangle_t* tris, uint32_t n, uint32_t interval_count,
                  uint32_t subdivide_single_prim, uint32_t max_leaf_prims,
                  uint8_t** out_blob, uint64_t* out_size) {
    if (!out_blob || !out_size || (n > 0 && !tris) || interval_count < 2) return -1;
    builder b;
    memset(&b, 0, sizeof(b));
    b.interval_count = interval_count;
    b.subdivide_single_prim = subdivide_single_prim;
    b.max_leaf_prims = max_leaf_prims;
    b.n = n;
    uint32_t ncap = n * 2 < 2 ? 2 : n * 2;
    b.tris = (bvh_triangle_t*)calloc(n ? n : 1, sizeof(bvh_triangle_t));
    b.idx = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    b.centroid = (f3*)calloc(n ? n : 1, sizeof(f3));
    b.nodes = (bvh_node_t*)calloc(ncap, sizeof(bvh_node_t));
    b.bmin = (float*)malloc(sizeof(float) * 3 * interval_count);
    b.bmax = (float*)malloc(sizeof(float) * 3 * interval_count);
    b.bcnt = (uint32_t*)malloc(sizeof(uint32_t) * interval_count);
    b.larea = (float*)malloc(sizeof(float) * interval_count);
    b.rarea = (float*)malloc(sizeof(float) * interval_count);
    for (uint32_t i = 0; i < n; ++i) {
        memcpy(b.tris[i].p0, tris[i].v0.position, 12);
        memcpy(b.tris[i].p1, tris[i].v1.position, 12);
        memcpy(b.tris[i].p2, tris[i].v2.position, 12);
        b.idx[i] = i;
        b.centroid[i] = centroid_of(&b.tris[i]);
    }
    b.nodes[0].left_first = 0;
    b.nodes[0].prim_count = n;
    b.node_at = 2;  /* node 1 stays unused so sibling pairs share a 64-byte line */
    subdivide(&b);

    /* extract (bvh_builder.cpp:52-69) behind the 12-byte header the renderer
     * uploads in front of it (renderer.cpp:113-155). */
    uint64_t nodes_bytes = 32ull * b.node_at, tri_bytes = 36ull * n, idx_bytes = 4ull * n;
    uint64_t size = 12 + nodes_bytes + tri_bytes + idx_bytes;
    uint8_t* blob = (uint8_t*)malloc(size);
    bvh_header_t h;
    h.nodes_offset = 12;
    h.triangles_offset = (uint32_t)(12 + nodes_bytes);
    h.indices_offset = (uint32_t)(12 + nodes_bytes + tri_bytes);
    memcpy(blob, &h, 12);
    memcpy(blob + 12, b.nodes, nodes_bytes);
    if (n) {
        memcpy(blob + h.triangles_offset, b.tris, tri_bytes);
        memcpy(blob + h.indices_offset, b.idx, idx_bytes);
    }
    free(b.tris); free(b.idx); free(b.centroid); free(b.nodes);
    free(b.bmin); free(b.bmax); free(b.bcnt); free(b.larea); free(b.rarea);
    *out_blob = blob;
    *out_size = size;
    return 0;
}

/* find_best_match (tlas_builder.cpp:86-110), including the reference's
 * argument order: the "max" corner is max(A.min, B.min) and the "min" corner
 * is max(A.max, B.max); the metric is half_area of that box. */
static uint32_t best_match(const tlas_node_t* nodes, uint32_t A, const uint32_t* idx, uint32_t count,
                           uint32_t metric) {
    float smallest = FLT_MAX;
    uint32_t best = 0xFFFFFFFFu;
    const tlas_node_t* na = &nodes[idx[A]];
    for (uint32_t B = 0; B < count; ++B) {
        if (B == A) continue;
        const tlas_node_t* nb = &nodes[idx[B]];
        float bmx[3], bmn[3];
        for (int a = 0; a < 3; ++a) {
            if (metric == 0) {
                bmx[a] = gmax(na->aabb_min[a], nb->aabb_min[a]);
                bmn[a] = gmax(na->aabb_max[a], nb->aabb_max[a]);
            } else {
                /* merged box: the metric the reference's comment describes */
                bmn[a] = gmin(na->aabb_min[a], nb->aabb_min[a]);
                bmx[a] = gmax(na->aabb_max[a], nb->aabb_max[a]);
            }
        }
        float area = half_area(bmn, bmx);
        if (area < smallest) { smallest = area; best = B; }
    }
    return best;
}

/* ---- TLAS metric 2: parallel locally-ordered clustering ---------------------
 * (Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding
 * Volume Hierarchy Construction", 2018), the GPU library's fast TLAS build.
 * Instances are ordered by the 30-bit Morton code of their box centres (ties
 * by instance index).  Each round every cluster picks the cluster within
 * PLOC_RADIUS list positions whose merged box has the smallest half area
 * (ties to the lower position); mutual pairs merge into a new node (numbered
 * in list order, left child = the lower position), and the list is compacted
 * in order.  Leaves are nodes 1..n (instance order), the root is copied to 0. */
#ifndef PLOC_RADIUS
#define PLOC_RADIUS 2
#endif

static uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t code = 0;
    for (int b = 0; b < 10; ++b) {
        code |= ((x >> b) & 1u) << (3 * b + 2);
        code |= ((y >> b) & 1u) << (3 * b + 1);
        code |= ((z >> b) & 1u) << (3 * b);
    }
    return code;
}

static uint32_t quantize10(float c, float lo, float ext) {
    float q = (ext > 0.0f) ? (c - lo) / ext : 0.0f;
    if (!(q >= 0.0f)) q = 0.0f;
    if (q > 1.0f) q = 1.0f;
    return (uint32_t)(q * 1023.0f);
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return (x > y) - (x < y);
}

static float merged_half_area(const float* amn, const float* amx, const float* bmn, const float* bmx) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) { lo[a] = gmin(amn[a], bmn[a]); hi[a] = gmax(amx[a], bmx[a]); }
    return half_area(lo, hi);
}

static void tlas_ploc(const bvh_instance_t* inst, uint32_t n, tlas_node_t* nodes) {
    for (uint32_t i = 0; i < n; ++i) {
        memcpy(nodes[1 + i].aabb_min, inst[i].aabb_min, 12);
        memcpy(nodes[1 + i].aabb_max, inst[i].aabb_max, 12);
        nodes[1 + i].instance_idx = i;
        nodes[1 + i].left_right = 0;
    }
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            float c = (inst[i].aabb_min[a] + inst[i].aabb_max[a]) * 0.5f;
            lo[a] = gmin(lo[a], c);
            hi[a] = gmax(hi[a], c);
        }
    float ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * n);
    for (uint32_t i = 0; i < n; ++i) {
        float c[3];
        for (int a = 0; a < 3; ++a) c[a] = (inst[i].aabb_min[a] + inst[i].aabb_max[a]) * 0.5f;
        uint32_t code = morton3(quantize10(c[0], lo[0], ext[0]), quantize10(c[1], lo[1], ext[1]),
                                quantize10(c[2], lo[2], ext[2]));
        key[i] = ((uint64_t)code << 32) | i;
    }
    qsort(key, n, sizeof(uint64_t), cmp_u64);
    uint32_t* cl = (uint32_t*)malloc(sizeof(uint32_t) * n * 2);
    uint32_t* nn = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* ncl = cl + n;
    for (uint32_t k = 0; k < n; ++k) cl[k] = 1 + (uint32_t)(key[k] & 0xFFFFFFFFu);
    uint32_t count = n, next = n + 1;
    while (count > 1) {
        for (uint32_t k = 0; k < count; ++k) {
            const tlas_node_t* a = &nodes[cl[k]];
            uint32_t j0 = k > PLOC_RADIUS ? k - PLOC_RADIUS : 0;
            uint32_t j1 = k + PLOC_RADIUS < count - 1 ? k + PLOC_RADIUS : count - 1;
            float best = FLT_MAX;
            uint32_t bj = (k == 0) ? 1 : k - 1;
            for (uint32_t j = j0; j <= j1; ++j) {
                if (j == k) continue;
                const tlas_node_t* b = &nodes[cl[j]];
                float d = merged_half_area(a->aabb_min, a->aabb_max, b->aabb_min, b->aabb_max);
                if (d < best) { best = d; bj = j; }
            }
            nn[k] = bj;
        }
        uint32_t merges = 0, pos = 0;
        for (uint32_t k = 0; k < count; ++k) merges += (nn[nn[k]] == k && k < nn[k]) ? 1u : 0u;
        int forced = merges == 0;
        if (forced) { nn[0] = 1; nn[1] = 0; merges = 1; }
        uint32_t made = 0;
        for (uint32_t k = 0; k < count; ++k) {
            uint32_t m = nn[k];
            int mutual = nn[m] == k;
            if (mutual && k > m) continue;   /* merged into the lower position */
            if (mutual) {
                uint32_t id = next + made++;
                tlas_node_t* t = &nodes[id];
                const tlas_node_t* a = &nodes[cl[k]];
                const tlas_node_t* b = &nodes[cl[m]];
                for (int ax = 0; ax < 3; ++ax) {
                    t->aabb_min[ax] = gmin(a->aabb_min[ax], b->aabb_min[ax]);
                    t->aabb_max[ax] = gmax(a->aabb_max[ax], b->aabb_max[ax]);
                }
                t->left_right = (cl[k] << 16) | cl[m];
                t->instance_idx = 0;
                ncl[pos++] = id;
            } else {
                ncl[pos++] = cl[k];
            }
        }
        memcpy(cl, ncl, sizeof(uint32_t) * pos);
        count = pos;
        next += made;
    }
    if (n > 0) nodes[0] = nodes[cl[0]];
    free(key);
    free(cl);
    free(nn);
}

/* ---- TLAS metric 3: top-down full-sweep SAH ---------------------------------
 * The GPU library's highest-quality TLAS build (MacDonald and Booth's surface
 * area heuristic, evaluated at every boundary).  Three lists hold the
 * instances ordered by box centre along x, y and z (centre = (min + max) *
 * 0.5, its bits mapped so that unsigned order is float order with -0 below
 * +0; ties by instance index).  A list range [s, e) of two or more instances
 * splits after the position k (s <= k < e - 1) of smallest cost
 * A(s..k) * (k - s + 1) + A(k+1..e-1) * (e - k - 1), A the half area of the
 * range part's union box in float (unions by smin / smax), over the three axes' lists (ties to the
 * lower axis, then the lower k); the other two lists are partitioned stably
 * by side, so a range holds the same instances in all three lists.  Every
 * boundary between list positions is split exactly once, so the interior
 * node of a range split after position k is node n + 1 + k; leaves are nodes
 * 1..n (instance order); the root is copied to node 0. */
static uint32_t sortable_bits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* min / max in the order of sortable_bits (-0 below +0): associative and
 * commutative, so a union box's bits do not depend on the order it is
 * accumulated in (the GPU build scans ranges in warp-sized pieces) */
static inline float smin(float x, float y) { return sortable_bits(y) < sortable_bits(x) ? y : x; }
static inline float smax(float x, float y) { return sortable_bits(x) < sortable_bits(y) ? y : x; }

typedef struct {
    const bvh_instance_t* inst;
    tlas_node_t* nodes;
    uint32_t n;
    uint32_t* list[3];
    uint32_t* tmp;
    uint8_t* left;
    float* pre;    /* 6 floats per position: prefix union box */
    float* cost;   /* per position k: the cost of splitting after k */
} Sweep;

/* Splits list range [s, e) (two or more instances): returns the position k
 * the range splits after, the range's box in mn / mx, and leaves the three
 * lists partitioned. */
static uint32_t sweep_split(Sweep* w, uint32_t s, uint32_t e, float* rmn, float* rmx) {
    float best = FLT_MAX;
    int bax = -1;
    uint32_t bk = s;
    for (int ax = 0; ax < 3; ++ax) {
        const uint32_t* L = w->list[ax];
        float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = s; i < e; ++i) {
            const bvh_instance_t* b = &w->inst[L[i]];
            for (int a = 0; a < 3; ++a) { mn[a] = smin(mn[a], b->aabb_min[a]); mx[a] = smax(mx[a], b->aabb_max[a]); }
            memcpy(&w->pre[6ull * i], mn, 12);
            memcpy(&w->pre[6ull * i + 3], mx, 12);
        }
        if (ax == 0) { memcpy(rmn, mn, 12); memcpy(rmx, mx, 12); }
        /* suffix sweep from the end: the candidate after k pairs prefix k with suffix k + 1 */
        float smn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, smx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = e - 1; i > s; --i) {
            const bvh_instance_t* b = &w->inst[L[i]];
            for (int a = 0; a < 3; ++a) { smn[a] = smin(smn[a], b->aabb_min[a]); smx[a] = smax(smx[a], b->aabb_max[a]); }
            w->cost[i - 1] = half_area(&w->pre[6ull * (i - 1)], &w->pre[6ull * (i - 1) + 3]) * (float)(i - s) +
                             half_area(smn, smx) * (float)(e - i);
        }
        for (uint32_t k = s; k + 1 < e; ++k)
            if (w->cost[k] < best) { best = w->cost[k]; bax = ax; bk = k; }
    }
    if (bax < 0) { bax = 0; bk = s; }   /* no cost below FLT_MAX (not for finite boxes) */
    for (uint32_t i = s; i < e; ++i) w->left[w->list[bax][i]] = (uint8_t)(i <= bk);
    for (int ax = 0; ax < 3; ++ax) {
        if (ax == bax) continue;
        uint32_t* L = w->list[ax];
        uint32_t p = s;
        for (uint32_t i = s; i < e; ++i) if (w->left[L[i]]) w->tmp[p++] = L[i];
        for (uint32_t i = s; i < e; ++i) if (!w->left[L[i]]) w->tmp[p++] = L[i];
        memcpy(&L[s], &w->tmp[s], sizeof(uint32_t) * (e - s));
    }
    return bk;
}

static void tlas_sweep(const bvh_instance_t* inst, uint32_t n, tlas_node_t* nodes) {
    for (uint32_t i = 0; i < n; ++i) {
        memcpy(nodes[1 + i].aabb_min, inst[i].aabb_min, 12);
        memcpy(nodes[1 + i].aabb_max, inst[i].aabb_max, 12);
        nodes[1 + i].instance_idx = i;
        nodes[1 + i].left_right = 0;
    }
    if (n == 0) return;
    Sweep w;
    w.inst = inst;
    w.nodes = nodes;
    w.n = n;
    uint64_t* key = (uint64_t*)malloc(sizeof(uint64_t) * n);
    for (int ax = 0; ax < 3; ++ax) {
        for (uint32_t i = 0; i < n; ++i) {
            const float c = (inst[i].aabb_min[ax] + inst[i].aabb_max[ax]) * 0.5f;
            key[i] = ((uint64_t)sortable_bits(c) << 32) | i;
        }
        qsort(key, n, sizeof(uint64_t), cmp_u64);
        w.list[ax] = (uint32_t*)malloc(sizeof(uint32_t) * n);
        for (uint32_t i = 0; i < n; ++i) w.list[ax][i] = (uint32_t)(key[i] & 0xFFFFFFFFu);
    }
    w.tmp = (uint32_t*)malloc(sizeof(uint32_t) * n);
    w.left = (uint8_t*)malloc(n);
    w.pre = (float*)malloc(sizeof(float) * 6 * n);
    w.cost = (float*)malloc(sizeof(float) * n);
    /* ranges to split: (s, e, parent node, 0 = left / 1 = right child); an
     * explicit stack, since a range can be as deep as it is long */
    uint32_t* task = (uint32_t*)malloc(sizeof(uint32_t) * 4 * n);
    uint32_t top = 0, root = 1;
    task[0] = 0; task[1] = n; task[2] = 0; task[3] = 2;
    top = 1;
    while (top) {
        --top;
        const uint32_t s = task[4 * top], e = task[4 * top + 1], parent = task[4 * top + 2], slot = task[4 * top + 3];
        uint32_t id;
        if (e - s == 1) {
            id = 1 + w.list[0][s];
        } else {
            float mn[3], mx[3];
            const uint32_t k = sweep_split(&w, s, e, mn, mx);
            id = n + 1 + k;
            tlas_node_t* t = &nodes[id];
            memcpy(t->aabb_min, mn, 12);
            memcpy(t->aabb_max, mx, 12);
            t->left_right = 0;
            t->instance_idx = 0;
            /* right range below the left one: the left is taken first */
            task[4 * top] = k + 1; task[4 * top + 1] = e; task[4 * top + 2] = id; task[4 * top + 3] = 1;
            ++top;
            task[4 * top] = s; task[4 * top + 1] = k + 1; task[4 * top + 2] = id; task[4 * top + 3] = 0;
            ++top;
        }
        if (slot == 2) root = id;
        else nodes[parent].left_right |= (slot == 0) ? (id << 16) : id;
    }
    nodes[0] = nodes[root];
    for (int ax = 0; ax < 3; ++ax) free(w.list[ax]);
    free(w.tmp);
    free(w.left);
    free(w.pre);
    free(w.cost);
    free(task);
    free(key);
}

/* tlas_builder_t::build + extract (tlas_builder.cpp:6-84).  The reference's
 * working list is a 256-entry stack array (:14); this one is sized to n.
 * metric 0 is the reference's pairing metric; metric 1 replaces it by the
 * half area of the merged box (same walk, same tie rule). */
int orc_tlas_build_metric(const bvh_instance_t* inst, uint32_t n, uint32_t metric, uint8_t** out_blob,
                          uint64_t* out_size) {
    if (!out_blob || !out_size || (n > 0 && !inst) || n > 32768 || metric > 3) return -1;
    uint32_t ncount = n * 2;
    tlas_node_t* nodes = (tlas_node_t*)calloc(ncount ? ncount : 1, sizeof(tlas_node_t));
    uint32_t* idx = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    uint32_t remaining = n, at = 1;
    for (uint32_t i = 0; i < n; ++i) {
        idx[i] = at;
        memcpy(nodes[at].aabb_min, inst[i].aabb_min, 12);
        memcpy(nodes[at].aabb_max, inst[i].aabb_max, 12);
        nodes[at].instance_idx = i;
        nodes[at].left_right = 0;
        at++;
    }
    if (metric == 2 || metric == 3) {
        if (metric == 2) tlas_ploc(inst, n, nodes);
        else tlas_sweep(inst, n, nodes);
        at = n ? 2 * n : 1;
    } else if (n > 0) {
        uint32_t A = 0;
        uint32_t B = best_match(nodes, A, idx, remaining, metric);
        while (remaining > 1) {
            uint32_t C = best_match(nodes, B, idx, remaining, metric);
            if (A == C) {
                uint32_t ia = idx[A], ib = idx[B];
                tlas_node_t* nn = &nodes[at];
                nn->left_right = ia + (ib << 16);
                for (int a = 0; a < 3; ++a) {
                    nn->aabb_min[a] = gmin(nodes[ia].aabb_min[a], nodes[ib].aabb_min[a]);
                    nn->aabb_max[a] = gmax(nodes[ia].aabb_max[a], nodes[ib].aabb_max[a]);
                }
                idx[A] = at++;
                idx[B] = idx[remaining - 1];
                B = best_match(nodes, A, idx, --remaining, metric);
            } else {
                A = B;
                B = C;
            }
        }
        nodes[0] = nodes[idx[A]];
    }
    uint64_t nodes_bytes = 32ull * at, inst_bytes = 92ull * n;
    uint64_t size = 8 + nodes_bytes + inst_bytes;
    uint8_t* blob = (uint8_t*)malloc(size);
    tlas_header_t h;
    h.nodes_offset = 8;
    h.instances_offset = (uint32_t)(8 + nodes_bytes);
    memcpy(blob, &h, 8);
    memcpy(blob + 8, nodes, nodes_bytes);
    if (n) memcpy(blob + h.instances_offset, inst, inst_bytes);
    free(nodes); free(idx);
    *out_blob = blob;
    *out_size = size;
    return 0;
}

int orc_tlas_build(const bvh_instance_t* inst, uint32_t n, uint8_t** out_blob, uint64_t* out_size) {
    return orc_tlas_build_metric(inst, n, 0, out_blob, out_size);
}

void orc_free(void* p) { free(p); }
