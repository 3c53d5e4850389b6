// wf_batch.cu — batched rendering of many independent scenes (wf_batch_* in
// include/wf.h; no counterpart in the reference, whose renderer draws one scene).
//
// Design.  All scenes share one pool of paths in flight (capacity entries).
// Every pool entry carries its scene id, so scenes of very different sizes
// keep one set of queues busy instead of each scene owning a fixed, mostly
// idle segment.  One iteration of the pipeline is
//     begin      (1 thread)  decide how many new camera paths to admit
//     regenerate             admit them: camera rays appended to the queue
//     extend                 closest hit of every queued ray (persistent traversal)
//     shade                  shade_one(), the single-scene shading arithmetic;
//                            continuing paths go to the other queue, finished
//                            paths store their radiance, shadow rays queue up
//     connect                any-hit shadow rays add their contribution
//     end        (1 thread)  loop bookkeeping and the loop condition
// Every stage reads its sizes from a control block in device memory, so the
// host records the iterations once: four iterations (queues A -> B -> A -> B
// -> A) form the body of a CUDA-graph while-loop whose condition the last
// kernel sets, and one graph launch renders the whole batch.  Each connect
// runs on a second stream beside the next iteration's begin / regenerate /
// extend (shadow queues, counts and hand-out counters alternate by iteration
// parity); the next shade waits for it.
//
// Camera paths are numbered scene by scene, pixel-major inside a scene
// (path = path_base + pixel * spp + sample, so a pixel's identical camera rays
// share a warp), and admitted in that order.  A
// path's random numbers are keyed by (scene-local pixel, sample, depth) as in
// wf_render, its radiance is summed in the same order, and each finished path
// stores its radiance at its own index; the resolve adds a pixel's samples in
// sample order.  A scene's image therefore equals wf_render's image of the same
// scene bit for bit, whatever the pool size, threshold or interleaving.
//
// Termination.  Every path ends within max_bounces + 1 iterations of its
// admission, so an iteration in which no path ends can repeat at most
// max_bounces + 1 times; the end kernel stops the loop with ERRF_TIMEOUT if
// that bound is ever exceeded, which keeps the device-side loop finite even
// if an invariant were broken.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "wf_ctx.h"
#include "wf_shade.cuh"
#include "wf_traverse.cuh"

namespace wf {
namespace {

constexpr uint32_t kSceneShift = 16;       // queue flags word: bits 0-7 path flags, 8-15 depth, 16-31 scene
constexpr uint32_t kDepthShift = 8;
constexpr uint32_t kFinishedBit = 0x80000000u;  // shadow target: radiance slot of a finished path
constexpr int kBodyIterations = 4;              // iterations per graph-loop body (even: queues alternate)

struct BatchScene {
    float4 clip_to_view[4];
    float4 view_to_world[4];
    float dim_x, dim_y;
    uint32_t width, np;            // np = width * height
    uint32_t spp, path_base, pix_base, root;   // root: TLAS root node, kInvalid = no instances
    uint32_t light_off, light_count;
    float light_total, env_strength;
    float env[3];
    uint32_t frame_seed;
    uint32_t max_bounces, nee, rr_start, cosine;
    TexRef env_tex;                // texels null: constant env
};
static_assert(sizeof(BatchScene) == 224, "BatchScene layout");

// Pool entry i of queue k: qo {origin, flags word}, qd {direction, pixel},
// qT {throughput, pdf of the last BSDF sample}, qL {radiance, sample}.
struct BatchQueues {
    float4* qo[2];
    float4* qd[2];
    float4* qT[2];
    float4* qL[2];
    float4* h_tuvp;
    uint32_t* h_inst;
    float4* s_o[2];   // by iteration parity: {origin, tmax}
    float4* s_d[2];   // {direction, target}: pool slot of the continuing path, or kFinishedBit | camera path
    float4* s_c[2];   // {contribution, scene}
    float4* out_L;    // per camera path: its radiance
    // checked builds: bounds of the pool, the camera paths and the scene ids
    uint32_t capacity, total_paths, nscenes;
    uint32_t* status;
};

struct BatchCtl {
    uint32_t count[2];        // entries in queue k
    uint32_t shadow[2];       // shadow rays of the iteration on queue k
    uint32_t fetch[3];        // persistent traversal hand-out counters: extend, connect on queue 0 / 1
    uint32_t regen_n, regen_g0, regen_slot0;
    uint32_t next, total;     // next camera path to admit, number of camera paths
    uint32_t capacity, threshold;
    uint32_t iter, stall, stall_limit, done, body_runs;
    uint32_t max_iter;        // hard bound on iterations (a loose upper bound of a correct run)
    unsigned long long rays_ext, rays_con;
};

__device__ __forceinline__ uint32_t scene_of(const uint32_t* base, uint32_t ns, uint32_t g) {
    uint32_t lo = 0, hi = ns - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (base[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_bbegin(BatchCtl* c, int cur) {
    const uint32_t n = c->done ? 0u : c->count[cur];
    uint32_t take = 0;
    if (!c->done) {
        const uint32_t rem = c->total - c->next;
        if (rem && n < c->threshold) take = min(rem, c->capacity - n);
    }
    c->count[cur] = n + take;
    c->regen_n = take;
    c->regen_g0 = c->next;
    c->regen_slot0 = n;
    c->next += take;
    c->count[cur ^ 1] = 0;
    c->shadow[cur] = 0;
    c->fetch[0] = 0;
    c->fetch[1 + cur] = 0;   // the other parity's connect may still be running
    c->rays_ext += n + take;
}

// generate.hlsl:12-20 for the admitted camera paths (clear_buffers.hlsl's
// path-state reset is the entry's initial throughput / radiance).
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_bregen(const BatchScene* sc, const uint32_t* pbase, uint32_t ns,
                                                  BatchQueues Q, const BatchCtl* c, int cur) {
    const uint32_t m = c->regen_n, g0 = c->regen_g0, s0 = c->regen_slot0;
    // queue pointers picked by selects: a dynamic index into the parameter
    // arrays would copy them to local memory
    float4* const qo = cur ? Q.qo[1] : Q.qo[0];
    float4* const qd = cur ? Q.qd[1] : Q.qd[0];
    float4* const qT = cur ? Q.qT[1] : Q.qT[0];
    float4* const qL = cur ? Q.qL[1] : Q.qL[0];
    for (uint32_t j = blockIdx.x * BLOCK + threadIdx.x; j < m; j += gridDim.x * BLOCK) {
        const uint32_t g = g0 + j;
        if (!in_bounds(s0 + j, Q.capacity, Q.status) || !in_bounds(g, Q.total_paths, Q.status)) continue;
        const uint32_t s = scene_of(pbase, ns, g);
        const BatchScene& S = sc[s];
        const uint32_t local = g - S.path_base;
        const uint32_t pixel = local / S.spp, sample = local - pixel * S.spp;
        V3 o, d;
        primary_ray(S, pixel % S.width, pixel / S.width, o, d);
        const uint32_t slot = s0 + j;
        qo[slot] = make_float4(o.x, o.y, o.z, __uint_as_float(kFlagSpecular | (s << kSceneShift)));
        qd[slot] = make_float4(d.x, d.y, d.z, __uint_as_float(pixel));
        qT[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        qL[slot] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(sample));
    }
}

struct BatchExtendIO {
    const float4* qo;
    const float4* qd;
    float4* tuvp;
    uint32_t* inst;
    const uint32_t* roots;
    uint32_t nscenes;    // checked builds
    uint32_t* status;
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        const float4 a = qo[i], b = qd[i];
        o = xyz(a); d = xyz(b); tmax = FLT_MAX;
        nc = (__float_as_uint(a.w) & kFlagInside) != 0u;
    }
    __device__ __forceinline__ uint32_t root(uint32_t i, const SceneRefs&) const {
        const uint32_t scene = __float_as_uint(qo[i].w) >> kSceneShift;
        return in_bounds(scene, nscenes, status) ? roots[scene] : kInvalid;
    }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool) const {
        tuvp[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        inst[i] = h.inst;
    }
};

struct BatchConnectIO {
    const float4* so;
    const float4* sd;
    const float4* sc;
    const uint32_t* roots;
    uint32_t nscenes, capacity, total_paths;   // checked builds
    uint32_t* status;
    float4* qL;       // radiance of the continuing paths (the next queue)
    float4* out_L;    // radiance of finished camera paths
    __device__ __forceinline__ void load(uint32_t i, V3& o, V3& d, float& tmax, bool& nc) const {
        const float4 a = so[i], b = sd[i];
        o = xyz(a); d = xyz(b); tmax = a.w; nc = false;
    }
    __device__ __forceinline__ uint32_t root(uint32_t i, const SceneRefs&) const {
        const uint32_t scene = __float_as_uint(sc[i].w);
        return in_bounds(scene, nscenes, status) ? roots[scene] : kInvalid;
    }
    __device__ __forceinline__ void store(uint32_t i, const Hit& h, bool ok) const {
        if (!ok || h.inst != kInvalid) return;
        const float4 k = sc[i];
        const uint32_t t = __float_as_uint(sd[i].w);
        if ((t & kFinishedBit) ? !in_bounds(t & ~kFinishedBit, total_paths, status) : !in_bounds(t, capacity, status))
            return;
        float4* dst = (t & kFinishedBit) ? out_L + (t & ~kFinishedBit) : qL + t;
        float4 acc = *dst;
        acc.x = acc.x + k.x;
        acc.y = acc.y + k.y;
        acc.z = acc.z + k.z;
        *dst = acc;
    }
};

template <bool ANY, class IO>
__global__ void __launch_bounds__(kTraceBlock, WF_TRACE_MIN_BLOCKS) k_btrace(SceneRefs S, IO io, const uint32_t* count, uint32_t* fetch,
                                                        uint32_t* status) {
    const uint32_t n = *count;
    if (n == 0) return;
    LocalCounters lc = {0, 0, 0, 0};
    bool overflow = false;
    trace_persistent<ANY, false, 0>(S, io, n, fetch, lc, overflow);   // the binary BLAS layout
    if (overflow) atomicOr(status, ERRF_STACK);
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_bshade(ShadeRefs SH, const BatchScene* sc, BatchQueues Q, BatchCtl* c,
                                                  int cur) {
    const uint32_t n = c->count[cur];
    const AdjointRefs none = {nullptr, nullptr, nullptr, nullptr, 0.0f, 1u, 0u};
    const float4* const qo = cur ? Q.qo[1] : Q.qo[0];
    const float4* const qd = cur ? Q.qd[1] : Q.qd[0];
    const float4* const qT = cur ? Q.qT[1] : Q.qT[0];
    const float4* const qL = cur ? Q.qL[1] : Q.qL[0];
    float4* const no = cur ? Q.qo[0] : Q.qo[1];
    float4* const nd = cur ? Q.qd[0] : Q.qd[1];
    float4* const nT = cur ? Q.qT[0] : Q.qT[1];
    float4* const nL = cur ? Q.qL[0] : Q.qL[1];
    uint32_t* const ncount = cur ? &c->count[0] : &c->count[1];
    uint32_t* const shadow_tail = cur ? &c->shadow[1] : &c->shadow[0];
    float4* const s_o = cur ? Q.s_o[1] : Q.s_o[0];
    float4* const s_d = cur ? Q.s_d[1] : Q.s_d[0];
    float4* const s_c = cur ? Q.s_c[1] : Q.s_c[0];
    for (uint32_t base = blockIdx.x * BLOCK; base < n; base += gridDim.x * BLOCK) {
        const uint32_t i = base + threadIdx.x;
        ShadeOut o;
        o.enqueue = false; o.shadow = false;
        uint32_t scene = 0, depth = 0, pixel = 0, gidx = 0;
        float4 L4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (i < n) {
            const float4 a = qo[i], b = qd[i], T4 = qT[i];
            L4 = qL[i];
            const uint32_t f = __float_as_uint(a.w);
            scene = f >> kSceneShift;
            if (!in_bounds(scene, Q.nscenes, Q.status)) scene = 0u;   // checked builds: flagged, scene 0 stands in
            depth = (f >> kDepthShift) & 0xFFu;
            pixel = __float_as_uint(b.w);
            const BatchScene& S = sc[scene];
            ShadeCtl K;
            K.frame_seed = S.frame_seed; K.max_bounces = S.max_bounces; K.nee = S.nee; K.rr_start = S.rr_start;
            K.cosine = S.cosine; K.env_strength = S.env_strength;
            K.env0 = S.env[0]; K.env1 = S.env[1]; K.env2 = S.env[2];
            K.lights = SH.lights + S.light_off; K.light_count = S.light_count; K.light_total = S.light_total;
            K.env_tex = S.env_tex; K.view_mode = 0u; K.far_plane = 1.0f;
            ShadeIn in;
            in.rd = xyz(b);
            in.tuvp = Q.h_tuvp[i];
            in.inst = Q.h_inst[i];
            in.T = xyz(T4);
            in.last_pdf = T4.w;
            in.flags = f & 0xFFu;
            in.pixel = pixel;
            in.sample = __float_as_uint(L4.w);
            in.depth = depth;
            shade_one(SH, K, in, none, 0u, 0u, o);
            if (o.has_add) {
                L4.x = L4.x + o.add.x;
                L4.y = L4.y + o.add.y;
                L4.z = L4.z + o.add.z;
            }
            if (!o.enqueue) {
                gidx = S.path_base + pixel * S.spp + in.sample;
                if (in_bounds(gidx, Q.total_paths, Q.status)) Q.out_L[gidx] = L4;
            }
        }
        const uint32_t slot = warp_append(ncount, o.enqueue);
        if (o.enqueue && in_bounds(slot, Q.capacity, Q.status)) {
            const uint32_t f = (o.flags & 0xFFu) | ((depth + 1u) << kDepthShift) | (scene << kSceneShift);
            no[slot] = make_float4(o.org.x, o.org.y, o.org.z, __uint_as_float(f));
            nd[slot] = make_float4(o.dir.x, o.dir.y, o.dir.z, __uint_as_float(pixel));
            nT[slot] = make_float4(o.T.x, o.T.y, o.T.z, o.pdf);
            nL[slot] = L4;
        }
        const uint32_t sslot = warp_append(shadow_tail, o.shadow);
        if (o.shadow && in_bounds(sslot, Q.capacity, Q.status)) {
            const uint32_t target = o.enqueue ? slot : (kFinishedBit | gidx);
            s_o[sslot] = make_float4(o.spos.x, o.spos.y, o.spos.z, o.stmax);
            s_d[sslot] = make_float4(o.sdir.x, o.sdir.y, o.sdir.z, __uint_as_float(target));
            s_c[sslot] = make_float4(o.contrib.x, o.contrib.y, o.contrib.z, __uint_as_float(scene));
        }
    }
}

__global__ void k_bend(BatchCtl* c, int cur, uint32_t* status, cudaGraphConditionalHandle h, int set_cond) {
    if (!c->done) {
        c->iter++;
        c->rays_con += c->shadow[cur];
        const uint32_t n = c->count[cur], m = c->count[cur ^ 1];
        c->stall = (n > 0u && m >= n) ? c->stall + 1u : 0u;   // m >= n: no path ended
        if (c->stall > c->stall_limit || c->iter >= c->max_iter) {
            atomicOr(status, ERRF_TIMEOUT);
            c->done = 1;
        }
        if (m == 0u && c->next >= c->total) c->done = 1;
        c->count[cur] = 0;   // queue cur is consumed: its paths continued into the other queue or finished
    }
    if (set_cond) {
        c->body_runs++;
        cudaGraphSetConditional(h, c->done ? 0u : 1u);
    }
}

// A pixel's samples in sample order: the sum wf_render's accumulator holds,
// then k_resolve's division.
__global__ void k_bresolve(const BatchScene* sc, const uint32_t* pixbase, uint32_t ns, const float4* out_L,
                           float4* image, uint32_t npix) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < npix; q += gridDim.x * blockDim.x) {
        const uint32_t s = scene_of(pixbase, ns, q);
        const BatchScene& S = sc[s];
        const uint32_t p = q - S.pix_base;
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (uint32_t k = 0; k < S.spp; ++k) {
            const float4 L = out_L[(size_t)S.path_base + (size_t)p * S.spp + k];
            acc.x = acc.x + L.x;
            acc.y = acc.y + L.y;
            acc.z = acc.z + L.z;
            acc.w = acc.w + 1.0f;
        }
        image[q] = acc.w > 0.0f ? make_float4(acc.x / acc.w, acc.y / acc.w, acc.z / acc.w, acc.w)
                                : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// Instance rows of one scene's TLAS, built with local indices at node base
// 2 * inst_base, rebased to the batch-wide node and instance arrays.
__global__ void k_tlas_rebase(float4* nodes, uint32_t node_count, uint32_t node_base, uint32_t inst_base) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < node_count; k += gridDim.x * blockDim.x) {
        float4 a = nodes[2ull * k], b = nodes[2ull * k + 1];
        const uint32_t lr = __float_as_uint(a.w);
        if (lr != 0u) {
            const uint32_t l = (lr >> 16) + node_base, r = (lr & 0xFFFFu) + node_base;
            a.w = __uint_as_float((l << 16) | r);
            nodes[2ull * k] = a;
        } else {
            b.w = __uint_as_float(__float_as_uint(b.w) + inst_base);
            nodes[2ull * k + 1] = b;
        }
    }
}

// ---------------------------------------------------------------------------- host

#define BCUDA(call)                                                                                   \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return fail_code(e_ == cudaErrorMemoryAllocation ? WF_ERR_OOM : WF_ERR_CUDA,              \
                             std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t cap = 0;
    int reserve(size_t n) {
        if (n == 0) n = 1;
        if (n <= cap && p) return WF_OK;
        release();
        if (dmalloc(reinterpret_cast<void**>(&p), n * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return fail_code(WF_ERR_OOM, "wf_batch: device allocation of " + std::to_string(n * sizeof(T)) +
                                             " bytes failed");
        }
        cap = n;
        return WF_OK;
    }
    void release() {
        if (p) dfree(p);
        p = nullptr;
        cap = 0;
    }
};

struct HostScene {
    uint32_t width, height, spp;
    view_t view;
    float env[3];
    uint32_t env_texture;
    std::vector<Instance> inst;
};

bool valid_block(uint32_t b) { return b == 128 || b == 256 || b == 512; }

}  // namespace
}  // namespace wf

using namespace wf;

struct wf_batch {
    wf_ctx* ctx = nullptr;
    std::vector<HostScene> scenes;
    bool in_scene = false;
    bool tables_ready = false;
    wf_batch_config cfg{};

    // batch-wide scene tables
    uint32_t nscenes = 0, total_paths = 0, total_pixels = 0, total_inst = 0;
    std::vector<uint32_t> light_off, light_cnt, roots;
    std::vector<float> light_total;
    DBuf<float4> tnodes, tinst, sinst;
    DBuf<float> aabbs;
    DBuf<uint32_t> tlas_scratch, d_roots, d_pbase, d_pixbase;
    DBuf<LightTri> lights;
    DBuf<BlasRef> blas;
    DBuf<const float4*> stri;
    DBuf<BatchScene> d_scenes;
    DBuf<float4> out_L, image;

    // pool (capacity dependent)
    uint32_t pool_cap = 0;
    uint32_t pool_block = 0;
    DBuf<float4> q[8];
    DBuf<float4> h_tuvp, s_o[2], s_d[2], s_c[2];
    DBuf<uint32_t> h_inst;
    BatchCtl* ctl = nullptr;
    BatchCtl* ctl_host = nullptr;   // pinned

    // graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graph_valid = false;

    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaStream_t side = nullptr;                         // the connect stage
    cudaEvent_t ev_shade[kBodyIterations] = {}, ev_conn[kBodyIterations] = {};
    wf_batch_stats stats{};
    uint64_t host_launches = 0;
    bool rendered = false;
};

namespace {

void drop_graph(wf_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_valid = false;
}

void default_config(wf_batch_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->capacity = 1u << 21;
    c->regen_threshold = 1.0f;
    c->block = 256;
    c->use_graph = 1;
}

int check_config(const wf_batch_config* in, wf_batch_config* out) {
    wf_batch_config c = *in;
    if (c.capacity == 0) c.capacity = 1u << 21;
    if (c.regen_threshold == 0.0f) c.regen_threshold = 1.0f;
    if (c.block == 0) c.block = 256;
    if (c.capacity < 1024 || c.capacity > (1u << 27))
        return fail_code(WF_ERR_INVALID, "wf_batch config: capacity must be in [1024, 2^27]");
    if (!(c.regen_threshold > 0.0f && c.regen_threshold <= 1.0f))
        return fail_code(WF_ERR_INVALID, "wf_batch config: regen_threshold must be in (0, 1]");
    if (!valid_block(c.block)) return fail_code(WF_ERR_INVALID, "wf_batch config: block must be 128, 256 or 512");
    if (c.use_graph > 1) return fail_code(WF_ERR_INVALID, "wf_batch config: use_graph must be 0 or 1");
    *out = c;
    return WF_OK;
}

// Scene tables: instances, per-scene TLAS (rebased), emitters, path and pixel bases.
int build_tables(wf_batch* b) {
    wf_ctx* c = b->ctx;
    cudaStream_t st = ctx_stream(c);
    const uint32_t ns = (uint32_t)b->scenes.size();
    uint64_t paths = 0, pixels = 0, inst = 0;
    for (const HostScene& s : b->scenes) {
        paths += (uint64_t)s.width * s.height * s.spp;
        pixels += (uint64_t)s.width * s.height;
        inst += s.inst.size();
    }
    if (paths >= (1ull << 31)) return fail_code(WF_ERR_CAPACITY, "wf_batch: more than 2^31 - 1 camera paths");
    if (2 * inst > 65536) return fail_code(WF_ERR_CAPACITY, "wf_batch: more than 32768 instances over all scenes");
    b->nscenes = ns;
    b->total_paths = (uint32_t)paths;
    b->total_pixels = (uint32_t)pixels;
    b->total_inst = (uint32_t)inst;
    // mesh tables (every mesh of the context, by mesh id)
    const uint32_t nm = ctx_mesh_count(c);
    std::vector<BlasRef> br(nm ? nm : 1);
    std::vector<const float4*> sp(nm ? nm : 1);
    for (uint32_t i = 0; i < nm; ++i) {
        MeshView mv;
        ctx_mesh(c, i, &mv);
        br[i].nodes = mv.d_nodes;
        br[i].tris = mv.d_tris;
        br[i].node_count = mv.node_count;
        br[i].tri_count = mv.tri_count;
        sp[i] = mv.d_stri;
    }
    int rc;
    if ((rc = b->blas.reserve(br.size())) || (rc = b->stri.reserve(sp.size()))) return rc;
    BCUDA(ctx_h2d(c, b->blas.p, br.data(), br.size() * sizeof(BlasRef)));
    BCUDA(ctx_h2d(c, b->stri.p, sp.data(), sp.size() * sizeof(void*)));
    // instances
    const uint32_t ni = b->total_inst;
    std::vector<float4> ti(4ull * ni), si((size_t)kInstRows * ni);
    std::vector<float> ab(6ull * ni);
    std::vector<LightTri> lt;
    b->light_off.assign(ns, 0);
    b->light_cnt.assign(ns, 0);
    b->light_total.assign(ns, 0.0f);
    b->roots.assign(ns, kInvalid);
    std::vector<uint32_t> ibase(ns, 0), pbase(ns + 1, 0), pixbase(ns + 1, 0);
    uint32_t k = 0;
    for (uint32_t s = 0; s < ns; ++s) {
        const HostScene& H = b->scenes[s];
        ibase[s] = k;
        b->light_off[s] = (uint32_t)lt.size();
        float run = 0.0f;
        for (const Instance& in : H.inst) {
            instance_rows(in, &ti[4ull * k], &si[(size_t)kInstRows * k], &ab[6ull * k]);
            MeshView mv;
            ctx_mesh(c, in.mesh, &mv);
            append_emitters(in, k, mv, lt, run);
            ++k;
        }
        b->light_cnt[s] = (uint32_t)lt.size() - b->light_off[s];
        b->light_total[s] = run;
        if (!H.inst.empty()) b->roots[s] = 2u * ibase[s];
        pbase[s + 1] = pbase[s] + H.width * H.height * H.spp;
        pixbase[s + 1] = pixbase[s] + H.width * H.height;
    }
    if ((rc = b->tnodes.reserve(4ull * std::max<uint32_t>(ni, 1))) || (rc = b->tinst.reserve(ti.size())) ||
        (rc = b->sinst.reserve(si.size())) || (rc = b->aabbs.reserve(ab.size())) ||
        (rc = b->tlas_scratch.reserve(tlas_scratch_words(ni, ctx_tlas_metric(c)))) || (rc = b->lights.reserve(lt.size())) ||
        (rc = b->d_roots.reserve(ns)) || (rc = b->d_pbase.reserve(ns + 1)) || (rc = b->d_pixbase.reserve(ns + 1)) ||
        (rc = b->d_scenes.reserve(ns)) || (rc = b->out_L.reserve(b->total_paths)) ||
        (rc = b->image.reserve(b->total_pixels)))
        return rc;
    if (ni) {
        BCUDA(ctx_h2d(c, b->tinst.p, ti.data(), ti.size() * 16));
        BCUDA(ctx_h2d(c, b->sinst.p, si.data(), si.size() * 16));
        BCUDA(ctx_h2d(c, b->aabbs.p, ab.data(), ab.size() * 4));
    }
    if (!lt.empty()) BCUDA(ctx_h2d(c, b->lights.p, lt.data(), lt.size() * sizeof(LightTri)));
    BCUDA(ctx_h2d(c, b->d_roots.p, b->roots.data(), ns * 4));
    BCUDA(ctx_h2d(c, b->d_pbase.p, pbase.data(), (ns + 1) * 4));
    BCUDA(ctx_h2d(c, b->d_pixbase.p, pixbase.data(), (ns + 1) * 4));
    const uint32_t metric = ctx_tlas_metric(c);
    for (uint32_t s = 0; s < ns; ++s) {
        const uint32_t n = (uint32_t)b->scenes[s].inst.size();
        if (n == 0) continue;
        float4* nodes = b->tnodes.p + 4ull * ibase[s];
        BCUDA(launch_tlas_build(b->aabbs.p + 6ull * ibase[s], n, nodes, b->tlas_scratch.p, metric, st));
        k_tlas_rebase<<<(2 * n + 127) / 128, 128, 0, st>>>(nodes, 2 * n, 2 * ibase[s], ibase[s]);
        BCUDA(cudaGetLastError());
    }
    BCUDA(cudaStreamSynchronize(st));
    b->tables_ready = true;
    drop_graph(b);
    return WF_OK;
}

int ensure_pool(wf_batch* b) {
    const uint32_t C = b->cfg.capacity;
    if (b->pool_cap == C && b->ctl) return WF_OK;
    drop_graph(b);
    int rc;
    for (int k = 0; k < 8; ++k)
        if ((rc = b->q[k].reserve(C))) return rc;
    if ((rc = b->h_tuvp.reserve(C)) || (rc = b->h_inst.reserve(C))) return rc;
    for (int k = 0; k < 2; ++k)
        if ((rc = b->s_o[k].reserve(C)) || (rc = b->s_d[k].reserve(C)) || (rc = b->s_c[k].reserve(C))) return rc;
    if (!b->ctl) {
        if (dmalloc(reinterpret_cast<void**>(&b->ctl), sizeof(BatchCtl)) != cudaSuccess) {
            cudaGetLastError();
            b->ctl = nullptr;
            return fail_code(WF_ERR_OOM, "wf_batch: control block allocation failed");
        }
        if (cudaMallocHost(&b->ctl_host, sizeof(BatchCtl)) != cudaSuccess) {
            cudaGetLastError();
            b->ctl_host = nullptr;
            return fail_code(WF_ERR_OOM, "wf_batch: pinned control block allocation failed");
        }
    }
    b->pool_cap = C;
    return WF_OK;
}

BatchQueues queues(wf_batch* b) {
    BatchQueues Q;
    for (int k = 0; k < 2; ++k) {
        Q.qo[k] = b->q[4 * k].p;
        Q.qd[k] = b->q[4 * k + 1].p;
        Q.qT[k] = b->q[4 * k + 2].p;
        Q.qL[k] = b->q[4 * k + 3].p;
    }
    Q.h_tuvp = b->h_tuvp.p;
    Q.h_inst = b->h_inst.p;
    for (int k = 0; k < 2; ++k) {
        Q.s_o[k] = b->s_o[k].p;
        Q.s_d[k] = b->s_d[k].p;
        Q.s_c[k] = b->s_c[k].p;
    }
    Q.out_L = b->out_L.p;
    Q.capacity = b->cfg.capacity;
    Q.total_paths = b->total_paths;
    Q.nscenes = b->nscenes;
    Q.status = ctx_status(b->ctx);
    return Q;
}

unsigned stage_grid(uint32_t block) { return (unsigned)sm_count() * (2048u / block); }

template <int BLOCK>
cudaError_t launch_regen_shade(bool shade, wf_batch* b, const ShadeRefs& SH, const BatchQueues& Q, int cur,
                               cudaStream_t st) {
    if (shade) k_bshade<BLOCK><<<stage_grid(BLOCK), BLOCK, 0, st>>>(SH, b->d_scenes.p, Q, b->ctl, cur);
    else k_bregen<BLOCK><<<stage_grid(BLOCK), BLOCK, 0, st>>>(b->d_scenes.p, b->d_pbase.p, b->nscenes, Q, b->ctl, cur);
    return cudaGetLastError();
}

cudaError_t regen_or_shade(bool shade, wf_batch* b, const ShadeRefs& SH, const BatchQueues& Q, int cur,
                           cudaStream_t st) {
    switch (b->cfg.block) {
        case 128: return launch_regen_shade<128>(shade, b, SH, Q, cur, st);
        case 512: return launch_regen_shade<512>(shade, b, SH, Q, cur, st);
        default: return launch_regen_shade<256>(shade, b, SH, Q, cur, st);
    }
}

// Iteration k of a group (queue cur = k & 1; 6 kernels).  Its connect goes to
// the side stream; its shade first waits for the previous iteration's connect
// (join_prev), and the last iteration of a group joins its own connect before
// its end kernel (join_self).  set_cond: the end kernel sets the graph loop's
// condition.
int enqueue_iteration(wf_batch* b, int k, bool join_prev, bool join_self, cudaGraphConditionalHandle h,
                      bool set_cond) {
    const int cur = k & 1;
    cudaStream_t st = ctx_stream(b->ctx);
    uint32_t* status = ctx_status(b->ctx);
    const BatchQueues Q = queues(b);
    SceneRefs S;
    S.tnodes = b->tnodes.p;
    S.tinst = b->tinst.p;
    S.blas = b->blas.p;
    S.inst_count = b->total_inst;
    S.tnode_count = 2u * b->total_inst;
    S.mesh_count = ctx_mesh_count(b->ctx);
    S.status = status;
    ShadeRefs SH;
    SH.sinst = b->sinst.p;
    SH.stri = b->stri.p;
    SH.lights = b->lights.p;
    SH.light_count = 0;
    SH.light_total = 0.0f;
    SH.tri_albedo = nullptr;
    SH.inst_tri_offset = nullptr;
    SH.textures = ctx_texture_table(b->ctx);
    SH.blas = b->blas.p;
    SH.inst_count = b->total_inst;
    SH.mesh_count = ctx_mesh_count(b->ctx);
    SH.texture_count = ctx_texture_count(b->ctx);
    SH.albedo_count = 0;
    SH.status = status;
    k_bbegin<<<1, 1, 0, st>>>(b->ctl, cur);
    BCUDA(cudaGetLastError());
    BCUDA(regen_or_shade(false, b, SH, Q, cur, st));
    BatchExtendIO ex;
    ex.qo = Q.qo[cur]; ex.qd = Q.qd[cur]; ex.tuvp = Q.h_tuvp; ex.inst = Q.h_inst; ex.roots = b->d_roots.p;
    ex.nscenes = b->nscenes; ex.status = status;
    auto ke = k_btrace<false, BatchExtendIO>;
    ke<<<persistent_grid(ke), kTraceBlock, 0, st>>>(S, ex, &b->ctl->count[cur], &b->ctl->fetch[0], status);
    BCUDA(cudaGetLastError());
    const int kp = (k + kBodyIterations - 1) % kBodyIterations;
    if (join_prev) BCUDA(cudaStreamWaitEvent(st, b->ev_conn[kp], 0));   // both add to the path radiance
    BCUDA(regen_or_shade(true, b, SH, Q, cur, st));
    BCUDA(cudaEventRecord(b->ev_shade[k], st));
    BCUDA(cudaStreamWaitEvent(b->side, b->ev_shade[k], 0));
    BatchConnectIO cn;
    cn.so = Q.s_o[cur]; cn.sd = Q.s_d[cur]; cn.sc = Q.s_c[cur]; cn.roots = b->d_roots.p; cn.qL = Q.qL[cur ^ 1];
    cn.nscenes = b->nscenes; cn.capacity = b->cfg.capacity; cn.total_paths = b->total_paths; cn.status = status;
    cn.out_L = Q.out_L;
    auto kc = k_btrace<true, BatchConnectIO>;
    kc<<<persistent_grid(kc), kTraceBlock, 0, b->side>>>(S, cn, &b->ctl->shadow[cur], &b->ctl->fetch[1 + cur], status);
    BCUDA(cudaGetLastError());
    BCUDA(cudaEventRecord(b->ev_conn[k], b->side));
    if (join_self) BCUDA(cudaStreamWaitEvent(st, b->ev_conn[k], 0));
    k_bend<<<1, 1, 0, st>>>(b->ctl, cur, status, h, set_cond ? 1 : 0);
    BCUDA(cudaGetLastError());
    return WF_OK;
}

constexpr uint32_t kKernelsPerIteration = 6;

int build_graph(wf_batch* b) {
    drop_graph(b);
    cudaStream_t st = ctx_stream(b->ctx);
    // occupancy queries before capture
    (void)persistent_grid(k_btrace<false, BatchExtendIO>);
    (void)persistent_grid(k_btrace<true, BatchConnectIO>);
    (void)sm_count();
    BCUDA(cudaGraphCreate(&b->graph, 0));
    cudaGraphConditionalHandle h;
    BCUDA(cudaGraphConditionalHandleCreate(&h, b->graph, 1u, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    BCUDA(cudaGraphAddNode(&node, b->graph, nullptr, nullptr, 0, &p));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    BCUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int rc = WF_OK;
    for (int k = 0; k < kBodyIterations && rc == WF_OK; ++k)
        rc = enqueue_iteration(b, k, k > 0, k == kBodyIterations - 1, h, k == kBodyIterations - 1);
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &captured);
    if (rc) return rc;
    BCUDA(e);
    BCUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->graph_valid = true;
    return WF_OK;
}

int upload_scene_table(wf_batch* b, const render_settings_t* s, const wf_render_options* o, uint32_t frame_seed) {
    std::vector<BatchScene> t(b->nscenes);
    uint32_t pb = 0, xb = 0;
    for (uint32_t i = 0; i < b->nscenes; ++i) {
        const HostScene& H = b->scenes[i];
        BatchScene& S = t[i];
        std::memset(&S, 0, sizeof(S));
        for (int k = 0; k < 4; ++k) {
            const float* m1 = H.view.clip_to_view + 4 * k;
            const float* m2 = H.view.view_to_world + 4 * k;
            S.clip_to_view[k] = make_float4(m1[0], m1[1], m1[2], m1[3]);
            S.view_to_world[k] = make_float4(m2[0], m2[1], m2[2], m2[3]);
        }
        S.dim_x = H.view.render_dim[0];
        S.dim_y = H.view.render_dim[1];
        S.width = H.width;
        S.np = H.width * H.height;
        S.spp = H.spp;
        S.path_base = pb;
        S.pix_base = xb;
        S.root = b->roots[i];
        S.light_off = b->light_off[i];
        S.light_count = b->light_cnt[i];
        S.light_total = b->light_total[i];
        S.env_strength = s->hdr_env_strength;
        std::memcpy(S.env, H.env, 12);
        S.env_tex = ctx_texture(b->ctx, H.env_texture);
        S.frame_seed = frame_seed;
        S.max_bounces = s->max_bounces;
        S.nee = o->nee ? 1u : 0u;
        S.rr_start = o->rr_start_depth;
        S.cosine = s->cosine_weighted_diffuse ? 1u : 0u;
        pb += S.np * H.spp;
        xb += S.np;
    }
    BCUDA(ctx_h2d(b->ctx, b->d_scenes.p, t.data(), t.size() * sizeof(BatchScene)));
    return WF_OK;
}

int render(wf_batch* b, const render_settings_t* s, const wf_render_options* o, uint32_t frame_seed) {
    wf_ctx* c = b->ctx;
    int rc = ctx_use_device(c);
    if (rc) return rc;
    if (!b->tables_ready && (rc = build_tables(b))) return rc;
    if ((rc = ensure_pool(b))) return rc;
    if (b->cfg.block != b->pool_block) {
        drop_graph(b);
        b->pool_block = b->cfg.block;
    }
    if ((rc = upload_scene_table(b, s, o, frame_seed))) return rc;
    cudaStream_t st = ctx_stream(c);
    BatchCtl& h = *b->ctl_host;
    std::memset(&h, 0, sizeof(h));
    h.total = b->total_paths;
    h.capacity = b->cfg.capacity;
    double thr = std::floor((double)b->cfg.regen_threshold * b->cfg.capacity);
    h.threshold = (uint32_t)std::max(1.0, std::min(thr, (double)b->cfg.capacity));
    h.stall_limit = s->max_bounces + 2u;
    // every admission adds at least capacity - threshold + 1 paths and
    // happens at least once per max_bounces + 1 iterations
    const double per_admit = std::max(1.0, (double)h.capacity - (double)h.threshold + 1.0);
    const double bound = (std::ceil((double)h.total / per_admit) + 2.0) * (s->max_bounces + 2.0) + 1024.0;
    h.max_iter = (uint32_t)std::min(bound, 2.0e9);
    if (b->cfg.max_iterations) h.max_iter = std::min(h.max_iter, b->cfg.max_iterations);
    BCUDA(ctx_h2d(c, b->ctl, &h, sizeof(BatchCtl)));
    BCUDA(cudaEventRecord(b->t0, st));
    uint64_t graph_launches = 0;
    b->host_launches = 0;
    if (b->cfg.use_graph) {
        if (!b->graph_valid && (rc = build_graph(b))) return rc;
        BCUDA(cudaGraphLaunch(b->exec, st));
        graph_launches = 1;
    } else {
        // host-driven loop: iterations in groups, then a look at `done`
        for (uint32_t group = 0;; ++group) {
            for (int k = 0; k < kBodyIterations; ++k) {
                if ((rc = enqueue_iteration(b, k, k > 0, k == kBodyIterations - 1, 0, false))) return rc;
                b->host_launches += kKernelsPerIteration;
            }
            BCUDA(ctx_d2h(c, b->ctl_host, b->ctl, sizeof(BatchCtl)));
            BCUDA(cudaStreamSynchronize(st));
            if (b->ctl_host->done) break;
            if (group > (1u << 26)) return fail_code(WF_ERR_TIMEOUT, "wf_batch_render: host loop did not finish");
        }
    }
    k_bresolve<<<stage_grid(256), 256, 0, st>>>(b->d_scenes.p, b->d_pixbase.p, b->nscenes, b->out_L.p, b->image.p,
                                                b->total_pixels);
    BCUDA(cudaGetLastError());
    BCUDA(cudaEventRecord(b->t1, st));
    BCUDA(ctx_d2h(c, b->ctl_host, b->ctl, sizeof(BatchCtl)));
    BCUDA(cudaEventSynchronize(b->t1));
    BCUDA(cudaStreamSynchronize(st));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, b->t0, b->t1);
    const BatchCtl& r = *b->ctl_host;
    wf_batch_stats& S = b->stats;
    std::memset(&S, 0, sizeof(S));
    S.ms_total = ms;
    S.paths = b->total_paths;
    S.rays_extend = r.rays_ext;
    S.rays_connect = r.rays_con;
    S.iterations = r.iter;
    S.graph_launches = (uint32_t)graph_launches;
    S.kernel_launches =
        (b->cfg.use_graph ? (uint64_t)r.body_runs * kBodyIterations * kKernelsPerIteration : b->host_launches) + 1;
    S.scenes = b->nscenes;
    b->rendered = true;
    rc = ctx_take_status(c);
    if (rc) return rc;
    if (r.next != r.total || r.count[0] != 0 || r.count[1] != 0)
        return fail_code(WF_ERR_TIMEOUT, "wf_batch_render: the pipeline stopped before every path finished");
    return WF_OK;
}

int validate(wf_batch* b, const render_settings_t* s, const wf_render_options* o, const char* who) {
    const std::string w(who);
    if (!b || !s || !o) return fail_code(WF_ERR_INVALID, w + ": null argument");
    if (b->in_scene) return fail_code(WF_ERR_STATE, w + ": a scene is still open (wf_batch_scene_end)");
    if (b->scenes.empty()) return fail_code(WF_ERR_STATE, w + ": the batch has no scenes");
    if (s->max_bounces >= kMaxDepth - 1) return fail_code(WF_ERR_INVALID, w + ": max_bounces must be < 15");
    if (s->render_view_mode != RENDER_VIEW_MODE_NONE)
        return fail_code(WF_ERR_INVALID, w + ": a batch renders RENDER_VIEW_MODE_NONE only");
    return WF_OK;
}

}  // namespace

extern "C" {

int wf_batch_create(wf_ctx* ctx, wf_batch** out) {
    if (!ctx || !out) return fail_code(WF_ERR_INVALID, "wf_batch_create: null argument");
    int rc = ctx_use_device(ctx);
    if (rc) return rc;
    wf_batch* b = new wf_batch();
    b->ctx = ctx;
    default_config(&b->cfg);
    bool ok = cudaEventCreate(&b->t0) == cudaSuccess && cudaEventCreate(&b->t1) == cudaSuccess &&
              cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) == cudaSuccess;
    for (int k = 0; ok && k < kBodyIterations; ++k)
        ok = cudaEventCreateWithFlags(&b->ev_shade[k], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->ev_conn[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        wf_batch_destroy(b);
        return fail_code(WF_ERR_CUDA, "wf_batch_create: stream or event creation failed");
    }
    *out = b;
    return WF_OK;
}

int wf_batch_destroy(wf_batch* b) {
    if (!b) return WF_OK;
    ctx_use_device(b->ctx);
    cudaStreamSynchronize(ctx_stream(b->ctx));
    drop_graph(b);
    b->tnodes.release(); b->tinst.release(); b->sinst.release(); b->aabbs.release();
    b->tlas_scratch.release(); b->d_roots.release(); b->d_pbase.release(); b->d_pixbase.release();
    b->lights.release(); b->blas.release(); b->stri.release(); b->d_scenes.release();
    b->out_L.release(); b->image.release();
    for (auto& q : b->q) q.release();
    b->h_tuvp.release(); b->h_inst.release();
    for (int k = 0; k < 2; ++k) { b->s_o[k].release(); b->s_d[k].release(); b->s_c[k].release(); }
    for (int k = 0; k < kBodyIterations; ++k) {
        if (b->ev_shade[k]) cudaEventDestroy(b->ev_shade[k]);
        if (b->ev_conn[k]) cudaEventDestroy(b->ev_conn[k]);
    }
    if (b->side) cudaStreamDestroy(b->side);
    if (b->ctl) dfree(b->ctl);
    if (b->ctl_host) cudaFreeHost(b->ctl_host);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    delete b;
    return WF_OK;
}

int wf_batch_scene_begin(wf_batch* b, uint32_t width, uint32_t height, uint32_t spp, const view_t* view,
                         const wf_env* env, uint32_t* out_scene) {
    if (!b || !view) return fail_code(WF_ERR_INVALID, "wf_batch_scene_begin: null argument");
    if (b->in_scene) return fail_code(WF_ERR_STATE, "wf_batch_scene_begin: the previous scene is still open");
    if (width == 0 || height == 0 || spp == 0)
        return fail_code(WF_ERR_INVALID, "wf_batch_scene_begin: width, height and spp must be >= 1");
    if ((uint64_t)width * height * spp >= (1ull << 31))
        return fail_code(WF_ERR_CAPACITY, "wf_batch_scene_begin: more than 2^31 - 1 camera paths");
    if (b->scenes.size() >= 65535) return fail_code(WF_ERR_CAPACITY, "wf_batch_scene_begin: more than 65535 scenes");
    HostScene H;
    H.width = width;
    H.height = height;
    H.spp = spp;
    H.view = *view;
    if (env && env->texture > ctx_texture_count(b->ctx))
        return fail_code(WF_ERR_INVALID, "wf_batch_scene_begin: unknown env texture");
    if (env) std::memcpy(H.env, env->color, 12);
    else H.env[0] = H.env[1] = H.env[2] = 1.0f;
    H.env_texture = env ? env->texture : 0u;
    b->scenes.push_back(H);
    b->in_scene = true;
    b->tables_ready = false;
    b->rendered = false;
    if (out_scene) *out_scene = (uint32_t)b->scenes.size() - 1;
    return WF_OK;
}

int wf_batch_instance_submit(wf_batch* b, uint32_t mesh, const float l2w[16], const wf_material_ext* mat) {
    if (!b || !mat) return fail_code(WF_ERR_INVALID, "wf_batch_instance_submit: null argument");
    if (!b->in_scene) return fail_code(WF_ERR_STATE, "wf_batch_instance_submit: no open scene");
    Instance in;
    int rc = make_instance(b->ctx, mesh, l2w, &mat->base, mat->bsdf, mat->ior, "wf_batch_instance_submit", &in);
    if (rc) return rc;
    b->scenes.back().inst.push_back(in);
    return WF_OK;
}

int wf_batch_scene_end(wf_batch* b) {
    if (!b) return fail_code(WF_ERR_INVALID, "wf_batch_scene_end: null argument");
    if (!b->in_scene) return fail_code(WF_ERR_STATE, "wf_batch_scene_end: no open scene");
    b->in_scene = false;
    return WF_OK;
}

int wf_batch_set_config(wf_batch* b, const wf_batch_config* cfg) {
    if (!b || !cfg) return fail_code(WF_ERR_INVALID, "wf_batch_set_config: null argument");
    wf_batch_config c;
    int rc = check_config(cfg, &c);
    if (rc) return rc;
    if (c.capacity != b->cfg.capacity || c.block != b->cfg.block) drop_graph(b);
    b->cfg = c;
    return WF_OK;
}

int wf_batch_get_config(wf_batch* b, wf_batch_config* out) {
    if (!b || !out) return fail_code(WF_ERR_INVALID, "wf_batch_get_config: null argument");
    *out = b->cfg;
    return WF_OK;
}

int wf_batch_render(wf_batch* b, const render_settings_t* s, const wf_render_options* o, uint32_t frame_seed) {
    int rc = validate(b, s, o, "wf_batch_render");
    if (rc) return rc;
    return render(b, s, o, frame_seed);
}

int wf_batch_autotune(wf_batch* b, const render_settings_t* s, const wf_render_options* o, uint32_t frame_seed,
                      wf_batch_config* out) {
    int rc = validate(b, s, o, "wf_batch_autotune");
    if (rc) return rc;
    // Coordinate descent over pool capacity, then regeneration threshold, then
    // block size; each candidate is rendered once to warm up (buffers, graph)
    // and timed on a second render.
    wf_batch_config best = b->cfg;
    best.use_graph = 1;
    double best_ms = 1e30;
    auto trial = [&](const wf_batch_config& cand, double* ms) -> int {
        int r = wf_batch_set_config(b, &cand);
        if (r) return r;
        if ((r = render(b, s, o, frame_seed))) return r;
        if ((r = render(b, s, o, frame_seed))) return r;
        *ms = b->stats.ms_total;
        return WF_OK;
    };
    {
        double ms;
        if ((rc = trial(best, &ms))) return rc;
        best_ms = ms;
    }
    uint64_t tp = 0;
    for (const HostScene& H : b->scenes) tp += (uint64_t)H.width * H.height * H.spp;
    const uint32_t caps[] = {1u << 19, 1u << 20, 1u << 21, 1u << 22, 1u << 23, 1u << 24};
    wf_batch_config base = best;
    for (uint32_t cap : caps) {
        if (cap == base.capacity) continue;
        if (cap > 2 * tp && cap > (1u << 19)) continue;   // a pool far larger than the batch adds nothing
        wf_batch_config cand = base;
        cand.capacity = cap;
        double ms;
        if ((rc = trial(cand, &ms))) return rc;
        if (ms < best_ms) { best_ms = ms; best = cand; }
    }
    base = best;
    const float thrs[] = {0.5f, 0.75f, 0.9f, 1.0f};
    for (float t : thrs) {
        if (t == base.regen_threshold) continue;
        wf_batch_config cand = base;
        cand.regen_threshold = t;
        double ms;
        if ((rc = trial(cand, &ms))) return rc;
        if (ms < best_ms) { best_ms = ms; best = cand; }
    }
    base = best;
    const uint32_t blocks[] = {128, 256, 512};
    for (uint32_t blk : blocks) {
        if (blk == base.block) continue;
        wf_batch_config cand = base;
        cand.block = blk;
        double ms;
        if ((rc = trial(cand, &ms))) return rc;
        if (ms < best_ms) { best_ms = ms; best = cand; }
    }
    if ((rc = wf_batch_set_config(b, &best))) return rc;
    if (out) *out = best;
    return WF_OK;
}

int wf_batch_read_image(wf_batch* b, uint32_t scene, float* out, uint64_t nfloat) {
    if (!b || !out) return fail_code(WF_ERR_INVALID, "wf_batch_read_image: null argument");
    if (!b->rendered) return fail_code(WF_ERR_STATE, "wf_batch_read_image: nothing rendered");
    if (scene >= b->scenes.size()) return fail_code(WF_ERR_INVALID, "wf_batch_read_image: unknown scene");
    const HostScene& H = b->scenes[scene];
    const uint64_t np = (uint64_t)H.width * H.height;
    if (nfloat < 4 * np) return fail_code(WF_ERR_CAPACITY, "wf_batch_read_image: output smaller than width*height*4");
    uint64_t base = 0;
    for (uint32_t s = 0; s < scene; ++s) base += (uint64_t)b->scenes[s].width * b->scenes[s].height;
    int rc = ctx_use_device(b->ctx);
    if (rc) return rc;
    BCUDA(ctx_d2h(b->ctx, out, b->image.p + base, np * sizeof(float4)));
    BCUDA(cudaStreamSynchronize(ctx_stream(b->ctx)));
    return WF_OK;
}

int wf_batch_get_stats(wf_batch* b, wf_batch_stats* out) {
    if (!b || !out) return fail_code(WF_ERR_INVALID, "wf_batch_get_stats: null argument");
    *out = b->stats;
    return WF_OK;
}

}  // extern "C"
