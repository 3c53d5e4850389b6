// wf_api.cu — the C ABI (include/wf.h): context, meshes, scene, wavefront
// orchestration, ray queries and the stand-alone builders.
//
// The orchestration mirrors renderer::render (renderer.cpp:742-939): per
// wave, generate once, then for depth 0..max_bounces extend -> shade ->
// connect.  The reference sizes its indirect dispatches on the GPU
// (init_args.hlsl:15-22); here every stage reads its queue length from device
// memory and runs a grid-stride loop, so the host never reads a count back.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <unordered_map>

#include <nvtx3/nvToolsExt.h>

#include "../../include/wf.h"
#include "wf_bvh.h"
#include "wf_ctx.h"
#include "wf_kernels.h"

using namespace wf;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

#define WF_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            return fail(e_ == cudaErrorMemoryAllocation ? WF_ERR_OOM : WF_ERR_CUDA,            \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                   \
        }                                                                                      \
    } while (0)

template <typename T>
int dev_alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = dmalloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(WF_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return WF_OK;
}

template <typename T>
void dev_free(T*& p) {
    if (p) dfree(const_cast<void*>(reinterpret_cast<const void*>(p)));
    p = nullptr;
}

// Grow-only device buffer.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    int reserve(size_t n) {
        if (n <= cap && p) return WF_OK;
        dev_free(p);
        cap = 0;
        int rc = dev_alloc(&p, n);
        if (rc == WF_OK) cap = n ? n : 1;
        return rc;
    }
    void release() { dev_free(p); cap = 0; }
};

struct Texture {
    float4* d = nullptr;
    uint32_t w = 0, h = 0;
};

constexpr uint32_t kHullBoxes = 4096;   // instance_bounds 1: frontier boxes per BLAS

struct Mesh {
    uint32_t tri_count = 0, node_count = 0;
    std::vector<triangle_t> tris;     // original order (create_render_mesh keeps them too)
    std::vector<uint8_t> blob;        // [bvh_header_t | nodes | bvh_triangle_t | uint32]
    float root_min[3], root_max[3];
    float4* d_nodes = nullptr;
    float4* d_tris = nullptr;         // traversal triangles, leaf order
    float4* d_stri = nullptr;         // shading triangles, original order
    float4* d_qnodes = nullptr;       // quantized 4-wide nodes (blas_layout 1)
    uint32_t qnode_count = 0, root_count = 0;
    float4* d_hull = nullptr;         // instance_bounds 1: the BLAS frontier boxes {min, max}
    uint32_t hull_count = 0;
};

struct EventPair {
    cudaEvent_t a, b;
    int stage;
    int depth;   // the bounce depth of an extend / connect launch, else -1
};

enum Stage { ST_GENERATE = 0, ST_EXTEND, ST_SHADE, ST_CONNECT, ST_POST, ST_TLAS, ST_TAIL, ST_COUNT };
// NVTX range names: the reference's GPU profiler scope labels (gpu_profiler.h:59-66)
// plus the added connect stage.
const char* const kStageLabel[ST_COUNT] = {"Wavefront Generate", "Wavefront Extend", "Wavefront Shade",
                                           "Wavefront Connect", "Post-Process", "TLAS Build", "Wavefront Tail"};

}  // namespace

struct wf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t width = 0, height = 0, capacity = 0, tlas_metric = 0, blas_layout = 0, instance_bounds = 0;
    std::vector<Mesh> meshes;
    std::vector<Instance> instances;
    view_t view{};
    bool view_valid = false, in_scene = false, scene_ready = false, view_changed = true;
    float env[3] = {1.0f, 1.0f, 1.0f};
    uint32_t env_texture = 0;
    uint32_t last_view_mode = 0;
    uint32_t last_frame_seed = 0;
    std::vector<Texture> textures;          // id k + 1
    DevBuf<TexRef> tex_table;               // entry 0 unused

    // device scene
    DevBuf<float4> tnodes, tinst, sinst;
    DevBuf<BlasRef> blas;
    DevBuf<const float4*> stri;
    DevBuf<LightTri> lights;
    DevBuf<float> aabbs;
    DevBuf<HullRef> hulls;                  // instance_bounds 1: per mesh
    DevBuf<uint32_t> tlas_scratch;
    uint32_t light_count = 0;
    float light_total = 0.0f;
    std::vector<bvh_instance_t> scene_bi;
    bool bounds_pending = false;            // scene_bi's boxes still on the device (aabbs)
    uint64_t scene_triangles = 0;           // sum of the instances' triangle counts
    bool albedo_set = false;
    DevBuf<float4> tri_albedo;              // per scene triangle (wf_scene_set_albedo)
    DevBuf<uint32_t> inst_tri_offset;
    DevBuf<float4> L_final, dimage, g_albedo;   // adjoint buffers
    DevBuf<float> g_emission;
    DevBuf<float> g_em_rep;                 // adjoint: shadow rays' emitter gradients, 32 replicas
    DevBuf<float4> L_comp, L_final_lo;      // adjoint: rounding errors of the path radiance sums

    // wavefront buffers
    bool buffers_ready = false;
    RenderBuffers B{};
    float4* accum = nullptr;
    uint32_t accum_samples = 0;
    unsigned long long* totals = nullptr;   // [0] extension rays, [1] shadow rays, [2 + d] extension
                                            // rays at depth d, [2 + kMaxDepth + d] shadow rays at depth d
    DevBuf<float4> image;
    DevBuf<uchar4> image_ldr;
    DevBuf<uint8_t> trace_io;
    DevBuf<uint32_t> sort_scratch;          // WF_TRACE_REORDER: keys, permutation, digit counts
    uint32_t* status = nullptr;
    uint32_t* trace_fetch = nullptr;        // fetch counter of wf_trace / wf_trace_device
    Counters* counters = nullptr;

    // timing
    std::vector<EventPair> events;
    size_t events_used = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    // connect at depth d runs on `side` while extend at depth d + 1 runs on
    // `stream`; shade at d + 1 waits for it (both add to the path radiance)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_shade[kMaxDepth] = {}, ev_conn[kMaxDepth] = {};
    bool timing_pending = false;
    // queue sizes of the last wave, copied to pinned host memory after it; they
    // choose where the next wave hands its remaining bounces to the tail kernel
    uint32_t* h_counts = nullptr;           // pinned, kMaxDepth extension counts
    cudaEvent_t ev_counts = nullptr;
    // wf_read_image_async: the resolved image is copied to the host on `copy`
    // (after img_ready on `stream`) while the next frame renders; the next
    // resolve into `image` waits for img_copied
    cudaStream_t copy = nullptr;
    cudaEvent_t img_ready = nullptr, img_copied = nullptr;
    bool img_copy_pending = false;
    bool counts_pending = false, counts_known = false;
    uint32_t last_counts[kMaxDepth] = {};
    wf_stats stats{};
    uint64_t launches = 0, launches_extend = 0, launches_connect = 0, tail_depth = 0;
    bool count_traffic = false;
    uint64_t h2d_bytes = 0, d2h_bytes = 0;   // cumulative over the context's life
};

namespace {

int use_device(wf_ctx* c) {
    WF_CUDA(cudaSetDevice(c->device));
    return WF_OK;
}

// Host<->device copies on the context stream, counted for wf_stats.
cudaError_t h2d(wf_ctx* c, void* dst, const void* src, size_t bytes) {
    c->h2d_bytes += bytes;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
}
cudaError_t d2h(wf_ctx* c, void* dst, const void* src, size_t bytes) {
    c->d2h_bytes += bytes;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
}

// An NVTX range around a stage's enqueue (seen by Nsight Systems), and a CUDA
// event pair around its GPU work when profiling.
struct StageTimer {
    wf_ctx* c;
    cudaStream_t st;
    EventPair* ev = nullptr;
    StageTimer(wf_ctx* ctx, bool on, int stage, cudaStream_t stream = nullptr, int depth = -1)
        : c(ctx), st(stream ? stream : ctx->stream) {
        nvtxRangePushA(kStageLabel[stage]);
        if (!on) return;
        if (c->events_used == c->events.size()) {
            EventPair p{};
            cudaEventCreate(&p.a);
            cudaEventCreate(&p.b);
            c->events.push_back(p);
        }
        ev = &c->events[c->events_used++];
        ev->stage = stage;
        ev->depth = depth;
        cudaEventRecord(ev->a, st);
    }
    ~StageTimer() {
        if (ev) cudaEventRecord(ev->b, st);
        nvtxRangePop();
    }
};

// 4x4 inverse by cofactor expansion in double precision, rounded to float.
// Input and output are glm column-major (m[4*col + row]).
bool invert4(const float* m, float* out) {
    double a[4][4];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) a[r][c] = m[4 * c + r];
    double inv[4][4];
    double det = 0.0;
    auto minor3 = [&](int rr, int cc) {
        double s[3][3];
        for (int r = 0, i = 0; r < 4; ++r) {
            if (r == rr) continue;
            for (int c2 = 0, j = 0; c2 < 4; ++c2) {
                if (c2 == cc) continue;
                s[i][j++] = a[r][c2];
            }
            ++i;
        }
        return s[0][0] * (s[1][1] * s[2][2] - s[1][2] * s[2][1]) - s[0][1] * (s[1][0] * s[2][2] - s[1][2] * s[2][0]) +
               s[0][2] * (s[1][0] * s[2][1] - s[1][1] * s[2][0]);
    };
    double cof[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c2 = 0; c2 < 4; ++c2) cof[r][c2] = (((r + c2) & 1) ? -1.0 : 1.0) * minor3(r, c2);
    for (int c2 = 0; c2 < 4; ++c2) det += a[0][c2] * cof[0][c2];
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    for (int r = 0; r < 4; ++r)
        for (int c2 = 0; c2 < 4; ++c2) inv[r][c2] = cof[c2][r] / det;
    for (int c2 = 0; c2 < 4; ++c2)
        for (int r = 0; r < 4; ++r) out[4 * c2 + r] = (float)inv[r][c2];
    return true;
}

// glm mat4 * vec4 (type_mat4x4.inl): (m0*v0 + m1*v1) + (m2*v2 + m3*v3).
void glm_mul_point(const float* m, const float v[3], float out[3]) {
    for (int j = 0; j < 3; ++j) {
        float a0 = m[j] * v[0];
        float a1 = m[4 + j] * v[1];
        float a2 = m[8 + j] * v[2];
        float a3 = m[12 + j] * 1.0f;
        out[j] = (a0 + a1) + (a2 + a3);
    }
}

// HLSL mul(float4(v, w), M) order, as the kernels and the oracle evaluate it.
void hlsl_xform(const float* m, const float v[3], float w, float out[3]) {
    for (int j = 0; j < 3; ++j) out[j] = v[0] * m[j] + v[1] * m[4 + j] + v[2] * m[8 + j] + w * m[12 + j];
}

int check_blob(const void* blob, uint64_t size, uint32_t n, uint32_t* out_nodes) {
    if (size < 12) return fail(WF_ERR_INVALID, "BLAS blob shorter than its header");
    bvh_header_t h;
    std::memcpy(&h, blob, 12);
    if (h.nodes_offset != 12 || h.triangles_offset < 12 || ((h.triangles_offset - 12) % 32) != 0)
        return fail(WF_ERR_INVALID, "BLAS blob header offsets are not [header | nodes | ...]");
    uint64_t nc = (h.triangles_offset - 12) / 32;
    if (nc < 2) return fail(WF_ERR_INVALID, "BLAS blob has fewer than 2 nodes");
    if ((uint64_t)h.indices_offset != (uint64_t)h.triangles_offset + 36ull * n ||
        size != (uint64_t)h.indices_offset + 4ull * n)
        return fail(WF_ERR_INVALID, "BLAS blob size does not match the triangle count");
    const uint8_t* b = static_cast<const uint8_t*>(blob);
    for (uint64_t i = 0; i < nc; ++i) {
        if (i == 1) continue;
        bvh_node_t node;
        std::memcpy(&node, b + 12 + 32 * i, 32);
        if (node.prim_count > 0) {
            if ((uint64_t)node.left_first + node.prim_count > n) return fail(WF_ERR_INVALID, "BLAS leaf range out of bounds");
        } else if (!(node.left_first > i && (uint64_t)node.left_first + 1 < nc)) {
            // children are allocated after their parent, which also rules out cycles
            return fail(WF_ERR_INVALID, "BLAS child index out of range or not after its parent");
        }
    }
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t t;
        std::memcpy(&t, b + h.indices_offset + 4ull * i, 4);
        if (t >= n) return fail(WF_ERR_INVALID, "BLAS index list entry out of range");
    }
    *out_nodes = (uint32_t)nc;
    return WF_OK;
}

void free_mesh(Mesh& m) {
    dev_free(m.d_nodes);
    dev_free(m.d_tris);
    dev_free(m.d_stri);
    dev_free(m.d_qnodes);
    dev_free(m.d_hull);
}

// instance_bounds 1: up to kHullBoxes boxes of the mesh's BLAS that together
// hold every triangle, the frontier reached from the root by repeatedly
// opening the interior node of largest surface area (ties: lower node index).
// An instance's world box is then the union of these boxes' world boxes,
// much closer to the transformed geometry's own box than the world box of the
// transformed root box (for a randomly rotated sphere, about half its area).
int upload_hull(wf_ctx* c, Mesh& m) {
    if (c->instance_bounds != 1 || m.node_count == 0) return WF_OK;
    bvh_header_t h;
    std::memcpy(&h, m.blob.data(), 12);
    auto node = [&](uint32_t i) {
        bvh_node_t n;
        std::memcpy(&n, m.blob.data() + h.nodes_offset + 32ull * i, 32);
        return n;
    };
    auto area = [](const bvh_node_t& n) {
        const float ex = n.aabb_max[0] - n.aabb_min[0], ey = n.aabb_max[1] - n.aabb_min[1],
                    ez = n.aabb_max[2] - n.aabb_min[2];
        return ex * ey + ey * ez + ez * ex;
    };
    // max-heap on (area, then lower index): interior nodes still to open
    auto cmp = [](const std::pair<float, uint32_t>& a, const std::pair<float, uint32_t>& b) {
        return a.first < b.first || (a.first == b.first && a.second > b.second);
    };
    std::vector<std::pair<float, uint32_t>> open;
    std::vector<uint32_t> done;   // leaves: cannot be opened
    const bvh_node_t root = node(0);
    if (root.prim_count > 0) done.push_back(0);
    else open.push_back({area(root), 0});
    while (!open.empty() && open.size() + done.size() < kHullBoxes) {
        std::pop_heap(open.begin(), open.end(), cmp);
        const uint32_t i = open.back().second;
        open.pop_back();
        const uint32_t l = node(i).left_first;
        if (l + 1 >= m.node_count) return fail(WF_ERR_INVALID, "BLAS child index out of range");
        for (uint32_t ch = l; ch <= l + 1; ++ch) {
            const bvh_node_t n = node(ch);
            if (n.prim_count > 0) {
                done.push_back(ch);
            } else {
                open.push_back({area(n), ch});
                std::push_heap(open.begin(), open.end(), cmp);
            }
        }
    }
    for (const auto& e : open) done.push_back(e.second);
    std::sort(done.begin(), done.end());
    std::vector<float4> boxes(2 * done.size());
    for (size_t k = 0; k < done.size(); ++k) {
        const bvh_node_t n = node(done[k]);
        boxes[2 * k] = make_float4(n.aabb_min[0], n.aabb_min[1], n.aabb_min[2], 0.0f);
        boxes[2 * k + 1] = make_float4(n.aabb_max[0], n.aabb_max[1], n.aabb_max[2], 0.0f);
    }
    m.hull_count = (uint32_t)done.size();
    int rc = dev_alloc(&m.d_hull, boxes.size());
    if (rc) return rc;
    WF_CUDA(h2d(c, m.d_hull, boxes.data(), boxes.size() * sizeof(float4)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    return WF_OK;
}

// The 4-wide nodes of the mesh's BLAS (blas_layout 1: quantized, 64 bytes;
// 2: exact, 128 bytes), from its blob.
int upload_qnodes(wf_ctx* c, Mesh& m) {
    if (c->blas_layout == 0) return WF_OK;
    std::vector<uint32_t> words;
    const char* err = nullptr;
    const bool exact = c->blas_layout == 2;
    int rc = qbvh_convert(m.blob.data(), m.blob.size(), words, &m.root_count, &err, exact);
    if (rc) return fail(rc, err);
    m.qnode_count = (uint32_t)(words.size() / (exact ? 32 : 16));
    if (m.qnode_count == 0) return WF_OK;
    if ((rc = dev_alloc(&m.d_qnodes, words.size() / 4))) return rc;
    WF_CUDA(h2d(c, m.d_qnodes, words.data(), words.size() * 4));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int upload_shading_tris(wf_ctx* c, Mesh& m) {
    std::vector<float4> st(6ull * m.tri_count);
    host_parallel(m.tri_count, 1u << 15, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            const triangle_t& t = m.tris[i];
            const vertex_t* v[3] = {&t.v0, &t.v1, &t.v2};
            for (int k = 0; k < 3; ++k) {
                st[6 * i + k] = make_float4(v[k]->position[0], v[k]->position[1], v[k]->position[2], 0.0f);
                st[6 * i + 3 + k] = make_float4(v[k]->normal[0], v[k]->normal[1], v[k]->normal[2], 0.0f);
            }
            // vertex uv in the .w slots: {p0, u0} {p1, v0} {p2, u1} {n0, v1} {n1, u2} {n2, v2}
            for (int k = 0; k < 3; ++k) {
                st[6 * i + 2 * k].w = v[k]->uv[0];
                st[6 * i + 2 * k + 1].w = v[k]->uv[1];
            }
        }
    });
    int rc = dev_alloc(&m.d_stri, st.size());
    if (rc) return rc;
    WF_CUDA(h2d(c, m.d_stri, st.data(), st.size() * sizeof(float4)));
    return WF_OK;
}

// Device copies of a BLAS given as a blob (host).
int upload_blob(wf_ctx* c, Mesh& m) {
    bvh_header_t h;
    std::memcpy(&h, m.blob.data(), 12);
    std::vector<float4> nodes(2ull * m.node_count);
    std::memcpy(nodes.data(), m.blob.data() + 12, 32ull * m.node_count);
    std::vector<float4> tt(3ull * m.tri_count);
    const uint8_t* tb = m.blob.data() + h.triangles_offset;
    const uint8_t* ib = m.blob.data() + h.indices_offset;
    for (uint32_t i = 0; i < m.tri_count; ++i) {
        uint32_t t;
        std::memcpy(&t, ib + 4ull * i, 4);
        bvh_triangle_t tri;
        std::memcpy(&tri, tb + 36ull * t, 36);
        float e1[3], e2[3];
        for (int a = 0; a < 3; ++a) { e1[a] = tri.p1[a] - tri.p0[a]; e2[a] = tri.p2[a] - tri.p0[a]; }
        float w;
        std::memcpy(&w, &t, 4);
        tt[3ull * i] = make_float4(tri.p0[0], tri.p0[1], tri.p0[2], w);
        tt[3ull * i + 1] = make_float4(e1[0], e1[1], e1[2], 0.0f);
        tt[3ull * i + 2] = make_float4(e2[0], e2[1], e2[2], 0.0f);
    }
    bvh_node_t root;
    std::memcpy(&root, m.blob.data() + 12, 32);
    std::memcpy(m.root_min, root.aabb_min, 12);
    std::memcpy(m.root_max, root.aabb_max, 12);
    int rc = dev_alloc(&m.d_nodes, nodes.size());
    if (rc) return rc;
    rc = dev_alloc(&m.d_tris, tt.size());
    if (rc) return rc;
    WF_CUDA(h2d(c, m.d_nodes, nodes.data(), nodes.size() * sizeof(float4)));
    WF_CUDA(h2d(c, m.d_tris, tt.data(), tt.size() * sizeof(float4)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    return WF_OK;
}

int ensure_buffers(wf_ctx* c) {
    if (c->buffers_ready) return WF_OK;
    const size_t C = c->capacity, npix = (size_t)c->width * c->height;
    RenderBuffers& B = c->B;
    B.ps_Lc = nullptr;   // only wf_adjoint's passes keep rounding errors
    int rc = 0;
    for (int k = 0; k < 2; ++k) {
        if ((rc = dev_alloc(&B.q_o[k], C)) || (rc = dev_alloc(&B.q_d[k], C)) || (rc = dev_alloc(&B.q_path[k], C)))
            return rc;
    }
    if ((rc = dev_alloc(&B.h_tuvp, C)) || (rc = dev_alloc(&B.h_inst, C)) || (rc = dev_alloc(&B.ps_T, C)) ||
        (rc = dev_alloc(&B.ps_flags, C)) || (rc = dev_alloc(&B.ps_L, C)) || (rc = dev_alloc(&B.counts, 4 * kMaxDepth)) ||
        (rc = dev_alloc(&c->accum, npix)))
        return rc;
    for (int k = 0; k < 2; ++k)
        if ((rc = dev_alloc(&B.s_o[k], C)) || (rc = dev_alloc(&B.s_d[k], C)) || (rc = dev_alloc(&B.s_c[k], C)))
        return rc;
    B.accum = c->accum;
    B.status = c->status;
    B.counters = c->counters;
    B.capacity = c->capacity;
    WF_CUDA(cudaMemsetAsync(c->accum, 0, npix * sizeof(float4), c->stream));
    c->accum_samples = 0;
    c->buffers_ready = true;
    return WF_OK;
}

void release_buffers(wf_ctx* c) {
    RenderBuffers& B = c->B;
    for (int k = 0; k < 2; ++k) { dev_free(B.q_o[k]); dev_free(B.q_d[k]); dev_free(B.q_path[k]); }
    dev_free(B.h_tuvp); dev_free(B.h_inst); dev_free(B.ps_T); dev_free(B.ps_flags); dev_free(B.ps_L);
    for (int k = 0; k < 2; ++k) { dev_free(B.s_o[k]); dev_free(B.s_d[k]); dev_free(B.s_c[k]); }
    dev_free(B.counts);
    dev_free(c->accum);
    c->buffers_ready = false;
}

SceneRefs scene_refs(wf_ctx* c) {
    SceneRefs S;
    S.tnodes = c->tnodes.p;
    S.tinst = c->tinst.p;
    S.blas = c->blas.p;
    S.inst_count = (uint32_t)c->scene_bi.size();
    S.tnode_count = 2u * S.inst_count;
    S.mesh_count = (uint32_t)c->meshes.size();
    S.status = c->status;
    S.qbvh = c->blas_layout;
    return S;
}

// Reads and clears the device status word (after a synchronization).
int take_status(wf_ctx* c) {
    uint32_t s = 0;
    WF_CUDA(d2h(c, &s, c->status, 4));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    if (s) {
        WF_CUDA(cudaMemsetAsync(c->status, 0, 4, c->stream));
        WF_CUDA(cudaStreamSynchronize(c->stream));
    }
    if (s & ERRF_STACK) return fail(WF_ERR_STACK, "a traversal stack overflowed; affected rays report a miss");
    if (s & ERRF_TIMEOUT) return fail(WF_ERR_TIMEOUT, "a bounded device wait gave up");
    if (s & ERRF_CAPACITY) return fail(WF_ERR_CAPACITY, "a device queue overflowed");
    if (s & ERRF_BOUNDS) return fail(WF_ERR_BOUNDS, "a device index was out of bounds (checked build); the access was skipped");
    return WF_OK;
}

int finish_timing(wf_ctx* c) {
    if (!c->timing_pending) return WF_OK;
    WF_CUDA(cudaEventSynchronize(c->t1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, c->t0, c->t1);
    c->stats.ms_total = ms;
    double st[ST_COUNT] = {0, 0, 0, 0, 0, 0, 0};
    for (size_t i = 0; i < c->events_used; ++i) {
        float e = 0.0f;
        cudaEventElapsedTime(&e, c->events[i].a, c->events[i].b);
        const EventPair& ev = c->events[i];
        st[ev.stage] += e;
        if (ev.depth >= 0 && ev.depth < (int)kMaxDepth) {
            if (ev.stage == ST_EXTEND) c->stats.ms_extend_depth[ev.depth] += e;
            if (ev.stage == ST_CONNECT) c->stats.ms_connect_depth[ev.depth] += e;
        }
    }
    c->stats.ms_generate = st[ST_GENERATE];
    c->stats.ms_extend = st[ST_EXTEND];
    c->stats.ms_shade = st[ST_SHADE];
    c->stats.ms_connect = st[ST_CONNECT];
    c->stats.ms_post = st[ST_POST];
    c->stats.ms_tlas_build = st[ST_TLAS];
    c->stats.ms_tail = st[ST_TAIL];
    unsigned long long tot[2 + 2 * kMaxDepth] = {};
    WF_CUDA(d2h(c, tot, c->totals, sizeof(tot)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    c->stats.rays_extend = tot[0];
    c->stats.rays_connect = tot[1];
    for (uint32_t d = 0; d < kMaxDepth; ++d) {
        c->stats.extend_rays_depth[d] = tot[2 + d];
        c->stats.shadow_rays_depth[d] = tot[2 + kMaxDepth + d];
    }
    if (c->count_traffic) {
        // one counter slot per depth: [d] extension rays, [kMaxDepth + d] shadow rays
        Counters k[2 * kMaxDepth];
        WF_CUDA(d2h(c, k, c->counters, sizeof(k)));
        WF_CUDA(cudaStreamSynchronize(c->stream));
        for (uint32_t d = 0; d < kMaxDepth; ++d) {
            const Counters& e = k[d];
            const Counters& h = k[kMaxDepth + d];
            c->stats.tlas_node_loads += e.tlas_node_loads;
            c->stats.instance_loads += e.instance_loads;
            c->stats.blas_node_loads += e.blas_node_loads;
            c->stats.triangle_tests += e.triangle_tests;
            c->stats.shadow_tlas_node_loads += h.tlas_node_loads;
            c->stats.shadow_instance_loads += h.instance_loads;
            c->stats.shadow_blas_node_loads += h.blas_node_loads;
            c->stats.shadow_triangle_tests += h.triangle_tests;
            const uint64_t ef[4] = {e.tlas_node_loads, e.instance_loads, e.blas_node_loads, e.triangle_tests};
            const uint64_t hf[4] = {h.tlas_node_loads, h.instance_loads, h.blas_node_loads, h.triangle_tests};
            for (int j = 0; j < 4; ++j) {
                c->stats.extend_fetch_depth[d][j] = ef[j];
                c->stats.shadow_fetch_depth[d][j] = hf[j];
            }
        }
    }
    c->timing_pending = false;
    return WF_OK;
}

int begin_call(wf_ctx* c, bool count_traffic) {
    int rc = finish_timing(c);
    if (rc) return rc;
    std::memset(&c->stats, 0, sizeof(c->stats));
    c->events_used = 0;
    c->launches = c->launches_extend = c->launches_connect = 0;
    c->tail_depth = 0;
    c->count_traffic = count_traffic;
    WF_CUDA(cudaMemsetAsync(c->totals, 0, (2 + 2 * kMaxDepth) * sizeof(unsigned long long), c->stream));
    WF_CUDA(cudaMemsetAsync(c->counters, 0, 2 * kMaxDepth * sizeof(Counters), c->stream));
    WF_CUDA(cudaEventRecord(c->t0, c->stream));
    return WF_OK;
}

int end_call(wf_ctx* c) {
    WF_CUDA(cudaEventRecord(c->t1, c->stream));
    c->timing_pending = true;
    c->stats.launches = c->launches;
    c->stats.launches_extend = c->launches_extend;
    c->stats.launches_connect = c->launches_connect;
    c->stats.tail_depth = c->tail_depth;
    return WF_OK;
}

}  // namespace

namespace wf {

namespace {
std::mutex g_mem_mutex;
std::unordered_map<void*, size_t> g_mem_blocks;
uint64_t g_mem_used = 0, g_mem_limit = 0;   // limit 0: none
}  // namespace

cudaError_t dmalloc(void** p, size_t bytes) {
    *p = nullptr;
    std::lock_guard<std::mutex> lock(g_mem_mutex);
    if (g_mem_limit && g_mem_used + bytes > g_mem_limit) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return e;
    }
    g_mem_blocks[*p] = bytes;
    g_mem_used += bytes;
    return cudaSuccess;
}

void dfree(void* p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lock(g_mem_mutex);
        auto it = g_mem_blocks.find(p);
        if (it != g_mem_blocks.end()) {
            g_mem_used -= it->second;
            g_mem_blocks.erase(it);
        }
    }
    cudaFree(p);
}

// Lets entry points defined in other translation units set wf_last_error().
int report_error(int code, const char* msg) { return fail(code, msg); }

int fail_code(int code, const std::string& msg) { return fail(code, msg); }
int ctx_use_device(wf_ctx* c) { return use_device(c); }
cudaStream_t ctx_stream(wf_ctx* c) { return c->stream; }
uint32_t* ctx_status(wf_ctx* c) { return c->status; }
uint32_t ctx_mesh_count(wf_ctx* c) { return (uint32_t)c->meshes.size(); }
uint32_t ctx_tlas_metric(wf_ctx* c) { return c->tlas_metric; }
const TexRef* ctx_texture_table(wf_ctx* c) { return c->tex_table.p; }
uint32_t ctx_texture_count(wf_ctx* c) { return (uint32_t)c->textures.size(); }
TexRef ctx_texture(wf_ctx* c, uint32_t id) {
    if (id == 0 || id > c->textures.size()) return TexRef{nullptr, 0u, 0u};
    const Texture& t = c->textures[id - 1];
    return TexRef{t.d, t.w, t.h};
}
int ctx_take_status(wf_ctx* c) { return take_status(c); }
cudaError_t ctx_h2d(wf_ctx* c, void* dst, const void* src, size_t bytes) { return h2d(c, dst, src, bytes); }
cudaError_t ctx_d2h(wf_ctx* c, void* dst, const void* src, size_t bytes) { return d2h(c, dst, src, bytes); }

bool ctx_mesh(wf_ctx* c, uint32_t mesh, MeshView* out) {
    if (mesh >= c->meshes.size()) return false;
    const Mesh& m = c->meshes[mesh];
    out->tri_count = m.tri_count;
    out->node_count = m.node_count;
    out->tris = m.tris.data();
    out->root_min = m.root_min;
    out->root_max = m.root_max;
    out->d_nodes = m.d_nodes;
    out->d_tris = m.d_tris;
    out->d_stri = m.d_stri;
    return true;
}

int make_instance(wf_ctx* c, uint32_t mesh, const float* l2w, const material_t* mat, uint32_t bsdf, float ior,
                  const char* who, Instance* out) {
    if (!l2w || !mat) return fail(WF_ERR_INVALID, std::string(who) + ": null argument");
    if (mesh >= c->meshes.size()) return fail(WF_ERR_INVALID, std::string(who) + ": unknown mesh");
    if (bsdf > WF_BSDF_DIELECTRIC) return fail(WF_ERR_INVALID, std::string(who) + ": unknown BSDF");
    const uint32_t ids[4] = {mat->base_color_index, mat->normal_index, mat->metallic_roughness_index,
                             mat->emissive_index};
    for (uint32_t id : ids)
        if (id > c->textures.size()) return fail(WF_ERR_INVALID, std::string(who) + ": material names an unknown texture");
    Instance& in = *out;
    in = Instance{};
    in.mesh = mesh;
    std::memcpy(in.l2w, l2w, 64);
    if (!invert4(l2w, in.w2l)) return fail(WF_ERR_INVALID, std::string(who) + ": transform is not invertible");
    in.mat = *mat;
    in.bsdf = bsdf;
    in.ior = ior;
    std::memcpy(in.bi.world_to_local, in.w2l, 64);
    in.bi.bvh_index = mesh;
    // world AABB of the BLAS root box (renderer.cpp:1324-1336), grown from
    // +/-FLT_MAX; the reference grows it from a zeroed box, so its box also
    // always contains the origin.
    const Mesh& m = c->meshes[mesh];
    for (int a = 0; a < 3; ++a) { in.bi.aabb_min[a] = FLT_MAX; in.bi.aabb_max[a] = -FLT_MAX; }
    for (uint32_t i = 0; i < 8; ++i) {
        float corner[3] = {(i & 1) ? m.root_max[0] : m.root_min[0], (i & 2) ? m.root_max[1] : m.root_min[1],
                           (i & 4) ? m.root_max[2] : m.root_min[2]};
        float wc[3];
        glm_mul_point(l2w, corner, wc);
        for (int a = 0; a < 3; ++a) {
            in.bi.aabb_min[a] = (wc[a] < in.bi.aabb_min[a]) ? wc[a] : in.bi.aabb_min[a];
            in.bi.aabb_max[a] = (in.bi.aabb_max[a] < wc[a]) ? wc[a] : in.bi.aabb_max[a];
        }
    }
    return WF_OK;
}

void instance_rows(const Instance& in, float4 ti[4], float4 si[kInstRows], float aabb[6]) {
    std::memcpy(aabb, in.bi.aabb_min, 12);
    std::memcpy(aabb + 3, in.bi.aabb_max, 12);
    float meshf, bsdff;
    std::memcpy(&meshf, &in.mesh, 4);
    std::memcpy(&bsdff, &in.bsdf, 4);
    const float* w = in.w2l;
    ti[0] = make_float4(w[0], w[1], w[2], meshf);
    ti[1] = make_float4(w[4], w[5], w[6], 0.0f);
    ti[2] = make_float4(w[8], w[9], w[10], 0.0f);
    ti[3] = make_float4(w[12], w[13], w[14], 0.0f);
    const float* l = in.l2w;
    const material_t& mt = in.mat;
    si[0] = make_float4(l[0], l[1], l[2], meshf);
    si[1] = make_float4(l[4], l[5], l[6], bsdff);
    si[2] = make_float4(l[8], l[9], l[10], in.ior);
    si[3] = make_float4(l[12], l[13], l[14], mt.roughness_factor);
    si[4] = make_float4(mt.base_color_factor[0], mt.base_color_factor[1], mt.base_color_factor[2], mt.metallic_factor);
    si[5] = make_float4(mt.emissive_strength * mt.emissive_factor[0], mt.emissive_strength * mt.emissive_factor[1],
                        mt.emissive_strength * mt.emissive_factor[2], mt.emissive_strength);
    float tb, tn, tm, te;
    std::memcpy(&tb, &mt.base_color_index, 4);
    std::memcpy(&tn, &mt.normal_index, 4);
    std::memcpy(&tm, &mt.metallic_roughness_index, 4);
    std::memcpy(&te, &mt.emissive_index, 4);
    si[6] = make_float4(tb, tn, tm, te);
}

void append_emitters(const Instance& in, uint32_t inst, const MeshView& m, std::vector<LightTri>& out, float& run) {
    float le[3] = {in.mat.emissive_strength * in.mat.emissive_factor[0],
                   in.mat.emissive_strength * in.mat.emissive_factor[1],
                   in.mat.emissive_strength * in.mat.emissive_factor[2]};
    if (!(le[0] != 0.0f || le[1] != 0.0f || le[2] != 0.0f)) return;
    for (uint32_t t = 0; t < m.tri_count; ++t) {
        float p0[3], p1[3], p2[3];
        hlsl_xform(in.l2w, m.tris[t].v0.position, 1.0f, p0);
        hlsl_xform(in.l2w, m.tris[t].v1.position, 1.0f, p1);
        hlsl_xform(in.l2w, m.tris[t].v2.position, 1.0f, p2);
        float e1[3], e2[3];
        for (int a = 0; a < 3; ++a) { e1[a] = p1[a] - p0[a]; e2[a] = p2[a] - p0[a]; }
        float cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        float len = sqrtf(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        float area = 0.5f * len;
        float il = 1.0f / len;
        run = run + area;
        LightTri L;
        L.p0 = make_float4(p0[0], p0[1], p0[2], area);
        L.e1 = make_float4(e1[0], e1[1], e1[2], run);
        L.e2 = make_float4(e2[0], e2[1], e2[2], 0.0f);
        float key;
        std::memcpy(&key, &inst, 4);
        L.n = make_float4(cr[0] * il, cr[1] * il, cr[2] * il, key);
        float tex;
        std::memcpy(&tex, &in.mat.emissive_index, 4);
        L.le = make_float4(le[0], le[1], le[2], tex);
        L.uv01 = make_float4(m.tris[t].v0.uv[0], m.tris[t].v0.uv[1], m.tris[t].v1.uv[0], m.tris[t].v1.uv[1]);
        L.uv2 = make_float4(m.tris[t].v2.uv[0], m.tris[t].v2.uv[1], 0.0f, 0.0f);
        out.push_back(L);
    }
}
}  // namespace wf

// ============================================================================ C ABI

extern "C" {

const char* wf_status_string(int s) {
    switch (s) {
        case WF_OK: return "ok";
        case WF_ERR_INVALID: return "invalid argument";
        case WF_ERR_OOM: return "out of memory";
        case WF_ERR_CAPACITY: return "capacity exceeded";
        case WF_ERR_TIMEOUT: return "device wait timed out";
        case WF_ERR_STACK: return "traversal stack overflow";
        case WF_ERR_CUDA: return "CUDA error";
        case WF_ERR_STATE: return "call out of order";
        default: return "unknown status";
    }
}

const char* wf_last_error(void) { return g_error.c_str(); }

int wf_abi_version(void) { return WF_ABI_VERSION; }
int wf_checked_build(void) { return WF_CHECKED; }

int wf_set_device_memory_limit(uint64_t bytes) {
    std::lock_guard<std::mutex> lock(g_mem_mutex);
    g_mem_limit = bytes;
    return WF_OK;
}

int wf_get_device_memory_usage(uint64_t* bytes) {
    if (!bytes) return fail(WF_ERR_INVALID, "wf_get_device_memory_usage: null argument");
    std::lock_guard<std::mutex> lock(g_mem_mutex);
    *bytes = g_mem_used;
    return WF_OK;
}

int wf_create(const wf_init_params* p, wf_ctx** out) {
    if (!p || !out) return fail(WF_ERR_INVALID, "wf_create: null argument");
    *out = nullptr;
    if (p->render_width == 0 || p->render_height == 0 || p->render_width > 16384 || p->render_height > 16384)
        return fail(WF_ERR_INVALID, "wf_create: render size must be 1..16384 per side");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(WF_ERR_CUDA, std::string("wf_create: no CUDA device: ") + cudaGetErrorString(e));
    }
    if (p->device < 0 || p->device >= ndev) return fail(WF_ERR_INVALID, "wf_create: device ordinal out of range");
    wf_ctx* c = new wf_ctx();
    c->device = p->device;
    c->width = p->render_width;
    c->height = p->render_height;
    if (p->tlas_metric > 3) {
        delete c;
        return fail(WF_ERR_INVALID, "wf_create: tlas_metric must be 0, 1, 2 or 3");
    }
    c->tlas_metric = p->tlas_metric;
    if (p->blas_layout > 2) {
        delete c;
        return fail(WF_ERR_INVALID, "wf_create: blas_layout must be 0, 1 or 2");
    }
    if (p->instance_bounds > 1) {
        delete c;
        return fail(WF_ERR_INVALID, "wf_create: instance_bounds must be 0 or 1");
    }
    c->blas_layout = p->blas_layout;
    c->instance_bounds = p->instance_bounds;
    const uint64_t npix = (uint64_t)c->width * c->height;
    // default: up to 16 samples of every pixel in flight, at most 2^25 paths
    const uint64_t cap = p->wave_capacity ? p->wave_capacity : std::min<uint64_t>(npix * 16, 1ull << 25);
    c->capacity = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(cap, 1ull << 30));
    int rc = use_device(c);
    if (rc == WF_OK) {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&c->t0) != cudaSuccess || cudaEventCreate(&c->t1) != cudaSuccess) {
            rc = fail(WF_ERR_CUDA, "wf_create: stream/event creation failed");
        }
        for (uint32_t d = 0; rc == WF_OK && d < kMaxDepth; ++d)
            if (cudaEventCreateWithFlags(&c->ev_shade[d], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&c->ev_conn[d], cudaEventDisableTiming) != cudaSuccess)
                rc = fail(WF_ERR_CUDA, "wf_create: event creation failed");
        if (rc == WF_OK && (cudaEventCreateWithFlags(&c->ev_counts, cudaEventDisableTiming) != cudaSuccess ||
                            cudaMallocHost(&c->h_counts, kMaxDepth * sizeof(uint32_t)) != cudaSuccess))
            rc = fail(WF_ERR_CUDA, "wf_create: event / pinned buffer creation failed");
        if (rc == WF_OK && (cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking) != cudaSuccess ||
                            cudaEventCreateWithFlags(&c->img_ready, cudaEventDisableTiming) != cudaSuccess ||
                            cudaEventCreateWithFlags(&c->img_copied, cudaEventDisableTiming) != cudaSuccess))
            rc = fail(WF_ERR_CUDA, "wf_create: copy stream / event creation failed");
    }
    if (rc == WF_OK) rc = dev_alloc(&c->status, 1);
    if (rc == WF_OK) rc = dev_alloc(&c->counters, 2 * kMaxDepth);
    if (rc == WF_OK) rc = dev_alloc(&c->trace_fetch, 1);
    if (rc == WF_OK) rc = dev_alloc(&c->totals, 2 + 2 * kMaxDepth);
    if (rc == WF_OK) {
        cudaMemset(c->status, 0, 4);
        cudaMemset(c->counters, 0, 2 * kMaxDepth * sizeof(Counters));
        cudaMemset(c->totals, 0, (2 + 2 * kMaxDepth) * sizeof(unsigned long long));
        if (cudaDeviceSynchronize() != cudaSuccess) rc = fail(WF_ERR_CUDA, "wf_create: device initialization failed");
    }
    if (rc != WF_OK) {
        wf_destroy(c);
        return rc;
    }
    *out = c;
    return WF_OK;
}

int wf_destroy(wf_ctx* c) {
    if (!c) return WF_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy) cudaStreamSynchronize(c->copy);
    for (Mesh& m : c->meshes) free_mesh(m);
    for (Texture& t : c->textures) dev_free(t.d);
    c->tex_table.release();
    release_buffers(c);
    c->tnodes.release(); c->tinst.release(); c->sinst.release(); c->blas.release(); c->stri.release();
    c->lights.release(); c->aabbs.release(); c->tlas_scratch.release();
    c->tri_albedo.release(); c->inst_tri_offset.release(); c->L_final.release(); c->dimage.release();
    c->g_albedo.release(); c->g_emission.release();
    c->image.release(); c->image_ldr.release(); c->trace_io.release(); c->sort_scratch.release();
    dev_free(c->status); dev_free(c->counters); dev_free(c->totals); dev_free(c->trace_fetch);
    for (EventPair& p : c->events) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    if (c->t0) cudaEventDestroy(c->t0);
    if (c->t1) cudaEventDestroy(c->t1);
    for (uint32_t d = 0; d < kMaxDepth; ++d) {
        if (c->ev_shade[d]) cudaEventDestroy(c->ev_shade[d]);
        if (c->ev_conn[d]) cudaEventDestroy(c->ev_conn[d]);
    }
    if (c->ev_counts) cudaEventDestroy(c->ev_counts);
    if (c->h_counts) cudaFreeHost(c->h_counts);
    if (c->side) { cudaStreamSynchronize(c->side); cudaStreamDestroy(c->side); }
    if (c->copy) { cudaStreamSynchronize(c->copy); cudaStreamDestroy(c->copy); }
    if (c->img_ready) cudaEventDestroy(c->img_ready);
    if (c->img_copied) cudaEventDestroy(c->img_copied);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return WF_OK;
}

int wf_get_stream(wf_ctx* c, void** out) {
    if (!c || !out) return fail(WF_ERR_INVALID, "wf_get_stream: null argument");
    *out = (void*)c->stream;
    return WF_OK;
}

int wf_synchronize(wf_ctx* c) {
    if (!c) return fail(WF_ERR_INVALID, "wf_synchronize: null context");
    int rc = use_device(c);
    if (rc) return rc;
    WF_CUDA(cudaStreamSynchronize(c->stream));
    if (c->img_copy_pending) {
        WF_CUDA(cudaStreamSynchronize(c->copy));
        c->img_copy_pending = false;
    }
    return take_status(c);
}

// ---------------------------------------------------------------------------- meshes

static int add_mesh(wf_ctx* c, Mesh&& m, uint32_t* out_mesh) {
    c->meshes.push_back(std::move(m));
    *out_mesh = (uint32_t)(c->meshes.size() - 1);
    c->scene_ready = false;
    return WF_OK;
}

int wf_mesh_create_prebuilt(wf_ctx* c, const triangle_t* tris, uint32_t n, const void* blob, uint64_t size,
                            uint32_t* out_mesh) {
    if (!c || !tris || !blob || !out_mesh || n == 0) return fail(WF_ERR_INVALID, "wf_mesh_create_prebuilt: bad argument");
    int rc = use_device(c);
    if (rc) return rc;
    Mesh m;
    if ((rc = check_blob(blob, size, n, &m.node_count))) return rc;
    m.tri_count = n;
    m.tris.assign(tris, tris + n);
    m.blob.assign(static_cast<const uint8_t*>(blob), static_cast<const uint8_t*>(blob) + size);
    if ((rc = upload_blob(c, m)) || (rc = upload_shading_tris(c, m)) || (rc = upload_qnodes(c, m)) ||
        (rc = upload_hull(c, m))) {
        free_mesh(m);
        return rc;
    }
    return add_mesh(c, std::move(m), out_mesh);
}

int wf_mesh_create(wf_ctx* c, const vertex_t* vertices, uint32_t nv, const uint32_t* indices, uint32_t ni,
                   const wf_bvh_options* opts, uint32_t* out_mesh) {
    if (!c || !vertices || !indices || !out_mesh || ni < 3 || ni % 3 != 0)
        return fail(WF_ERR_INVALID, "wf_mesh_create: bad argument");
    const uint32_t n = ni / 3;
    std::vector<triangle_t> tris(n);
    std::atomic<bool> bad{false};
    host_parallel(n, 1u << 15, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t t = lo; t < hi; ++t) {
            uint32_t a = indices[3 * t], b = indices[3 * t + 1], d = indices[3 * t + 2];
            if (a >= nv || b >= nv || d >= nv) {
                bad.store(true, std::memory_order_relaxed);
                return;
            }
            tris[t].v0 = vertices[a];
            tris[t].v1 = vertices[b];
            tris[t].v2 = vertices[d];
        }
    });
    if (bad.load()) return fail(WF_ERR_INVALID, "wf_mesh_create: index out of range");
    wf_bvh_options o = opts ? *opts : wf_bvh_options{8, 0, 0};
    int rc = use_device(c);
    if (rc) return rc;
    Mesh m;
    m.tri_count = n;
    m.tris = std::move(tris);
    BvhBuildOut bo;
    if ((rc = gpu_bvh_build(m.tris.data(), n, o, c->stream, &bo))) return fail(rc, bvh_last_error());
    m.node_count = bo.node_count;
    m.d_nodes = bo.d_nodes;
    m.d_tris = bo.d_tris;
    m.blob = std::move(bo.blob);
    std::memcpy(m.root_min, bo.root_min, 12);
    std::memcpy(m.root_max, bo.root_max, 12);
    if ((rc = upload_shading_tris(c, m)) || (rc = upload_qnodes(c, m)) || (rc = upload_hull(c, m))) {
        free_mesh(m);
        return rc;
    }
    return add_mesh(c, std::move(m), out_mesh);
}

int wf_mesh_get_blas(wf_ctx* c, uint32_t mesh, void* out, uint64_t* inout_size) {
    if (!c || !inout_size || mesh >= c->meshes.size()) return fail(WF_ERR_INVALID, "wf_mesh_get_blas: bad argument");
    const std::vector<uint8_t>& b = c->meshes[mesh].blob;
    if (!out || *inout_size < b.size()) {
        *inout_size = b.size();
        return fail(WF_ERR_CAPACITY, "wf_mesh_get_blas: output buffer too small");
    }
    std::memcpy(out, b.data(), b.size());
    *inout_size = b.size();
    return WF_OK;
}

// ---------------------------------------------------------------------------- textures

int wf_texture_create(wf_ctx* c, uint32_t w, uint32_t h, uint32_t format, const void* data, uint32_t* out) {
    if (!c || !data || !out) return fail(WF_ERR_INVALID, "wf_texture_create: null argument");
    if (w == 0 || h == 0 || w > 16384 || h > 16384)
        return fail(WF_ERR_INVALID, "wf_texture_create: width and height must be in [1, 16384]");
    if (format > WF_TEXTURE_BC7_SRGB) return fail(WF_ERR_INVALID, "wf_texture_create: unknown format");
    int rc = use_device(c);
    if (rc) return rc;
    const size_t n = (size_t)w * h;
    const bool srgb = format == WF_TEXTURE_RGBA8_SRGB || format == WF_TEXTURE_BC1_SRGB ||
                      format == WF_TEXTURE_BC2_SRGB || format == WF_TEXTURE_BC3_SRGB || format == WF_TEXTURE_BC7_SRGB;
    float lut[256];
    for (int k = 0; k < 256; ++k) {
        if (srgb) {
            // sRGB transfer function inverse (IEC 61966-2-1), evaluated in double
            const double v = k / 255.0;
            lut[k] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
        } else {
            lut[k] = k / 255.0f;
        }
    }
    Texture t;
    t.w = w;
    t.h = h;
    if ((rc = dev_alloc(&t.d, n))) return rc;
    cudaError_t e = cudaSuccess;
    if (format >= WF_TEXTURE_BC1) {
        // blocks to the device, expanded there (one thread per 4x4 block)
        const uint64_t bytes = bc_bytes(format, w, h);
        uint8_t* d_blocks = nullptr;
        float* d_lut = nullptr;
        if ((rc = dev_alloc(&d_blocks, bytes)) || (rc = dev_alloc(&d_lut, 256))) {
            dev_free(d_blocks);
            dev_free(t.d);
            return rc;
        }
        e = h2d(c, d_blocks, data, bytes);
        if (e == cudaSuccess) e = h2d(c, d_lut, lut, sizeof(lut));
        if (e == cudaSuccess) e = launch_decode_bc(d_blocks, format, w, h, d_lut, t.d, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        dev_free(d_blocks);
        dev_free(d_lut);
    } else {
        std::vector<float4> tx(n);
        const uint8_t* b = static_cast<const uint8_t*>(data);
        if (format == WF_TEXTURE_RGBA32F) {
            std::memcpy(tx.data(), data, n * sizeof(float4));
        } else if (format == WF_TEXTURE_RG8) {
            for (size_t i = 0; i < n; ++i) tx[i] = make_float4(b[2 * i] / 255.0f, b[2 * i + 1] / 255.0f, 0.0f, 1.0f);
        } else {
            for (size_t i = 0; i < n; ++i)
                tx[i] = make_float4(lut[b[4 * i]], lut[b[4 * i + 1]], lut[b[4 * i + 2]], b[4 * i + 3] / 255.0f);
        }
        e = h2d(c, t.d, tx.data(), n * sizeof(float4));
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    if (e != cudaSuccess) {
        dev_free(t.d);
        return fail(WF_ERR_CUDA, std::string("wf_texture_create: ") + cudaGetErrorString(e));
    }
    c->textures.push_back(t);
    std::vector<TexRef> table(c->textures.size() + 1);
    table[0] = TexRef{nullptr, 0u, 0u};
    for (size_t k = 0; k < c->textures.size(); ++k)
        table[k + 1] = TexRef{c->textures[k].d, c->textures[k].w, c->textures[k].h};
    if ((rc = c->tex_table.reserve(table.size()))) return rc;
    WF_CUDA(h2d(c, c->tex_table.p, table.data(), table.size() * sizeof(TexRef)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    *out = (uint32_t)c->textures.size();
    return WF_OK;
}

int wf_texture_read(wf_ctx* c, uint32_t id, float* out, uint64_t count) {
    if (!c || !out || id == 0 || id > c->textures.size()) return fail(WF_ERR_INVALID, "wf_texture_read: bad argument");
    const Texture& t = c->textures[id - 1];
    const uint64_t need = 4ull * t.w * t.h;
    if (count < need) return fail(WF_ERR_CAPACITY, "wf_texture_read: output buffer too small");
    int rc = use_device(c);
    if (rc) return rc;
    WF_CUDA(d2h(c, out, t.d, need * sizeof(float)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    return WF_OK;
}

// ---------------------------------------------------------------------------- scene

int wf_scene_begin(wf_ctx* c, const view_t* view, const wf_env* env) {
    if (!c || !view) return fail(WF_ERR_INVALID, "wf_scene_begin: null argument");
    // begin_scene resets accumulation when the view changes (renderer.cpp:601-604)
    c->view_changed = !c->view_valid || std::memcmp(&c->view.world_to_view, view->world_to_view, 64) != 0;
    c->view = *view;
    c->view_valid = true;
    if (env && env->texture > c->textures.size()) return fail(WF_ERR_INVALID, "wf_scene_begin: unknown env texture");
    if (env) std::memcpy(c->env, env->color, 12);
    else c->env[0] = c->env[1] = c->env[2] = 1.0f;
    c->env_texture = env ? env->texture : 0u;
    c->instances.clear();
    c->in_scene = true;
    c->scene_ready = false;
    c->albedo_set = false;
    return WF_OK;
}

static int submit(wf_ctx* c, uint32_t mesh, const float* l2w, const material_t* mat, uint32_t bsdf, float ior) {
    if (!c) return fail(WF_ERR_INVALID, "wf_instance_submit: null argument");
    if (!c->in_scene) return fail(WF_ERR_STATE, "wf_instance_submit: outside wf_scene_begin/wf_scene_end");
    if (c->instances.size() >= 32768) return fail(WF_ERR_CAPACITY, "wf_instance_submit: more than 32768 instances");
    Instance in{};
    int rc = make_instance(c, mesh, l2w, mat, bsdf, ior, "wf_instance_submit", &in);
    if (rc) return rc;
    c->instances.push_back(in);
    return WF_OK;
}

int wf_instance_submit(wf_ctx* c, uint32_t mesh, const float l2w[16], const material_t* mat) {
    return submit(c, mesh, l2w, mat, WF_BSDF_LAMBERT, 1.5f);
}

int wf_instance_submit_ex(wf_ctx* c, uint32_t mesh, const float l2w[16], const wf_material_ext* mat) {
    if (!mat) return fail(WF_ERR_INVALID, "wf_instance_submit_ex: null material");
    return submit(c, mesh, l2w, &mat->base, mat->bsdf, mat->ior);
}

int wf_instance_submit_many(wf_ctx* c, uint32_t count, const uint32_t* meshes, const float* l2w,
                            const wf_material_ext* mats) {
    if (!c || (count && (!meshes || !l2w || !mats))) return fail(WF_ERR_INVALID, "wf_instance_submit_many: null argument");
    if (!c->in_scene) return fail(WF_ERR_STATE, "wf_instance_submit_many: outside wf_scene_begin/wf_scene_end");
    if (c->instances.size() + count > 32768)
        return fail(WF_ERR_CAPACITY, "wf_instance_submit_many: more than 32768 instances");
    const size_t first = c->instances.size();
    c->instances.reserve(first + count);
    for (uint32_t i = 0; i < count; ++i) {
        Instance in{};
        int rc = make_instance(c, meshes[i], l2w + 16ull * i, &mats[i].base, mats[i].bsdf, mats[i].ior,
                               "wf_instance_submit_many", &in);
        if (rc) {
            c->instances.resize(first);   // all or nothing
            return rc;
        }
        c->instances.push_back(in);
    }
    return WF_OK;
}

int wf_scene_end(wf_ctx* c) {
    if (!c) return fail(WF_ERR_INVALID, "wf_scene_end: null context");
    if (!c->in_scene) return fail(WF_ERR_STATE, "wf_scene_end: no wf_scene_begin");
    int rc = use_device(c);
    if (rc) return rc;
    const uint32_t n = (uint32_t)c->instances.size();
    const uint32_t nm = (uint32_t)c->meshes.size();
    // per-mesh device tables
    {
        std::vector<BlasRef> br(nm ? nm : 1);
        std::vector<const float4*> sp(nm ? nm : 1);
        for (uint32_t i = 0; i < nm; ++i) {
            br[i].nodes = c->meshes[i].d_nodes;
            br[i].tris = c->meshes[i].d_tris;
            br[i].node_count = c->meshes[i].node_count;
            br[i].tri_count = c->meshes[i].tri_count;
            br[i].qnodes = c->meshes[i].d_qnodes;
            br[i].qnode_count = c->meshes[i].qnode_count;
            br[i].root_count = c->meshes[i].root_count;
            sp[i] = c->meshes[i].d_stri;
        }
        if ((rc = c->blas.reserve(br.size())) || (rc = c->stri.reserve(sp.size()))) return rc;
        WF_CUDA(h2d(c, c->blas.p, br.data(), br.size() * sizeof(BlasRef)));
        WF_CUDA(h2d(c, c->stri.p, sp.data(), sp.size() * sizeof(void*)));
    }
    // per-instance data
    std::vector<float> aabbs(6ull * n);
    std::vector<float4> ti(4ull * n), si((size_t)kInstRows * n);
    c->scene_bi.resize(n);
    c->scene_triangles = 0;
    for (uint32_t i = 0; i < n; ++i) c->scene_triangles += c->meshes[c->instances[i].mesh].tri_count;
    for (uint32_t i = 0; i < n; ++i) {
        const Instance& in = c->instances[i];
        c->scene_bi[i] = in.bi;
        instance_rows(in, &ti[4ull * i], &si[(size_t)kInstRows * i], &aabbs[6ull * i]);
    }
    if ((rc = c->tnodes.reserve(2ull * std::max<uint32_t>(2 * n, 1))) || (rc = c->tinst.reserve(ti.size())) ||
        (rc = c->sinst.reserve(si.size())) || (rc = c->aabbs.reserve(aabbs.size())) ||
        (rc = c->tlas_scratch.reserve(tlas_scratch_words(n, c->tlas_metric))))
        return rc;
    WF_CUDA(cudaMemsetAsync(c->tnodes.p, 0, 32, c->stream));
    const bool tight = c->instance_bounds == 1 && n > 0;
    if (tight) {
        std::vector<HullRef> hr(nm ? nm : 1);
        for (uint32_t i = 0; i < nm; ++i) hr[i] = HullRef{c->meshes[i].d_hull, c->meshes[i].hull_count, 0u};
        if ((rc = c->hulls.reserve(hr.size()))) return rc;
        WF_CUDA(h2d(c, c->hulls.p, hr.data(), hr.size() * sizeof(HullRef)));
    }
    if (n) {
        WF_CUDA(h2d(c, c->tinst.p, ti.data(), ti.size() * 16));
        WF_CUDA(h2d(c, c->sinst.p, si.data(), si.size() * 16));
        StageTimer st(c, true, ST_TLAS);
        if (tight) {
            // the instance boxes from the meshes' frontier boxes, on the device
            WF_CUDA(launch_instance_bounds(c->sinst.p, kInstRows, n, c->hulls.p, nm, c->aabbs.p, c->stream));
            c->launches++;
        } else {
            WF_CUDA(h2d(c, c->aabbs.p, aabbs.data(), aabbs.size() * 4));
        }
        WF_CUDA(launch_tlas_build(c->aabbs.p, n, c->tnodes.p, c->tlas_scratch.p, c->tlas_metric, c->stream));
        c->launches++;
    }
    // emitter table (every triangle of every emissive instance, world space)
    std::vector<LightTri> lt;
    float run = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        MeshView mv;
        ctx_mesh(c, c->instances[i].mesh, &mv);
        append_emitters(c->instances[i], i, mv, lt, run);
    }
    c->light_count = (uint32_t)lt.size();
    c->light_total = run;
    if ((rc = c->lights.reserve(lt.size()))) return rc;
    if (!lt.empty())
        WF_CUDA(h2d(c, c->lights.p, lt.data(), lt.size() * sizeof(LightTri)));
    // No wait: the uploads above are staged by the time their calls return and
    // the builds stay queued on the stream ahead of the render.  Device-built
    // boxes reach the host instance records when they are asked for.
    c->bounds_pending = tight;
    c->in_scene = false;
    c->scene_ready = true;
    return WF_OK;
}

// The instance records report the boxes the TLAS was built from: with
// instance_bounds 1 those were computed on the device by wf_scene_end.
static int fetch_bounds(wf_ctx* c) {
    if (!c->bounds_pending) return WF_OK;
    const size_t n = c->scene_bi.size();
    std::vector<float> aabbs(6 * n);
    WF_CUDA(d2h(c, aabbs.data(), c->aabbs.p, aabbs.size() * 4));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i) {
        std::memcpy(c->scene_bi[i].aabb_min, &aabbs[6 * i], 12);
        std::memcpy(c->scene_bi[i].aabb_max, &aabbs[6 * i + 3], 12);
    }
    c->bounds_pending = false;
    return WF_OK;
}

int wf_scene_get_instances(wf_ctx* c, bvh_instance_t* out, uint32_t cap, uint32_t* count) {
    if (!c || !count) return fail(WF_ERR_INVALID, "wf_scene_get_instances: null argument");
    if (!c->scene_ready) return fail(WF_ERR_STATE, "wf_scene_get_instances: no finished scene");
    int rc = use_device(c);
    if (rc || (rc = fetch_bounds(c))) return rc;
    *count = (uint32_t)c->scene_bi.size();
    if (!out || cap < *count) return fail(WF_ERR_CAPACITY, "wf_scene_get_instances: output too small");
    std::memcpy(out, c->scene_bi.data(), c->scene_bi.size() * sizeof(bvh_instance_t));
    return WF_OK;
}

int wf_scene_get_tlas(wf_ctx* c, void* out, uint64_t* inout_size) {
    if (!c || !inout_size) return fail(WF_ERR_INVALID, "wf_scene_get_tlas: null argument");
    if (!c->scene_ready) return fail(WF_ERR_STATE, "wf_scene_get_tlas: no finished scene");
    int rc = use_device(c);
    if (rc || (rc = fetch_bounds(c))) return rc;
    const uint32_t n = (uint32_t)c->scene_bi.size();
    const uint64_t nodes = n ? 2ull * n : 1ull;
    const uint64_t size = 8 + 32 * nodes + 92ull * n;
    if (!out || *inout_size < size) {
        *inout_size = size;
        return fail(WF_ERR_CAPACITY, "wf_scene_get_tlas: output buffer too small");
    }
    uint8_t* o = static_cast<uint8_t*>(out);
    tlas_header_t h{8u, (uint32_t)(8 + 32 * nodes)};
    std::memcpy(o, &h, 8);
    WF_CUDA(d2h(c, o + 8, c->tnodes.p, 32 * nodes));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    if (n) std::memcpy(o + h.instances_offset, c->scene_bi.data(), 92ull * n);
    *inout_size = size;
    return WF_OK;
}

// ---------------------------------------------------------------------------- rendering

}  // extern "C"

namespace {

struct Wave {
    uint32_t s0, k, p0, np;
};

// Waves: whole images of k samples when a wave holds at least one image, else
// pixel ranges of one sample.  Results do not depend on the split: every
// path's random numbers are keyed by (pixel, sample, depth) and the resolve
// adds paths to a pixel in sample order.
std::vector<Wave> plan_waves(uint32_t spp, uint32_t npix, uint32_t wave) {
    std::vector<Wave> waves;
    if (wave >= npix) {
        const uint32_t k = wave / npix;
        for (uint32_t si = 0; si < spp; si += k) waves.push_back({si, std::min(k, spp - si), 0u, npix});
    } else {
        for (uint32_t si = 0; si < spp; ++si)
            for (uint32_t p0 = 0; p0 < npix; p0 += wave) waves.push_back({si, 1u, p0, std::min(wave, npix - p0)});
    }
    return waves;
}

struct Pass {
    WaveParams W;
    SceneRefs S;
    ShadeRefs SH;
    RenderBuffers B;
    bool nee, prof, cnt, mega, fused, serial;
    uint32_t fuse_from;   // separate schedule: from this depth (>= 1) on, as fused; 0 = never
    uint32_t tail_paths;
};

int validate_render(wf_ctx* c, const render_settings_t* s, const wf_render_options* o, const char* who) {
    if (!c || !s || !o) return fail(WF_ERR_INVALID, std::string(who) + ": null argument");
    if (!c->scene_ready) return fail(WF_ERR_STATE, std::string(who) + ": call wf_scene_end first");
    if (s->max_bounces >= kMaxDepth - 1) return fail(WF_ERR_INVALID, std::string(who) + ": max_bounces must be < 15");
    if (o->spp == 0) return fail(WF_ERR_INVALID, std::string(who) + ": spp must be >= 1");
    if (s->render_view_mode >= RENDER_VIEW_MODE_COUNT)
        return fail(WF_ERR_INVALID, std::string(who) + ": unknown render_view_mode");
    if (o->trace_schedule > WF_SCHEDULE_SERIAL)
        return fail(WF_ERR_INVALID, std::string(who) + ": unknown trace_schedule");
    return WF_OK;
}

Pass make_pass(wf_ctx* c, const render_settings_t* s, const wf_render_options* o, uint32_t frame_seed) {
    Pass P{};
    WaveParams& W = P.W;
    for (int k = 0; k < 4; ++k) {
        const float* m1 = c->view.clip_to_view + 4 * k;
        const float* m2 = c->view.view_to_world + 4 * k;
        W.clip_to_view[k] = make_float4(m1[0], m1[1], m1[2], m1[3]);
        W.view_to_world[k] = make_float4(m2[0], m2[1], m2[2], m2[3]);
    }
    W.width = c->width;
    W.height = c->height;
    W.dim_x = c->view.render_dim[0];
    W.dim_y = c->view.render_dim[1];
    W.frame_seed = frame_seed;
    W.max_bounces = s->max_bounces;
    W.nee = o->nee ? 1u : 0u;
    W.rr_start = o->rr_start_depth;
    W.cosine = s->cosine_weighted_diffuse ? 1u : 0u;
    W.env_strength = s->hdr_env_strength;
    std::memcpy(W.env, c->env, 12);
    W.env_tex = TexRef{nullptr, 0u, 0u};
    if (c->env_texture) {
        const Texture& t = c->textures[c->env_texture - 1];
        W.env_tex = TexRef{t.d, t.w, t.h};
    }
    W.view_mode = s->render_view_mode;
    W.far_plane = c->view.far_plane;
    P.S = scene_refs(c);
    P.SH.sinst = c->sinst.p;
    P.SH.stri = c->stri.p;
    P.SH.lights = c->lights.p;
    P.SH.light_count = c->light_count;
    P.SH.light_total = c->light_total;
    P.SH.tri_albedo = c->albedo_set ? c->tri_albedo.p : nullptr;
    P.SH.inst_tri_offset = c->albedo_set ? c->inst_tri_offset.p : nullptr;
    P.SH.textures = c->tex_table.p;
    P.SH.blas = c->blas.p;
    P.SH.inst_count = (uint32_t)c->scene_bi.size();
    P.SH.mesh_count = (uint32_t)c->meshes.size();
    P.SH.texture_count = (uint32_t)c->textures.size();
    P.SH.albedo_count = (uint32_t)std::min<uint64_t>(c->scene_triangles, 0xFFFFFFFFull);
    P.SH.status = c->status;
    P.B = c->B;
    P.B.status = c->status;
    P.B.counters = c->counters;
    P.nee = W.nee && c->light_count > 0;
    P.prof = o->profile != 0;
    P.mega = s->use_wavefront_pathtracing == 0;
    P.cnt = o->count_traffic != 0;
    // traffic counting keeps per-kind counters, so it traces the kinds apart
    P.fused = P.nee && !P.cnt && o->trace_schedule == WF_SCHEDULE_FUSED;
    P.serial = o->trace_schedule == WF_SCHEDULE_SERIAL;
    P.fuse_from = (P.nee && !P.cnt && o->trace_schedule == WF_SCHEDULE_SEPARATE) ? o->fused_from_depth : 0u;
    P.tail_paths = o->tail_paths;
    return P;
}

// One wave through generate -> (extend -> shade -> connect) x depth [-> resolve].
int run_wave(wf_ctx* c, Pass& P, const Wave& wv, uint32_t sample_base, const AdjointRefs& A, bool resolve) {
    WaveParams& W = P.W;
    RenderBuffers& B = P.B;
    W.s0 = sample_base + wv.s0;
    W.nsamples = wv.k;
    W.pix0 = wv.p0;
    W.np = wv.np;
    W.npaths = wv.k * wv.np;
    WF_CUDA(cudaMemsetAsync(B.counts, 0, 4 * kMaxDepth * sizeof(uint32_t), c->stream));
    if (P.mega) {
        // pathtracer.hlsl: every bounce of a path in one thread
        {
            StageTimer t(c, P.prof, ST_EXTEND);
            WF_CUDA(launch_megakernel(P.S, P.SH, B, W, B.counts + 2 * kMaxDepth, c->totals, c->stream));
        }
        c->launches++;
        if (resolve) {
            {
                StageTimer t(c, P.prof, ST_POST);
                WF_CUDA(launch_wave_resolve(B, W, c->stream));
            }
            c->launches++;
        }
        return WF_OK;
    }
    // the depth from which the tail kernel finishes the wave: the first depth
    // whose queue, projected from the last wave's sizes, is below tail_paths
    uint32_t tail = kMaxDepth;
    // whether the extension launch of depth d also traces the shadow rays of d - 1
    auto fused_at = [&](uint32_t d) { return P.fused || (P.fuse_from != 0 && d >= P.fuse_from && !A.g_em_rep); };
    if (c->counts_pending) {
        const cudaError_t q = cudaEventQuery(c->ev_counts);
        if (q == cudaSuccess) {
            std::memcpy(c->last_counts, c->h_counts, sizeof(c->last_counts));
            c->counts_pending = false;
            c->counts_known = c->last_counts[0] > 0;
        } else if (q == cudaErrorNotReady) {
            (void)cudaGetLastError();   // not an error: the copy is still in flight
        } else {
            WF_CUDA(q);
        }
    }
    const bool tail_ok = !P.cnt && A.g_albedo == nullptr && P.tail_paths != 0u && c->counts_known;
    if (tail_ok) {
        const uint64_t limit = P.tail_paths;
        for (uint32_t d = 1; d <= W.max_bounces; ++d) {
            const uint64_t projected = (uint64_t)c->last_counts[d] * W.npaths / c->last_counts[0];
            if (projected < limit) { tail = d; break; }
        }
    }
    // generate.hlsl's camera rays are made inside the depth-0 traversal launch
    // and shade takes the starting path state at depth 0, so no pass writes them
    bool pending = false;   // a connect on the side stream not yet joined
    for (uint32_t d = 0; d <= W.max_bounces; ++d) {
        if (d == tail) {
            // connect at depth d - 1 has added its contributions first (also
            // under the fused schedule: no extension launch of this depth
            // takes them, so they had their own launch)
            if (pending) {
                WF_CUDA(cudaStreamWaitEvent(c->stream, c->ev_conn[d - 1], 0));
                pending = false;
            }
            StageTimer t(c, P.prof, ST_TAIL);
            WF_CUDA(launch_megakernel_tail(P.S, P.SH, B, W, d, B.counts + 2 * kMaxDepth + d, c->totals, c->stream));
            c->launches++;
            c->tail_depth = d;
            break;
        }
        if (d == 0) {
            StageTimer t(c, P.prof, ST_EXTEND, nullptr, (int)d);
            WF_CUDA(launch_extend_camera(P.S, B, W, P.cnt, c->totals, c->stream));
        } else if (fused_at(d)) {
            // the shadow rays of depth d - 1 with the extension rays of depth d
            StageTimer t(c, P.prof, ST_EXTEND, nullptr, (int)d);
            WF_CUDA(launch_trace_pair(P.S, B, d, c->totals, c->stream));
            c->launches_connect++;
        } else {
            StageTimer t(c, P.prof, ST_EXTEND, nullptr, (int)d);
            WF_CUDA(launch_extend(P.S, B, d, W.npaths, P.cnt, c->totals, c->stream));
        }
        // connect at depth d - 1 has added its contributions before shade adds more
        if (pending) {
            WF_CUDA(cudaStreamWaitEvent(c->stream, c->ev_conn[d - 1], 0));
            pending = false;
        }
        {
            StageTimer t(c, P.prof, ST_SHADE);
            WF_CUDA(launch_shade(P.SH, B, W, d, W.npaths, A, c->stream));
        }
        c->launches += 2;
        c->launches_extend++;
        // the shadow rays of depth d: their own launch unless the extension
        // launch of depth d + 1 takes them (the fused schedule, when depth
        // d + 1 is not the tail's)
        if (P.nee && !(fused_at(d + 1) && d + 1 < tail) && d < W.max_bounces) {
            // the shadow rays of depth d overlap the extension rays of depth d + 1
            // (the serial schedule keeps them on the main stream)
            cudaStream_t cs = P.serial ? c->stream : c->side;
            if (!P.serial) {
                WF_CUDA(cudaEventRecord(c->ev_shade[d], c->stream));
                WF_CUDA(cudaStreamWaitEvent(c->side, c->ev_shade[d], 0));
            }
            {
                StageTimer t(c, P.prof, ST_CONNECT, cs, (int)d);
                if (A.g_em_rep) {
                    const AdjConnect adj{A.dimage, P.SH.sinst, A.g_em_rep, A.instances, W.pix0, W.nsamples,
                                         A.inv_spp};
                    WF_CUDA(launch_connect(P.S, B, d, W.npaths, false, c->totals + 1, cs, &adj));
                } else {
                    WF_CUDA(launch_connect(P.S, B, d, W.npaths, P.cnt, c->totals + 1, cs));
                }
            }
            if (!P.serial) {
                WF_CUDA(cudaEventRecord(c->ev_conn[d], c->side));
                pending = true;
            }
            c->launches++;
            c->launches_connect++;
        }
    }
    if (pending) WF_CUDA(cudaStreamWaitEvent(c->stream, c->ev_conn[W.max_bounces - 1], 0));
    WF_CUDA(launch_depth_counts(B.counts, c->totals + 2, c->stream));
    c->launches++;
    if (!P.cnt) {
        WF_CUDA(d2h(c, c->h_counts, B.counts, kMaxDepth * sizeof(uint32_t)));
        WF_CUDA(cudaEventRecord(c->ev_counts, c->stream));
        c->counts_pending = true;
    }
    if (resolve) {
        {
            StageTimer t(c, P.prof, ST_POST);
            WF_CUDA(launch_wave_resolve(B, W, c->stream));
        }
        c->launches++;
    }
    return WF_OK;
}

}  // namespace

extern "C" {

int wf_render(wf_ctx* c, const render_settings_t* s, const wf_render_options* o, uint32_t frame_seed) {
    int rc = validate_render(c, s, o, "wf_render");
    if (rc) return rc;
    if ((rc = use_device(c))) return rc;
    if ((rc = ensure_buffers(c))) return rc;
    if ((rc = begin_call(c, o->count_traffic != 0))) return rc;
    const uint32_t npix = c->width * c->height;
    // a debug view replaces the accumulator every call (post_process.hlsl:44-51)
    if (!s->accumulate || c->view_changed || s->render_view_mode != RENDER_VIEW_MODE_NONE ||
        c->last_view_mode != RENDER_VIEW_MODE_NONE) {
        WF_CUDA(cudaMemsetAsync(c->accum, 0, (size_t)npix * sizeof(float4), c->stream));
        c->accum_samples = 0;
        c->view_changed = false;
    }
    const uint32_t wave = o->wave_paths ? std::min(o->wave_paths, c->capacity) : c->capacity;
    Pass P = make_pass(c, s, o, frame_seed);
    const AdjointRefs none{};
    for (const Wave& wv : plan_waves(o->spp, npix, wave))
        if ((rc = run_wave(c, P, wv, c->accum_samples, none, true))) return rc;
    c->accum_samples += o->spp;
    c->last_view_mode = s->render_view_mode;
    c->last_frame_seed = frame_seed;
    c->stats.paths = (uint64_t)npix * o->spp;
    uint64_t paths = c->stats.paths;
    rc = end_call(c);
    c->stats.paths = paths;
    return rc;
}

int wf_adjoint(wf_ctx* c, const render_settings_t* s, const wf_render_options* o, uint32_t frame_seed,
               const float* dloss_dimage, float* d_albedo, float* d_emission) {
    int rc = validate_render(c, s, o, "wf_adjoint");
    if (rc) return rc;
    if (!dloss_dimage || !d_albedo || !d_emission) return fail(WF_ERR_INVALID, "wf_adjoint: null argument");
    if (s->render_view_mode != RENDER_VIEW_MODE_NONE)
        return fail(WF_ERR_INVALID, "wf_adjoint: differentiates the path-traced image (RENDER_VIEW_MODE_NONE)");
    if (!s->use_wavefront_pathtracing)
        return fail(WF_ERR_INVALID, "wf_adjoint: replays the wavefront stages (use_wavefront_pathtracing = 1)");
    if (!c->albedo_set) return fail(WF_ERR_STATE, "wf_adjoint: set the per-triangle albedo first (wf_scene_set_albedo)");
    if ((rc = use_device(c))) return rc;
    if ((rc = ensure_buffers(c))) return rc;
    const uint32_t npix = c->width * c->height;
    const uint64_t ntri = c->scene_triangles, ninst = c->scene_bi.size();
    // gradient replicas spread the atomics of heavily hit triangles; at most 256 MiB
    uint32_t replicas = 32;
    while (replicas > 1 && (uint64_t)replicas * ntri * sizeof(float4) > (256ull << 20)) replicas >>= 1;
    if ((rc = c->L_final.reserve(c->capacity)) || (rc = c->dimage.reserve(npix)) ||
        (rc = c->g_albedo.reserve((uint64_t)replicas * ntri)) || (rc = c->g_emission.reserve(ninst)) ||
        (rc = c->g_em_rep.reserve(32ull * std::max<uint64_t>(ninst, 1))) ||
        (rc = c->L_comp.reserve(c->capacity)) || (rc = c->L_final_lo.reserve(c->capacity)))
        return rc;
    std::vector<float4> dimg(npix);
    for (uint32_t p = 0; p < npix; ++p)
        dimg[p] = make_float4(dloss_dimage[3ull * p], dloss_dimage[3ull * p + 1], dloss_dimage[3ull * p + 2], 0.0f);
    if ((rc = begin_call(c, false))) return rc;
    WF_CUDA(h2d(c, c->dimage.p, dimg.data(), dimg.size() * sizeof(float4)));
    WF_CUDA(cudaMemsetAsync(c->g_albedo.p, 0, (uint64_t)replicas * ntri * sizeof(float4), c->stream));
    WF_CUDA(cudaMemsetAsync(c->g_emission.p, 0, std::max<uint64_t>(ninst, 1) * sizeof(float), c->stream));
    WF_CUDA(cudaMemsetAsync(c->g_em_rep.p, 0, 32ull * std::max<uint64_t>(ninst, 1) * sizeof(float), c->stream));
    const uint32_t wave = o->wave_paths ? std::min(o->wave_paths, c->capacity) : c->capacity;
    Pass P = make_pass(c, s, o, frame_seed);
    P.fused = false;   // the replay's shadow rays need their own launches (AdjConnectIO)
    P.fuse_from = 0;
    P.cnt = false;
    P.tail_paths = 0;
    P.B.ps_Lc = c->L_comp.p;   // both passes keep the radiance sums' rounding errors
    AdjointRefs A{};
    A.g_em_rep = c->g_em_rep.p;
    A.L_final_lo = c->L_final_lo.p;
    A.instances = (uint32_t)ninst;
    A.L_final = c->L_final.p;
    A.dimage = c->dimage.p;
    A.g_albedo = c->g_albedo.p;
    A.g_emission = c->g_emission.p;
    A.inv_spp = 1.0f / (float)o->spp;
    A.replicas = replicas;
    A.triangles = (uint32_t)ntri;
    const AdjointRefs none{};
    for (const Wave& wv : plan_waves(o->spp, npix, wave)) {
        // forward pass: each path's radiance, kept for the replay
        if ((rc = run_wave(c, P, wv, 0, none, false))) return rc;
        WF_CUDA(cudaMemcpyAsync(c->L_final.p, c->B.ps_L, (size_t)wv.k * wv.np * sizeof(float4),
                                cudaMemcpyDeviceToDevice, c->stream));
        WF_CUDA(cudaMemcpyAsync(c->L_final_lo.p, c->L_comp.p, (size_t)wv.k * wv.np * sizeof(float4),
                                cudaMemcpyDeviceToDevice, c->stream));
        // replay: the same paths from the same seeds, accumulating gradients
        if ((rc = run_wave(c, P, wv, 0, A, false))) return rc;
    }
    WF_CUDA(launch_reduce_replicas(c->g_albedo.p, (uint32_t)ntri, replicas, c->stream));
    c->launches++;
    std::vector<float4> ga(ntri);
    std::vector<float> ge(ninst), gr(32ull * ninst);
    WF_CUDA(d2h(c, ga.data(), c->g_albedo.p, ntri * sizeof(float4)));
    if (ninst) {
        WF_CUDA(d2h(c, ge.data(), c->g_emission.p, ninst * sizeof(float)));
        WF_CUDA(d2h(c, gr.data(), c->g_em_rep.p, gr.size() * sizeof(float)));
    }
    if ((rc = end_call(c))) return rc;
    WF_CUDA(cudaStreamSynchronize(c->stream));
    for (uint64_t t = 0; t < ntri; ++t) {
        d_albedo[3 * t] = ga[t].x;
        d_albedo[3 * t + 1] = ga[t].y;
        d_albedo[3 * t + 2] = ga[t].z;
    }
    for (uint64_t i = 0; i < ninst; ++i) {
        float e = ge[i];
        for (uint32_t r = 0; r < 32; ++r) e = e + gr[(size_t)r * ninst + i];
        d_emission[i] = e;
    }
    c->stats.paths = (uint64_t)npix * o->spp;
    return take_status(c);
}

int wf_scene_triangle_count(wf_ctx* c, uint64_t* out) {
    if (!c || !out) return fail(WF_ERR_INVALID, "wf_scene_triangle_count: null argument");
    if (!c->scene_ready) return fail(WF_ERR_STATE, "wf_scene_triangle_count: no finished scene");
    *out = c->scene_triangles;
    return WF_OK;
}

int wf_scene_set_albedo(wf_ctx* c, const float* rgb, uint64_t count) {
    if (!c) return fail(WF_ERR_INVALID, "wf_scene_set_albedo: null context");
    if (!c->scene_ready) return fail(WF_ERR_STATE, "wf_scene_set_albedo: call wf_scene_end first");
    if (!rgb) {
        c->albedo_set = false;
        return WF_OK;
    }
    if (count != c->scene_triangles) return fail(WF_ERR_INVALID, "wf_scene_set_albedo: count != scene triangle count");
    int rc = use_device(c);
    if (rc) return rc;
    std::vector<float4> a(count);
    for (uint64_t t = 0; t < count; ++t) a[t] = make_float4(rgb[3 * t], rgb[3 * t + 1], rgb[3 * t + 2], 0.0f);
    std::vector<uint32_t> off(c->scene_bi.size());
    uint64_t run = 0;
    for (size_t i = 0; i < off.size(); ++i) {
        off[i] = (uint32_t)run;
        run += c->meshes[c->instances[i].mesh].tri_count;
    }
    if ((rc = c->tri_albedo.reserve(count)) || (rc = c->inst_tri_offset.reserve(off.size()))) return rc;
    WF_CUDA(h2d(c, c->tri_albedo.p, a.data(), count * sizeof(float4)));
    if (!off.empty()) WF_CUDA(h2d(c, c->inst_tri_offset.p, off.data(), off.size() * 4));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    c->albedo_set = true;
    return WF_OK;
}

int wf_scene_set_emission(wf_ctx* c, uint32_t instance, float strength) {
    if (!c) return fail(WF_ERR_INVALID, "wf_scene_set_emission: null context");
    if (!c->scene_ready) return fail(WF_ERR_STATE, "wf_scene_set_emission: call wf_scene_end first");
    if (instance >= c->instances.size()) return fail(WF_ERR_INVALID, "wf_scene_set_emission: unknown instance");
    c->instances[instance].mat.emissive_strength = strength;
    // rebuild the scene's device tables (instance data, TLAS, emitter table)
    c->in_scene = true;
    return wf_scene_end(c);
}

// ---------------------------------------------------------------------------- checkpoint / resume

namespace {
struct AccumHeader {
    char magic[8];              // "WFACCUM1"
    uint32_t width, height, samples, frame_seed;
    view_t view;
};
}  // namespace

int wf_save_accumulator(wf_ctx* c, const char* path) {
    if (!c || !path) return fail(WF_ERR_INVALID, "wf_save_accumulator: null argument");
    if (!c->buffers_ready || !c->view_valid) return fail(WF_ERR_STATE, "wf_save_accumulator: nothing rendered");
    int rc = use_device(c);
    if (rc) return rc;
    const size_t npix = (size_t)c->width * c->height;
    std::vector<float4> acc(npix);
    WF_CUDA(d2h(c, acc.data(), c->accum, npix * sizeof(float4)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    if ((rc = take_status(c))) return rc;
    AccumHeader h{};
    std::memcpy(h.magic, "WFACCUM1", 8);
    h.width = c->width;
    h.height = c->height;
    h.samples = c->accum_samples;
    h.frame_seed = c->last_frame_seed;
    h.view = c->view;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(WF_ERR_INVALID, std::string("wf_save_accumulator: cannot open ") + path);
    const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(acc.data(), sizeof(float4), npix, f) == npix;
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) return fail(WF_ERR_INVALID, std::string("wf_save_accumulator: write failed: ") + path);
    return WF_OK;
}

int wf_load_accumulator(wf_ctx* c, const char* path, uint32_t* out_samples, uint32_t* out_frame_seed) {
    if (!c || !path) return fail(WF_ERR_INVALID, "wf_load_accumulator: null argument");
    if (!c->view_valid) return fail(WF_ERR_STATE, "wf_load_accumulator: call wf_scene_begin with the saved view first");
    int rc = use_device(c);
    if (rc) return rc;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(WF_ERR_INVALID, std::string("wf_load_accumulator: cannot open ") + path);
    AccumHeader h{};
    const size_t npix = (size_t)c->width * c->height;
    std::vector<float4> acc(npix);
    bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, "WFACCUM1", 8) == 0 &&
              h.width == c->width && h.height == c->height;
    if (ok) ok = std::fread(acc.data(), sizeof(float4), npix, f) == npix;
    std::fclose(f);
    if (!ok) return fail(WF_ERR_INVALID, "wf_load_accumulator: not an accumulator of this image size");
    if (std::memcmp(&h.view, &c->view, sizeof(view_t)) != 0)
        return fail(WF_ERR_INVALID, "wf_load_accumulator: the checkpoint was rendered from another view");
    if ((rc = ensure_buffers(c))) return rc;
    WF_CUDA(h2d(c, c->accum, acc.data(), npix * sizeof(float4)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    c->accum_samples = h.samples;
    c->last_frame_seed = h.frame_seed;
    c->view_changed = false;
    c->last_view_mode = RENDER_VIEW_MODE_NONE;
    if (out_samples) *out_samples = h.samples;
    if (out_frame_seed) *out_frame_seed = h.frame_seed;
    return WF_OK;
}

// The resolved image in c->image, once an asynchronous copy out of it has
// finished (the stream waits for it on the device; a new buffer waits on the host).
static int resolve_image(wf_ctx* c, uint64_t npix) {
    if (c->img_copy_pending) {
        if (c->image.cap < npix) {
            WF_CUDA(cudaStreamSynchronize(c->copy));
            c->img_copy_pending = false;
        } else {
            WF_CUDA(cudaStreamWaitEvent(c->stream, c->img_copied, 0));
        }
    }
    int rc = c->image.reserve(npix);
    if (rc) return rc;
    WF_CUDA(launch_resolve(c->accum, (uint32_t)npix, c->image.p, c->stream));
    return WF_OK;
}

int wf_read_image(wf_ctx* c, float* out, uint64_t nfloat) {
    if (!c || !out) return fail(WF_ERR_INVALID, "wf_read_image: null argument");
    const uint64_t npix = (uint64_t)c->width * c->height;
    if (nfloat < 4 * npix) return fail(WF_ERR_CAPACITY, "wf_read_image: output smaller than width*height*4 floats");
    if (!c->buffers_ready) return fail(WF_ERR_STATE, "wf_read_image: nothing rendered");
    int rc = use_device(c);
    if (rc || (rc = resolve_image(c, npix))) return rc;
    WF_CUDA(d2h(c, out, c->image.p, npix * sizeof(float4)));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    return take_status(c);
}

int wf_read_image_async(wf_ctx* c, float* out, uint64_t nfloat) {
    if (!c || !out) return fail(WF_ERR_INVALID, "wf_read_image_async: null argument");
    const uint64_t npix = (uint64_t)c->width * c->height;
    if (nfloat < 4 * npix)
        return fail(WF_ERR_CAPACITY, "wf_read_image_async: output smaller than width*height*4 floats");
    if (!c->buffers_ready) return fail(WF_ERR_STATE, "wf_read_image_async: nothing rendered");
    int rc = use_device(c);
    if (rc || (rc = resolve_image(c, npix))) return rc;
    WF_CUDA(cudaEventRecord(c->img_ready, c->stream));
    WF_CUDA(cudaStreamWaitEvent(c->copy, c->img_ready, 0));
    c->d2h_bytes += npix * sizeof(float4);
    WF_CUDA(cudaMemcpyAsync(out, c->image.p, npix * sizeof(float4), cudaMemcpyDeviceToHost, c->copy));
    WF_CUDA(cudaEventRecord(c->img_copied, c->copy));
    c->img_copy_pending = true;
    return WF_OK;
}

int wf_read_image_ldr(wf_ctx* c, uint8_t* out, uint64_t nbytes) {
    if (!c || !out) return fail(WF_ERR_INVALID, "wf_read_image_ldr: null argument");
    const uint64_t npix = (uint64_t)c->width * c->height;
    if (nbytes < 4 * npix) return fail(WF_ERR_CAPACITY, "wf_read_image_ldr: output smaller than width*height*4 bytes");
    if (!c->buffers_ready) return fail(WF_ERR_STATE, "wf_read_image_ldr: nothing rendered");
    int rc = use_device(c);
    if (rc) return rc;
    if ((rc = c->image_ldr.reserve(npix))) return rc;
    WF_CUDA(launch_post(c->accum, (uint32_t)npix, c->last_view_mode, c->image_ldr.p, c->stream));
    WF_CUDA(d2h(c, out, c->image_ldr.p, npix * 4));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    return take_status(c);
}

int wf_get_stats(wf_ctx* c, wf_stats* out) {
    if (!c || !out) return fail(WF_ERR_INVALID, "wf_get_stats: null argument");
    int rc = use_device(c);
    if (rc) return rc;
    if ((rc = finish_timing(c))) return rc;
    *out = c->stats;
    out->h2d_bytes = c->h2d_bytes;
    out->d2h_bytes = c->d2h_bytes;
    return WF_OK;
}

// ---------------------------------------------------------------------------- ray queries

int wf_trace_device(wf_ctx* c, const RayDesc2* rays, uint32_t n, hit_result_t* hits, uint32_t flags) {
    if (!c || (n && (!rays || !hits))) return fail(WF_ERR_INVALID, "wf_trace_device: null argument");
    if ((reinterpret_cast<uintptr_t>(rays) & 15u) != 0 || (reinterpret_cast<uintptr_t>(hits) & 3u) != 0)
        return fail(WF_ERR_INVALID, "wf_trace_device: rays must be 16-byte and hits 4-byte aligned");
    if (flags & ~15u) return fail(WF_ERR_INVALID, "wf_trace_device: unknown flags");
    if (!c->scene_ready) return fail(WF_ERR_STATE, "wf_trace_device: call wf_scene_end first");
    int rc = use_device(c);
    if (rc) return rc;
    const bool count = (flags & WF_TRACE_COUNT_TRAFFIC) != 0;
    if ((rc = begin_call(c, count))) return rc;
    WF_CUDA(cudaMemsetAsync(c->trace_fetch, 0, 4, c->stream));
    const uint32_t *perm = nullptr, *varied = nullptr;
    if ((flags & WF_TRACE_REORDER) && n) {
        if ((rc = c->sort_scratch.reserve(reorder_scratch_words(n)))) return rc;
        StageTimer t(c, true, ST_EXTEND);
        WF_CUDA(launch_reorder_rays(reinterpret_cast<const float4*>(rays), n, c->tnodes.p, !c->scene_bi.empty(),
                                    c->sort_scratch.p, &perm, &varied, c->stream));
        c->launches += 2 + 3 * 5;   // keys, the decision, then upsweep + 3 scan kernels + downsweep per pass
    }
    {
        StageTimer t(c, true, ST_EXTEND);
        WF_CUDA(launch_trace_aos(scene_refs(c), rays, n, hits, flags & 3u, count, c->trace_fetch, c->status,
                                 c->counters, c->stream, perm, varied));
    }
    c->launches++;
    c->launches_extend++;
    c->stats.rays_extend = n;
    rc = end_call(c);
    return rc;
}

int wf_trace(wf_ctx* c, const RayDesc2* rays, uint32_t n, hit_result_t* hits, uint32_t flags) {
    if (!c || (n && (!rays || !hits))) return fail(WF_ERR_INVALID, "wf_trace: null argument");
    if (flags & ~15u) return fail(WF_ERR_INVALID, "wf_trace: unknown flags");
    if (!c->scene_ready) return fail(WF_ERR_STATE, "wf_trace: call wf_scene_end first");
    if (n == 0) return WF_OK;
    int rc = use_device(c);
    if (rc) return rc;
    const size_t rb = 32ull * n, hb = 20ull * n;
    if ((rc = c->trace_io.reserve(rb + ((hb + 15) & ~size_t(15))))) return rc;
    RayDesc2* dr = reinterpret_cast<RayDesc2*>(c->trace_io.p);
    hit_result_t* dh = reinterpret_cast<hit_result_t*>(c->trace_io.p + rb);
    WF_CUDA(h2d(c, dr, rays, rb));
    if ((rc = wf_trace_device(c, dr, n, dh, flags))) return rc;
    WF_CUDA(d2h(c, hits, dh, hb));
    WF_CUDA(cudaStreamSynchronize(c->stream));
    return take_status(c);
}

// ---------------------------------------------------------------------------- builders

int wf_bvh_build(wf_ctx* c, const triangle_t* tris, uint32_t n, const wf_bvh_options* opts, void* out,
                 uint64_t* inout_size) {
    if (!c || !tris || !inout_size || n == 0) return fail(WF_ERR_INVALID, "wf_bvh_build: bad argument");
    int rc = use_device(c);
    if (rc) return rc;
    wf_bvh_options o = opts ? *opts : wf_bvh_options{8, 0, 0};
    BvhBuildOut bo;
    bo.keep_device = false;
    bo.dst = static_cast<uint8_t*>(out);
    bo.dst_capacity = out ? *inout_size : 0;
    if ((rc = gpu_bvh_build(tris, n, o, c->stream, &bo))) return fail(rc, bvh_last_error());
    *inout_size = bo.blob_size;
    if (!bo.in_dst) return fail(WF_ERR_CAPACITY, "wf_bvh_build: output buffer too small");
    return WF_OK;
}

int wf_tlas_build(wf_ctx* c, const bvh_instance_t* inst, uint32_t n, void* out, uint64_t* inout_size) {
    if (!c || !inout_size || (n && !inst)) return fail(WF_ERR_INVALID, "wf_tlas_build: bad argument");
    if (n > 32768) return fail(WF_ERR_CAPACITY, "wf_tlas_build: more than 32768 instances");
    const uint64_t nodes = n ? 2ull * n : 1ull;
    const uint64_t size = 8 + 32 * nodes + 92ull * n;
    if (!out || *inout_size < size) {
        *inout_size = size;
        return fail(WF_ERR_CAPACITY, "wf_tlas_build: output buffer too small");
    }
    int rc = use_device(c);
    if (rc) return rc;
    std::vector<float> aabbs(6ull * n);
    for (uint32_t i = 0; i < n; ++i) {
        std::memcpy(&aabbs[6ull * i], inst[i].aabb_min, 12);
        std::memcpy(&aabbs[6ull * i + 3], inst[i].aabb_max, 12);
    }
    float* d_aabbs = nullptr;
    float4* d_nodes = nullptr;
    uint32_t* d_scratch = nullptr;
    if ((rc = dev_alloc(&d_aabbs, aabbs.size())) || (rc = dev_alloc(&d_nodes, 2 * nodes)) ||
        (rc = dev_alloc(&d_scratch, tlas_scratch_words(n, c->tlas_metric)))) {
        dev_free(d_aabbs); dev_free(d_nodes); dev_free(d_scratch);
        return rc;
    }
    cudaError_t e = cudaMemsetAsync(d_nodes, 0, 32 * nodes, c->stream);
    if (e == cudaSuccess && n)
        e = h2d(c, d_aabbs, aabbs.data(), aabbs.size() * 4);
    if (e == cudaSuccess) e = launch_tlas_build(d_aabbs, n, d_nodes, d_scratch, c->tlas_metric, c->stream);
    uint8_t* o = static_cast<uint8_t*>(out);
    if (e == cudaSuccess) e = d2h(c, o + 8, d_nodes, 32 * nodes);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    dev_free(d_aabbs); dev_free(d_nodes); dev_free(d_scratch);
    if (e != cudaSuccess) return fail(WF_ERR_CUDA, std::string("wf_tlas_build: ") + cudaGetErrorString(e));
    tlas_header_t h{8u, (uint32_t)(8 + 32 * nodes)};
    std::memcpy(o, &h, 8);
    if (n) std::memcpy(o + h.instances_offset, inst, 92ull * n);
    *inout_size = size;
    return WF_OK;
}

}  // extern "C"
