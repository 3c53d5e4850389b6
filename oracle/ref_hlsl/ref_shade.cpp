/*
 * ref_shade.cpp — the reference's wavefront shade stage, compiled from its
 * own shader text: source/renderer/shaders/wavefront/shade.hlsl:42-174 with
 * the helpers it includes (common.hlsl, sample.hlsl, material.hlsl,
 * brdf.hlsl) and RAYTRACING_MODE_SOFTWARE = 0, as renderer.cpp:394-416
 * compiles the wavefront kernels (hardware-ray make_ray /
 * make_primary_ray, common.hlsl:171-195).
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref/libref_hlsl.so, built by
 * oracle/build_ref.sh).
 *
 * refh_render runs the reference's wavefront loop (renderer.cpp:752-938) for
 * one frame, one thread at a time in dispatch order:
 *   clear_buffers + generate (clear_buffers.hlsl:21-39, generate.hlsl:12-20;
 *     restated here: pixel i = (i mod W, i div W), energy 0, throughput 1,
 *     ray_counts = {W*H, 0, ...}, rays[i] = make_primary_ray — the compiled
 *     reference function);
 *   for depth d = 0 .. max_bounces:
 *     extend: refh_trace (ref_trace.cpp, the software query);
 *     shade:  the compiled shade main for dispatch ids 0 .. ray_counts[d]-1,
 *             pixel coordinates ping-ponged by depth parity as
 *             renderer.cpp:908-909 binds them.
 * Executed in dispatch order, the stage's read of rays[id] and append to
 * rays[slot] (shade.hlsl:52,167) never overwrite an unread ray (slot <= id).
 *
 * Seeds: shade.hlsl:80 seeds each thread with random_seed + dispatch id.
 * To compare paths with the oracle and the GPU library, which key every
 * path's stream by (pixel, sample, depth) instead, the driver sets
 * random_seed = orc_path_seed(frame_seed, pixel, sample, d) - id before each
 * thread, so the shader's own seed expression yields the keyed seed.
 */
#include "hlsl_shim.h"

#define RAYTRACING_MODE_SOFTWARE 0
namespace ref_hw {
using namespace hlsl_shim;
#include "wavefront/shade.hlsl"
}  // namespace ref_hw

#include <string.h>
#include <vector>

using namespace hlsl_shim;

extern "C" {
int refh_trace(uint32_t tlas_slot, const void* rays, uint32_t n, void* hits);
uint32_t orc_path_seed(uint32_t frame_seed, uint32_t pixel, uint32_t sample, uint32_t depth);
}

static_assert(sizeof(ref_hw::view_t) == 272 && sizeof(ref_hw::render_settings_t) == 28, "ABI layout");
static_assert(sizeof(ref_hw::instance_data_t) == 184 && sizeof(ref_hw::triangle_t) == 144, "ABI layout");

namespace {
// Heap slots the driver's own wavefront buffers occupy.
enum : uint32_t {
    kSlotCounts = 8100,
    kSlotRays,
    kSlotHits,
    kSlotEnergy,
    kSlotThroughput,
    kSlotPixelsA,
    kSlotPixelsB,
};
}  // namespace

extern "C" {

typedef struct refh_frame {
    const void* view;        /* view_t */
    const void* settings;    /* render_settings_t */
    uint32_t width, height;
    uint32_t frame_seed, sample;
    uint32_t tlas_slot;      /* TLAS blob; BLAS blobs in the slots named by bvh_index */
    uint32_t instances_slot; /* instance_data_t[]; triangle buffers in the slots named by triangle_buffer_idx */
    uint32_t env_slot, env_width, env_height;
} refh_frame;

/* make_primary_ray (hardware-ray variant, common.hlsl:182-195). */
void refh_primary_ray(const void* view, uint32_t px, uint32_t py, void* out) {
    memcpy((void*)&ref_hw::cb_view, view, sizeof(ref_hw::view_t));
    ref_hw::RayDesc2 r = ref_hw::make_primary_ray(uint2(px, py), ref_hw::cb_view.render_dim);
    memcpy(out, (const void*)&r, 32);
}

/* cosine_weighted_hemisphere_sample / uniform_hemisphere_sample
 * (sample.hlsl:29-54) with create_orthonormal_basis (:13-27). */
void refh_hemisphere_sample(const float n[3], float r0, float r1, int cosine, float out[3]) {
    float3 N(n[0], n[1], n[2]);
    float3 L = cosine ? ref_hw::cosine_weighted_hemisphere_sample(N, float2(r0, r1))
                      : ref_hw::uniform_hemisphere_sample(N, float2(r0, r1));
    out[0] = L.x; out[1] = L.y; out[2] = L.z;
}

/* int_to_color (common.hlsl:285-295), direction_to_equirect_uv (sample.hlsl:4-11). */
void refh_int_to_color(uint32_t v, float out[3]) {
    float3 c = ref_hw::int_to_color(v);
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}
void refh_equirect_uv(const float d[3], float out[2]) {
    float2 uv = ref_hw::direction_to_equirect_uv(float3(d[0], d[1], d[2]));
    out[0] = uv.x; out[1] = uv.y;
}

/* One frame of the wavefront loop (see the file comment).  energy_out:
 * width*height RGBA floats (the energy texture after the last depth);
 * counts_out: the 9 ray counts.  Returns 0. */
int refh_render(const refh_frame* F, float* energy_out, uint32_t* counts_out) {
    const uint32_t W = F->width, H = F->height, n = W * H;
    ref_hw::render_settings_t settings;
    memcpy((void*)&settings, F->settings, sizeof(settings));
    memcpy((void*)&ref_hw::cb_settings, F->settings, sizeof(settings));
    memcpy((void*)&ref_hw::cb_view, F->view, sizeof(ref_hw::view_t));

    std::vector<uint32_t> counts(9, 0u);
    std::vector<uint8_t> rays(32ull * n), hits(20ull * n), pix_a(8ull * n), pix_b(8ull * n);
    std::vector<float> energy(4ull * n), throughput(4ull * n);
    g_heap[kSlotCounts] = descriptor{(uint8_t*)counts.data(), 36u, 0u, 0u};
    g_heap[kSlotRays] = descriptor{rays.data(), (uint32_t)rays.size(), 0u, 0u};
    g_heap[kSlotHits] = descriptor{hits.data(), (uint32_t)hits.size(), 0u, 0u};
    g_heap[kSlotPixelsA] = descriptor{pix_a.data(), (uint32_t)pix_a.size(), 0u, 0u};
    g_heap[kSlotPixelsB] = descriptor{pix_b.data(), (uint32_t)pix_b.size(), 0u, 0u};
    g_heap[kSlotEnergy] = descriptor{(uint8_t*)energy.data(), 16u * n, W, H};
    g_heap[kSlotThroughput] = descriptor{(uint8_t*)throughput.data(), 16u * n, W, H};

    // clear_buffers + generate
    counts[0] = n;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t px[2] = {i % W, i / W};
        memcpy(&pix_a[8ull * i], px, 8);
        for (int k = 0; k < 3; ++k) { energy[4ull * i + k] = 0.0f; throughput[4ull * i + k] = 1.0f; }
        ref_hw::RayDesc2 r = ref_hw::make_primary_ray(uint2(px[0], px[1]), ref_hw::cb_view.render_dim);
        memcpy(&rays[32ull * i], (const void*)&r, 32);
    }

    for (uint32_t d = 0; d <= settings.max_bounces && d < 9u; ++d) {
        const uint32_t count = counts[d];
        refh_trace(F->tlas_slot, rays.data(), count, hits.data());
        ref_hw::shader_input_t& cb = ref_hw::cb_in;
        cb.buffer_ray_counts_index = kSlotCounts;
        cb.buffer_rays_index = kSlotRays;
        cb.buffer_hit_results_index = kSlotHits;
        cb.texture_energy_index = kSlotEnergy;
        cb.texture_throughput_index = kSlotThroughput;
        cb.buffer_pixel_coords_index = (d % 2 == 0) ? kSlotPixelsA : kSlotPixelsB;
        cb.buffer_pixel_coords_two_index = (d % 2 == 0) ? kSlotPixelsB : kSlotPixelsA;
        cb.buffer_instances_index = F->instances_slot;
        cb.texture_hdr_env_index = F->env_slot;
        cb.texture_hdr_env_width = F->env_width;
        cb.texture_hdr_env_height = F->env_height;
        cb.recursion_depth = d;
        const std::vector<uint8_t>& pin = (d % 2 == 0) ? pix_a : pix_b;
        for (uint32_t id = 0; id < count; ++id) {
            uint32_t px[2];
            memcpy(px, &pin[8ull * id], 8);
            cb.random_seed = orc_path_seed(F->frame_seed, px[1] * W + px[0], F->sample, d) - id;
            ref_hw::main(uint3(id, 0u, 0u));
        }
    }
    memcpy(energy_out, energy.data(), 16ull * n);
    memcpy(counts_out, counts.data(), 36);
    for (uint32_t s = kSlotCounts; s <= kSlotPixelsB; ++s) g_heap[s] = descriptor{nullptr, 0u, 0u, 0u};
    return 0;
}

}  // extern "C"
