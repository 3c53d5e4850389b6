/*
 * C entry points around the reference's own builders, compiled from the
 * reference sources by oracle/build_ref.sh into oracle/_ref/libref_bvh.so.
 * TEST INFRASTRUCTURE ONLY: pins the oracle's builder restatement (and the
 * golden blobs) to the reference's bvh_builder_t / tlas_builder_t.
 * Output: [header | extract()] as renderer.cpp:113-155 and :649-652 upload it.
 */
#include <cstring>
#include "core/memory/memory_arena.h"
#include "renderer/bvh/bvh_builder.h"
#include "renderer/bvh/tlas_builder.h"

extern "C" int ref_bvh_build(const void* triangles, uint32_t count, uint32_t interval_count,
                             uint32_t subdivide_single_prim, uint8_t* out, uint64_t* inout_size) {
    memory_arena_t arena;
    bvh_builder_t builder{};
    bvh_builder_t::build_args_t args{};
    args.triangles = static_cast<const triangle_t*>(triangles);
    args.triangle_count = count;
    args.options.interval_count = interval_count;
    args.options.subdivide_single_prim = subdivide_single_prim != 0;
    builder.build(arena, args);
    bvh_t bvh;
    uint64_t size = 0;
    builder.extract(arena, bvh, size);
    uint64_t total = sizeof(bvh_header_t) + size;
    int rc = 0;
    if (!out || *inout_size < total) {
        rc = -3;
    } else {
        std::memcpy(out, &bvh.header, sizeof(bvh_header_t));
        std::memcpy(out + sizeof(bvh_header_t), bvh.data, size);
    }
    *inout_size = total;
    memory_arena::release(arena);
    return rc;
}

/* The reference keeps its merge list in a 256-entry stack array
 * (tlas_builder.cpp:14), so only up to 256 instances are accepted here. */
extern "C" int ref_tlas_build(const void* instances, uint32_t count, uint8_t* out, uint64_t* inout_size) {
    if (count > 256) return -1;
    memory_arena_t arena;
    tlas_builder_t builder{};
    builder.build(arena, const_cast<bvh_instance_t*>(static_cast<const bvh_instance_t*>(instances)), count);
    tlas_t tlas;
    uint64_t size = 0;
    builder.extract(arena, tlas, size);
    uint64_t total = sizeof(tlas_header_t) + size;
    int rc = 0;
    if (!out || *inout_size < total) {
        rc = -3;
    } else {
        std::memcpy(out, &tlas.header, sizeof(tlas_header_t));
        std::memcpy(out + sizeof(tlas_header_t), tlas.data, size);
    }
    *inout_size = total;
    memory_arena::release(arena);
    return rc;
}
