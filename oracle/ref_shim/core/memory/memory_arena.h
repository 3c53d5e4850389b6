/*
 * Stand-in for the reference's core/memory/memory_arena.h, used only when the
 * reference's own BVH/TLAS builder sources are compiled into the oracle's
 * cross-check library (oracle/build_ref.sh).  It provides the two allocation
 * macros those sources use, backed by the C heap; the driver releases every
 * block after extracting a blob.
 */
#pragma once
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

struct memory_arena_t {
    std::vector<void*> blocks;
};

namespace memory_arena {
inline void* alloc(memory_arena_t& arena, uint64_t size, uint64_t align) {
    if (align < sizeof(void*)) align = sizeof(void*);
    uint64_t rounded = (size + align - 1) / align * align;
    void* p = std::aligned_alloc(align, rounded ? rounded : align);
    arena.blocks.push_back(p);
    return p;
}
inline void* alloc_zero(memory_arena_t& arena, uint64_t size, uint64_t align) {
    void* p = alloc(arena, size, align);
    std::memset(p, 0, size);
    return p;
}
inline void release(memory_arena_t& arena) {
    for (void* p : arena.blocks) std::free(p);
    arena.blocks.clear();
}
}  // namespace memory_arena

#define ARENA_ALLOC(arena, size, align) memory_arena::alloc(arena, size, align)
#define ARENA_ALLOC_ZERO(arena, size, align) memory_arena::alloc_zero(arena, size, align)
#define ARENA_ALLOC_ARRAY(arena, type, count) (type*)memory_arena::alloc((arena), sizeof(type) * (count), alignof(type))
#define ARENA_ALLOC_ARRAY_ZERO(arena, type, count) \
    (type*)memory_arena::alloc_zero((arena), sizeof(type) * (count), alignof(type))
