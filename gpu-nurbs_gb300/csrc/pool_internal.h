// Pool functions used by the server (not part of the C-ABI).
#pragma once
#include <cstddef>

#include "gpu_nurbs.h"

namespace gnurbs {
bool pool_is_live(nurbs_pool_t P, int id);
// Frees a surface without waiting on any stream: the caller guarantees no queued work reads it.
int pool_release_surface(nurbs_pool_t P, int id);
// Device memory carved from the pool's budget (nullptr when it does not fit).
char* pool_arena_alloc(nurbs_pool_t P, size_t bytes, size_t* off);
void pool_arena_release(nurbs_pool_t P, size_t off, size_t bytes);
}  // namespace gnurbs
