// Stand-in for TBB's scalable allocator: plain malloc/free.
#pragma once
#include <cstdlib>
inline void *scalable_malloc(std::size_t n) { return std::malloc(n); }
inline void scalable_free(void *p) { std::free(p); }
