/* Stand-in for <Windows.h> so the reference's headers compile with g++ on Linux.
 * The reference uses only _aligned_malloc/_aligned_free and the MSVC keyword __assume.
 * Test infrastructure: part of the oracle's reference build, never linked into the product. */
#pragma once
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>
static inline void* _aligned_malloc(std::size_t size, std::size_t align) {
    void* p = nullptr;
    if (align < sizeof(void*)) align = sizeof(void*);
    if (posix_memalign(&p, align, size ? size : align) != 0) return nullptr;
    return p;
}
static inline void _aligned_free(void* p) { std::free(p); }
#define __assume(x) ((void)0)
