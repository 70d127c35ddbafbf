/* Forced-include shim for compiling the reference with g++ (test infrastructure only).
 * The reference issues 256/128-bit *aligned* loads and stores at offsets that are not
 * 32-byte aligned (MSVC emits unaligned moves for them, g++ emits vmovaps which faults).
 * Mapping them to the unaligned forms changes no arithmetic. */
#pragma once
#include <immintrin.h>
#define _mm256_load_ps _mm256_loadu_ps
#define _mm256_store_ps _mm256_storeu_ps
#define _mm256_load_pd _mm256_loadu_pd
#define _mm256_store_pd _mm256_storeu_pd
#define _mm_load_ps _mm_loadu_ps
#define _mm_store_ps _mm_storeu_ps
#define _mm_load_pd _mm_loadu_pd
#define _mm_store_pd _mm_storeu_pd
