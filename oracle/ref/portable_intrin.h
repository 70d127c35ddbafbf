/* Portable stand-in for <immintrin.h>, covering exactly the AVX/AVX2/FMA/SSE intrinsics that the
 * reference FFT (kjear/fyFFT) uses, so that its unmodified headers compile and run on hosts
 * without AVX2 (the aarch64 Grace host of the GPU machines).
 *
 * TEST INFRASTRUCTURE: part of the reference build recipe (oracle/ref/build_ref.sh
 * --emulate), used only to time the reference's own algorithm as the CPU baseline and to pin
 * the oracle.  The product never includes it.
 *
 * Written from the published semantics of each intrinsic (Intel Intrinsics Guide): lane
 * order, immediate-operand encodings, fused multiply-add rounding, truncating conversion
 * with the 0x80000000 "integer indefinite" result.  Every operation is exact with respect to
 * the instruction it stands for, so an emulated build computes bit-identical results to a
 * native AVX2 build when both are compiled with -ffp-contract=off (tested by
 * tests/test_ref_emulation.py on x86-64).  Types are GCC vector extensions; on aarch64 the
 * fused multiply-adds use NEON vfmaq_f32 (one fused operation per lane, like vfmadd*ps).
 */
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>
#if defined(__aarch64__)
#include <arm_neon.h>
#endif

#define FYEMU_INLINE static inline __attribute__((always_inline))

typedef float __m256 __attribute__((vector_size(32), __may_alias__));
typedef double __m256d __attribute__((vector_size(32), __may_alias__));
typedef long long __m256i __attribute__((vector_size(32), __may_alias__));
typedef float __m128 __attribute__((vector_size(16), __may_alias__));
typedef double __m128d __attribute__((vector_size(16), __may_alias__));
typedef long long __m128i __attribute__((vector_size(16), __may_alias__));
typedef int __m64 __attribute__((vector_size(8), __may_alias__));

typedef int fyemu_v8si __attribute__((vector_size(32)));
typedef unsigned int fyemu_v8su __attribute__((vector_size(32)));
typedef int fyemu_v4si __attribute__((vector_size(16)));
typedef unsigned int fyemu_v4su __attribute__((vector_size(16)));
typedef float fyemu_v4sf __attribute__((vector_size(16)));
typedef long long fyemu_v4di __attribute__((vector_size(32)));

#define _MM_SHUFFLE(z, y, x, w) (((z) << 6) | ((y) << 4) | ((x) << 2) | (w))

/* ---------------------------------------------------------------------------------------
 * MXCSR: the reference only saves and restores it; kept per thread, no effect on arithmetic.
 * ------------------------------------------------------------------------------------- */
static __thread unsigned int fyemu_csr = 0x1F80u;
FYEMU_INLINE unsigned int _mm_getcsr(void) { return fyemu_csr; }
FYEMU_INLINE void _mm_setcsr(unsigned int v) { fyemu_csr = v; }

/* ---------------------------------------------------------------------------------------
 * 256-bit float
 * ------------------------------------------------------------------------------------- */
FYEMU_INLINE __m256 _mm256_loadu_ps(const float* p) { __m256 r; memcpy(&r, p, 32); return r; }
FYEMU_INLINE __m256 _mm256_load_ps(const float* p) { return _mm256_loadu_ps(p); }
FYEMU_INLINE void _mm256_storeu_ps(float* p, __m256 a) { memcpy(p, &a, 32); }
FYEMU_INLINE void _mm256_store_ps(float* p, __m256 a) { _mm256_storeu_ps(p, a); }

FYEMU_INLINE __m256 _mm256_add_ps(__m256 a, __m256 b) { return a + b; }
FYEMU_INLINE __m256 _mm256_sub_ps(__m256 a, __m256 b) { return a - b; }
FYEMU_INLINE __m256 _mm256_mul_ps(__m256 a, __m256 b) { return a * b; }
FYEMU_INLINE __m256 _mm256_xor_ps(__m256 a, __m256 b) { return (__m256)((fyemu_v8su)a ^ (fyemu_v8su)b); }
FYEMU_INLINE __m256 _mm256_and_ps(__m256 a, __m256 b) { return (__m256)((fyemu_v8su)a & (fyemu_v8su)b); }

FYEMU_INLINE __m256 _mm256_set1_ps(float v) { return (__m256){v, v, v, v, v, v, v, v}; }
FYEMU_INLINE __m256 _mm256_setr_ps(float e0, float e1, float e2, float e3, float e4, float e5, float e6, float e7) {
    return (__m256){e0, e1, e2, e3, e4, e5, e6, e7};
}
FYEMU_INLINE __m256 _mm256_setzero_ps(void) { return (__m256){0, 0, 0, 0, 0, 0, 0, 0}; }

/* even lanes a - b, odd lanes a + b */
FYEMU_INLINE __m256 _mm256_addsub_ps(__m256 a, __m256 b) {
    __m256 s = a + b, d = a - b;
    return __builtin_shuffle(d, s, (fyemu_v8si){0, 9, 2, 11, 4, 13, 6, 15});
}

/* fused multiply-add family: one rounding per lane */
#if defined(__aarch64__)
FYEMU_INLINE __m256 fyemu_fma(__m256 a, __m256 b, __m256 c) {
    union { __m256 v; float32x4_t h[2]; } A, B, C, R;
    A.v = a; B.v = b; C.v = c;
    R.h[0] = vfmaq_f32(C.h[0], A.h[0], B.h[0]);
    R.h[1] = vfmaq_f32(C.h[1], A.h[1], B.h[1]);
    return R.v;
}
#else
FYEMU_INLINE __m256 fyemu_fma(__m256 a, __m256 b, __m256 c) {
    __m256 r;
    for (int i = 0; i < 8; ++i) r[i] = fmaf(a[i], b[i], c[i]);
    return r;
}
#endif
FYEMU_INLINE __m256 _mm256_fmadd_ps(__m256 a, __m256 b, __m256 c) { return fyemu_fma(a, b, c); }
FYEMU_INLINE __m256 _mm256_fmsub_ps(__m256 a, __m256 b, __m256 c) { return fyemu_fma(a, b, -c); }
/* -(a*b) + c: the negation of a product is exact, so this is fma(-a, b, c) */
FYEMU_INLINE __m256 _mm256_fnmadd_ps(__m256 a, __m256 b, __m256 c) { return fyemu_fma(-a, b, c); }
/* even lanes a*b - c, odd lanes a*b + c */
FYEMU_INLINE __m256 _mm256_fmaddsub_ps(__m256 a, __m256 b, __m256 c) {
    const __m256 sgn = (__m256)(fyemu_v8su){0x80000000u, 0, 0x80000000u, 0, 0x80000000u, 0, 0x80000000u, 0};
    return fyemu_fma(a, b, (__m256)((fyemu_v8su)c ^ (fyemu_v8su)sgn));
}
/* even lanes a*b + c, odd lanes a*b - c */
FYEMU_INLINE __m256 _mm256_fmsubadd_ps(__m256 a, __m256 b, __m256 c) {
    const __m256 sgn = (__m256)(fyemu_v8su){0, 0x80000000u, 0, 0x80000000u, 0, 0x80000000u, 0, 0x80000000u};
    return fyemu_fma(a, b, (__m256)((fyemu_v8su)c ^ (fyemu_v8su)sgn));
}

/* in each 128-bit half: dst[i] = a[imm8 bits 2i+1:2i] */
FYEMU_INLINE __m256 _mm256_permute_ps(__m256 a, const int imm) {
    const int s0 = imm & 3, s1 = (imm >> 2) & 3, s2 = (imm >> 4) & 3, s3 = (imm >> 6) & 3;
    return __builtin_shuffle(a, (fyemu_v8si){s0, s1, s2, s3, 4 + s0, 4 + s1, 4 + s2, 4 + s3});
}
/* in each 128-bit half: dst = {a[s0], a[s1], b[s2], b[s3]} */
FYEMU_INLINE __m256 _mm256_shuffle_ps(__m256 a, __m256 b, const int imm) {
    const int s0 = imm & 3, s1 = (imm >> 2) & 3, s2 = (imm >> 4) & 3, s3 = (imm >> 6) & 3;
    return __builtin_shuffle(a, b, (fyemu_v8si){s0, s1, 8 + s2, 8 + s3, 4 + s0, 4 + s1, 12 + s2, 12 + s3});
}
/* 128-bit halves chosen from {a.lo, a.hi, b.lo, b.hi} by imm8[1:0] / imm8[5:4], zeroed by bit 3 / 7 */
FYEMU_INLINE __m256 _mm256_permute2f128_ps(__m256 a, __m256 b, const int imm) {
    float src[16];
    memcpy(src, &a, 32);
    memcpy(src + 8, &b, 32);
    __m256 r;
    for (int h = 0; h < 2; ++h) {
        const int ctl = (imm >> (4 * h)) & 0xF;
        for (int i = 0; i < 4; ++i) r[4 * h + i] = (ctl & 8) ? 0.0f : src[4 * (ctl & 3) + i];
    }
    return r;
}
FYEMU_INLINE __m256 _mm256_moveldup_ps(__m256 a) { return __builtin_shuffle(a, (fyemu_v8si){0, 0, 2, 2, 4, 4, 6, 6}); }
FYEMU_INLINE __m256 _mm256_movehdup_ps(__m256 a) { return __builtin_shuffle(a, (fyemu_v8si){1, 1, 3, 3, 5, 5, 7, 7}); }
FYEMU_INLINE __m256 _mm256_unpacklo_ps(__m256 a, __m256 b) {
    return __builtin_shuffle(a, b, (fyemu_v8si){0, 8, 1, 9, 4, 12, 5, 13});
}
FYEMU_INLINE __m256 _mm256_unpackhi_ps(__m256 a, __m256 b) {
    return __builtin_shuffle(a, b, (fyemu_v8si){2, 10, 3, 11, 6, 14, 7, 15});
}
FYEMU_INLINE __m256 _mm256_blend_ps(__m256 a, __m256 b, const int imm) {
    __m256 r;
    for (int i = 0; i < 8; ++i) r[i] = ((imm >> i) & 1) ? b[i] : a[i];
    return r;
}
/* lane from b where the mask lane's sign bit is set */
FYEMU_INLINE __m256 _mm256_blendv_ps(__m256 a, __m256 b, __m256 mask) {
    const fyemu_v8si m = (fyemu_v8si)mask >> 31;  /* arithmetic shift: all ones or zero */
    return (__m256)(((fyemu_v8si)b & m) | ((fyemu_v8si)a & ~m));
}
FYEMU_INLINE __m256 _mm256_permutevar8x32_ps(__m256 a, __m256i idx) {
    return __builtin_shuffle(a, (fyemu_v8si)idx & 7);
}

FYEMU_INLINE __m128 _mm256_extractf128_ps(__m256 a, const int imm) {
    return (imm & 1) ? (__m128){a[4], a[5], a[6], a[7]} : (__m128){a[0], a[1], a[2], a[3]};
}
FYEMU_INLINE __m256 _mm256_insertf128_ps(__m256 a, __m128 b, const int imm) {
    __m256 r = a;
    const int o = (imm & 1) ? 4 : 0;
    for (int i = 0; i < 4; ++i) r[o + i] = b[i];
    return r;
}

/* casts (the upper half of a widened 128-bit value is unspecified by the ISA; zero here) */
FYEMU_INLINE __m256 _mm256_castpd_ps(__m256d a) { return (__m256)a; }
FYEMU_INLINE __m256d _mm256_castps_pd(__m256 a) { return (__m256d)a; }
FYEMU_INLINE __m256 _mm256_castsi256_ps(__m256i a) { return (__m256)a; }
FYEMU_INLINE __m128 _mm256_castps256_ps128(__m256 a) { return (__m128){a[0], a[1], a[2], a[3]}; }
FYEMU_INLINE __m256 _mm256_castps128_ps256(__m128 a) { return (__m256){a[0], a[1], a[2], a[3], 0, 0, 0, 0}; }

/* ---------------------------------------------------------------------------------------
 * 256-bit double
 * ------------------------------------------------------------------------------------- */
FYEMU_INLINE __m256d _mm256_loadu_pd(const double* p) { __m256d r; memcpy(&r, p, 32); return r; }
FYEMU_INLINE __m256d _mm256_load_pd(const double* p) { return _mm256_loadu_pd(p); }
FYEMU_INLINE void _mm256_storeu_pd(double* p, __m256d a) { memcpy(p, &a, 32); }
FYEMU_INLINE void _mm256_store_pd(double* p, __m256d a) { _mm256_storeu_pd(p, a); }
FYEMU_INLINE __m256d _mm256_permute2f128_pd(__m256d a, __m256d b, const int imm) {
    double src[8];
    memcpy(src, &a, 32);
    memcpy(src + 4, &b, 32);
    __m256d r;
    for (int h = 0; h < 2; ++h) {
        const int ctl = (imm >> (4 * h)) & 0xF;
        for (int i = 0; i < 2; ++i) r[2 * h + i] = (ctl & 8) ? 0.0 : src[2 * (ctl & 3) + i];
    }
    return r;
}
FYEMU_INLINE __m256d _mm256_unpacklo_pd(__m256d a, __m256d b) {
    return __builtin_shuffle(a, b, (fyemu_v4di){0, 4, 2, 6});
}
FYEMU_INLINE __m256d _mm256_unpackhi_pd(__m256d a, __m256d b) {
    return __builtin_shuffle(a, b, (fyemu_v4di){1, 5, 3, 7});
}
/* dst[i] = a[imm8 bits 2i+1:2i] */
FYEMU_INLINE __m256d _mm256_permute4x64_pd(__m256d a, const int imm) {
    return __builtin_shuffle(a, (fyemu_v4di){imm & 3, (imm >> 2) & 3, (imm >> 4) & 3, (imm >> 6) & 3});
}
/* within each 128-bit half: bit i selects the high (1) or low (0) double of that half */
FYEMU_INLINE __m256d _mm256_permute_pd(__m256d a, const int imm) {
    return __builtin_shuffle(a, (fyemu_v4di){imm & 1, (imm >> 1) & 1, 2 + ((imm >> 2) & 1), 2 + ((imm >> 3) & 1)});
}
FYEMU_INLINE __m256d _mm256_blend_pd(__m256d a, __m256d b, const int imm) {
    __m256d r;
    for (int i = 0; i < 4; ++i) r[i] = ((imm >> i) & 1) ? b[i] : a[i];
    return r;
}
/* dst[i] = *(double*)((char*)base + idx[i] * scale), idx: four 32-bit lanes */
FYEMU_INLINE __m256d _mm256_i32gather_pd(const double* base, __m128i vindex, const int scale) {
    const fyemu_v4si idx = (fyemu_v4si)vindex;
    __m256d r;
    for (int i = 0; i < 4; ++i) memcpy(&r[i], (const char*)base + (long long)idx[i] * scale, 8);
    return r;
}

/* ---------------------------------------------------------------------------------------
 * 256-bit integer (32-bit lanes)
 * ------------------------------------------------------------------------------------- */
FYEMU_INLINE __m256i _mm256_set1_epi32(int v) { return (__m256i)(fyemu_v8si){v, v, v, v, v, v, v, v}; }
FYEMU_INLINE __m256i _mm256_setr_epi32(int e0, int e1, int e2, int e3, int e4, int e5, int e6, int e7) {
    return (__m256i)(fyemu_v8si){e0, e1, e2, e3, e4, e5, e6, e7};
}
FYEMU_INLINE __m256i _mm256_setzero_si256(void) { return (__m256i){0, 0, 0, 0}; }
FYEMU_INLINE __m256i _mm256_and_si256(__m256i a, __m256i b) { return a & b; }
FYEMU_INLINE __m256i _mm256_add_epi32(__m256i a, __m256i b) {
    return (__m256i)((fyemu_v8su)a + (fyemu_v8su)b);
}
/* counts above 31 give zero */
FYEMU_INLINE __m256i _mm256_slli_epi32(__m256i a, const int imm) {
    if ((unsigned)imm > 31u) return _mm256_setzero_si256();
    return (__m256i)((fyemu_v8su)a << (unsigned)imm);
}
FYEMU_INLINE __m256i _mm256_cmpeq_epi32(__m256i a, __m256i b) {
    return (__m256i)((fyemu_v8si)a == (fyemu_v8si)b);
}
/* truncation toward zero; NaN and out-of-range lanes give 0x80000000 */
FYEMU_INLINE __m256i _mm256_cvttps_epi32(__m256 a) {
    fyemu_v8si r;
    for (int i = 0; i < 8; ++i) {
        const float v = a[i];
        r[i] = (v >= -2147483648.0f && v < 2147483648.0f) ? (int)v : (int)0x80000000u;
    }
    return (__m256i)r;
}
FYEMU_INLINE __m256 _mm256_cvtepi32_ps(__m256i a) {
    const fyemu_v8si v = (fyemu_v8si)a;
    __m256 r;
    for (int i = 0; i < 8; ++i) r[i] = (float)v[i];
    return r;
}

/* ---------------------------------------------------------------------------------------
 * 128-bit float / double / integer
 * ------------------------------------------------------------------------------------- */
FYEMU_INLINE __m128 _mm_loadu_ps(const float* p) { __m128 r; memcpy(&r, p, 16); return r; }
FYEMU_INLINE __m128 _mm_load_ps(const float* p) { return _mm_loadu_ps(p); }
FYEMU_INLINE void _mm_storeu_ps(float* p, __m128 a) { memcpy(p, &a, 16); }
FYEMU_INLINE void _mm_store_ps(float* p, __m128 a) { _mm_storeu_ps(p, a); }
FYEMU_INLINE __m128 _mm_add_ps(__m128 a, __m128 b) { return a + b; }
FYEMU_INLINE __m128 _mm_sub_ps(__m128 a, __m128 b) { return a - b; }
FYEMU_INLINE __m128 _mm_mul_ps(__m128 a, __m128 b) { return a * b; }
FYEMU_INLINE __m128 _mm_xor_ps(__m128 a, __m128 b) { return (__m128)((fyemu_v4su)a ^ (fyemu_v4su)b); }
FYEMU_INLINE __m128 _mm_setzero_ps(void) { return (__m128){0, 0, 0, 0}; }
FYEMU_INLINE __m128 _mm_set1_ps(float v) { return (__m128){v, v, v, v}; }
FYEMU_INLINE __m128 _mm_setr_ps(float e0, float e1, float e2, float e3) { return (__m128){e0, e1, e2, e3}; }
FYEMU_INLINE float _mm_cvtss_f32(__m128 a) { return a[0]; }
/* dst = {a[s0], a[s1], b[s2], b[s3]} */
FYEMU_INLINE __m128 _mm_shuffle_ps(__m128 a, __m128 b, const int imm) {
    return __builtin_shuffle(a, b, (fyemu_v4si){imm & 3, (imm >> 2) & 3, 4 + ((imm >> 4) & 3), 4 + ((imm >> 6) & 3)});
}
FYEMU_INLINE __m128 _mm_movelh_ps(__m128 a, __m128 b) { return __builtin_shuffle(a, b, (fyemu_v4si){0, 1, 4, 5}); }
FYEMU_INLINE __m128 _mm_movehl_ps(__m128 a, __m128 b) { return __builtin_shuffle(a, b, (fyemu_v4si){6, 7, 2, 3}); }
FYEMU_INLINE __m128 _mm_unpacklo_ps(__m128 a, __m128 b) { return __builtin_shuffle(a, b, (fyemu_v4si){0, 4, 1, 5}); }
FYEMU_INLINE __m128 _mm_unpackhi_ps(__m128 a, __m128 b) { return __builtin_shuffle(a, b, (fyemu_v4si){2, 6, 3, 7}); }
/* the two low floats of a (8 bytes) / the two high floats */
FYEMU_INLINE void _mm_storel_pi(__m64* p, __m128 a) { memcpy(p, &a, 8); }
FYEMU_INLINE void _mm_storeh_pi(__m64* p, __m128 a) { memcpy(p, (const char*)&a + 8, 8); }
/* low two floats from memory, high two from a */
FYEMU_INLINE __m128 _mm_loadl_pi(__m128 a, const __m64* p) {
    __m128 r = a;
    memcpy(&r, p, 8);
    return r;
}
FYEMU_INLINE __m128 _mm_castpd_ps(__m128d a) { return (__m128)a; }
FYEMU_INLINE __m128d _mm_castps_pd(__m128 a) { return (__m128d)a; }
FYEMU_INLINE __m128d _mm_load_sd(const double* p) { __m128d r = {0.0, 0.0}; memcpy(&r, p, 8); return r; }
FYEMU_INLINE void _mm_store_sd(double* p, __m128d a) { memcpy(p, &a, 8); }
FYEMU_INLINE void _mm_storeh_pd(double* p, __m128d a) { memcpy(p, (const char*)&a + 8, 8); }
/* arguments from the highest lane down: dst[0] = e0 */
FYEMU_INLINE __m128i _mm_set_epi32(int e3, int e2, int e1, int e0) { return (__m128i)(fyemu_v4si){e0, e1, e2, e3}; }
