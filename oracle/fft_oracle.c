/*
 * fft_oracle.c -- CPU oracle for the 1D complex FFT path of fyFFT.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only as the checker
 * or the timed CPU baseline.  The GPU library never calls it.
 *
 * It restates, in FP64 arithmetic with long-double twiddles and exact integer index
 * reduction, the algorithm of the reference (kjear/fyFFT, a header-only C++ library):
 *   - strategy selection               foye_FFT.hpp:101-126, :162-184
 *   - smooth-length registry           src/foye_FFT_radix_wrap.hpp:41-44, :75-79, :87-98
 *   - mixed-radix processability       src/foye_FFT_mix_radix.hpp:618-643
 *   - radix-r Cooley-Tukey stages      src/foye_FFT_radix{2,3,4,5,7}.hpp, src/foye_FFT_mix_radix.hpp
 *     (restated as one self-sorting Stockham sweep over the prime factors of N)
 *   - Rader for primes                 src/foye_FFT_rader.hpp:142-401
 *   - Bluestein chirp-z                src/foye_FFT_bluestein.hpp:79-355
 *   - number theory                    src/foye_FFT_utility.hpp:392-485
 *   - inverse = exp(+2 pi i kn/N) / N   e.g. src/foye_FFT_radix2.hpp:669-672, src/foye_FFT_dft.hpp:133-136
 * plus a naive long-double DFT (O(N^2)) used to pin the FFT itself at small N, and a
 * sampled long-double DFT for spot checks at large N.
 *
 * Where the reference falls back to its O(N^2) DFT (lengths > 39062 that are neither 7-smooth
 * nor Rader-processable, src/foye_FFT_dft.hpp), the oracle keeps using Rader / Bluestein with
 * the smallest 7-smooth convolution length, which computes the same transform.
 *
 * All complex buffers are interleaved (re, im) doubles.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } cd;

/* ------------------------------------------------------------------ */
/* Registry and strategy selection (reference semantics)               */
/* ------------------------------------------------------------------ */

/* src/foye_FFT_radix_wrap.hpp:93-98 -- the 38 directly supported lengths */
static const size_t k_smooth[38] = {
    2, 3, 4, 5, 7, 8, 9, 16, 25, 27, 32, 49, 64, 81,
    125, 128, 243, 256, 343, 512, 625, 729, 1024,
    2048, 2187, 2401, 3125, 4096, 6561, 8192, 15625,
    16384, 16807, 19683, 32768, 59049, 65536, 78125};

/* src/foye_FFT_radix_wrap.hpp:41-44 */
int orc_is_directly_supported(size_t n) {
    for (int i = 0; i < 38; ++i) if (k_smooth[i] == n) return 1;
    return 0;
}

/* src/foye_FFT_radix_wrap.hpp:75-79: smallest registered length >= n, or 0 */
size_t orc_next_smooth(size_t n) {
    for (int i = 0; i < 38; ++i) if (k_smooth[i] >= n) return k_smooth[i];
    return 0;
}

/* src/foye_FFT_mix_radix.hpp:618-643: greedy division by the largest registered length */
int orc_mixed_is_processable(size_t n) {
    if (n == 0) return 0;
    while (n > 1) {
        int found = 0;
        for (int i = 37; i >= 0; --i) {
            size_t f = k_smooth[i];
            if (f <= n && n % f == 0) { n /= f; found = 1; break; }
        }
        if (!found) return 0;
    }
    return 1;
}

/* src/foye_FFT_utility.hpp:392-418 */
int orc_is_prime(size_t n) {
    if (n < 2) return 0;
    if (n < 4) return 1;
    if (n % 2 == 0 || n % 3 == 0) return 0;
    for (size_t i = 5; i * i <= n; i += 6)
        if (n % i == 0 || n % (i + 2) == 0) return 0;
    return 1;
}

/* src/foye_FFT_rader.hpp:403-423: prime, not registered, next_smooth(2n-3) exists */
int orc_rader_is_processable(size_t n) {
    if (n < 2 || n > k_smooth[37]) return 0;
    if (orc_is_directly_supported(n) || !orc_is_prime(n)) return 0;
    return orc_next_smooth(2 * n - 3) != 0;
}

/* src/foye_FFT_bluestein.hpp:188-215 */
int orc_bluestein_is_processable(size_t n) { return n <= 39062; }

/* foye_FFT.hpp:153-184.  0 kernel_direct, 1 mix_radix, 2 rader, 3 bluestein, 4 DFT */
int orc_strategy(size_t n) {
    if (orc_is_directly_supported(n)) return 0;
    if (orc_mixed_is_processable(n)) return 1;
    if (orc_rader_is_processable(n)) return 2;
    if (orc_bluestein_is_processable(n)) return 3;
    return 4;
}

/* src/foye_FFT_utility.hpp:420-435 */
static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) {
    return (uint64_t)((unsigned __int128)a * b % m);
}
size_t orc_power_mod(size_t base, size_t e, size_t mod) {
    uint64_t r = 1 % mod, b = base % mod;
    while (e) { if (e & 1) r = mulmod(r, b, mod); b = mulmod(b, b, mod); e >>= 1; }
    return (size_t)r;
}

/* src/foye_FFT_utility.hpp:437-485: smallest primitive root of prime N */
size_t orc_find_primitive_root(size_t n) {
    if (n == 2) return 1;
    size_t phi = n - 1, m = phi, f[64]; int nf = 0;
    for (size_t p = 2; p * p <= m; ++p)
        if (m % p == 0) { f[nf++] = p; while (m % p == 0) m /= p; }
    if (m > 1) f[nf++] = m;
    for (size_t g = 2; g < n; ++g) {
        int ok = 1;
        for (int i = 0; i < nf && ok; ++i)
            if (orc_power_mod(g, phi / f[i], n) == 1) ok = 0;
        if (ok) return g;
    }
    return 0;
}

/* smallest 2^a 3^b 5^c 7^d >= n (extension used where the registry has no length) */
size_t orc_next_7smooth(size_t n) {
    if (n <= 1) return 1;
    for (size_t m = n;; ++m) {
        size_t t = m;
        while (t % 2 == 0) t /= 2;
        while (t % 3 == 0) t /= 3;
        while (t % 5 == 0) t /= 5;
        while (t % 7 == 0) t /= 7;
        if (t == 1) return m;
    }
}

/* ------------------------------------------------------------------ */
/* Twiddles: exp(-2 pi i t / n), long double, exact integer reduction  */
/* ------------------------------------------------------------------ */

static const long double k_two_pi_l = 6.283185307179586476925286766559005768L;

static cd twiddle_ld(uint64_t t, uint64_t n) {
    t %= n;
    long double a = k_two_pi_l * (long double)t / (long double)n;
    cd w = {(double)cosl(a), (double)(-sinl(a))};
    return w;
}

static cd* twiddle_table(size_t n) {
    cd* w = (cd*)malloc(sizeof(cd) * (n ? n : 1));
    if (!w) return NULL;
    for (size_t t = 0; t < n; ++t) w[t] = twiddle_ld(t, n);
    return w;
}

/* ------------------------------------------------------------------ */
/* Naive DFTs (long double accumulation)                               */
/* ------------------------------------------------------------------ */

/* Direct DFT, sign -1 forward; inverse uses +1 and scales by 1/n. */
int orc_dft(size_t n, int inverse, const double* in, double* out) {
    if (n == 0) return -1;
    cd* w = twiddle_table(n);
    if (!w) return -2;
    const cd* x = (const cd*)in;
    cd* y = (cd*)malloc(sizeof(cd) * n);
    for (size_t k = 0; k < n; ++k) {
        long double sr = 0, si = 0;
        size_t t = 0;
        for (size_t j = 0; j < n; ++j) {
            long double wr = w[t].re, wi = inverse ? -w[t].im : w[t].im;
            sr += (long double)x[j].re * wr - (long double)x[j].im * wi;
            si += (long double)x[j].re * wi + (long double)x[j].im * wr;
            t += k; if (t >= n) t -= n;
        }
        if (inverse) { sr /= (long double)n; si /= (long double)n; }
        y[k].re = (double)sr; y[k].im = (double)si;
    }
    memcpy(out, y, sizeof(cd) * n);
    free(y); free(w);
    return 0;
}

/* Direct DFT at selected output indices only (O(n * count)), long double accumulation. */
int orc_dft_sampled(size_t n, int inverse, const double* in, const int64_t* idx, size_t count, double* out) {
    const cd* x = (const cd*)in;
    for (size_t c = 0; c < count; ++c) {
        uint64_t k = (uint64_t)idx[c] % n;
        long double sr = 0, si = 0;
        uint64_t t = 0;
        for (size_t j = 0; j < n; ++j) {
            long double a = k_two_pi_l * (long double)t / (long double)n;
            long double wr = cosl(a), wi = inverse ? sinl(a) : -sinl(a);
            sr += (long double)x[j].re * wr - (long double)x[j].im * wi;
            si += (long double)x[j].re * wi + (long double)x[j].im * wr;
            t += k; if (t >= n) t -= n;
        }
        if (inverse) { sr /= (long double)n; si /= (long double)n; }
        out[2 * c] = (double)sr; out[2 * c + 1] = (double)si;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* FP64 Stockham sweep over the prime factors of n (radix-r stages)    */
/* ------------------------------------------------------------------ */

#define ORC_MAX_DIRECT_PRIME 67  /* larger prime factors go through Rader / Bluestein */

static int factorize(size_t n, int* f) {
    int nf = 0;
    while (n % 4 == 0) { f[nf++] = 4; n /= 4; }
    while (n % 2 == 0) { f[nf++] = 2; n /= 2; }
    for (size_t p = 3; p * p <= n; p += 2)
        while (n % p == 0) { f[nf++] = (int)p; n /= p; }
    if (n > 1) f[nf++] = (int)n;
    return nf;
}

static int max_factor(size_t n) {
    int f[64], nf = factorize(n, f), m = 1;
    for (int i = 0; i < nf; ++i) if (f[i] > m) m = f[i];
    return m;
}

static inline cd cmul(cd a, cd b) { cd r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cd cconj(cd a) { cd r = {a.re, -a.im}; return r; }

/* One transform with a precomputed table w[t] = exp(-2 pi i t/n).  sign: 0 forward (-), 1 (+).
 * Unscaled.  x is consumed (used as ping-pong storage); the result is written to y. */
static void stockham(size_t n, const cd* w, int conj_tw, cd* x, cd* y, cd* tmp) {
    int f[64], nf = factorize(n, f);
    cd* src = x; cd* dst = tmp;
    size_t Ns = 1;
    cd a[ORC_MAX_DIRECT_PRIME], b[ORC_MAX_DIRECT_PRIME];
    for (int s = 0; s < nf; ++s) {
        const size_t r = (size_t)f[s], m = n / r, nblk = m / Ns, tw_unit = n / (Ns * r), rs = n / r;
        for (size_t blk = 0; blk < nblk; ++blk) {
            for (size_t k = 0; k < Ns; ++k) {
                const size_t j = blk * Ns + k;
                for (size_t q = 0; q < r; ++q) {
                    cd v = src[j + q * m];
                    size_t t = q * k * tw_unit;
                    if (t) { cd tw = conj_tw ? cconj(w[t]) : w[t]; v = cmul(v, tw); }
                    a[q] = v;
                }
                if (r == 2) {
                    b[0].re = a[0].re + a[1].re; b[0].im = a[0].im + a[1].im;
                    b[1].re = a[0].re - a[1].re; b[1].im = a[0].im - a[1].im;
                } else if (r == 4) {
                    cd s0 = {a[0].re + a[2].re, a[0].im + a[2].im}, d0 = {a[0].re - a[2].re, a[0].im - a[2].im};
                    cd s1 = {a[1].re + a[3].re, a[1].im + a[3].im}, d1 = {a[1].re - a[3].re, a[1].im - a[3].im};
                    /* forward: -i * d1 ; inverse: +i * d1 */
                    cd rd1 = conj_tw ? (cd){-d1.im, d1.re} : (cd){d1.im, -d1.re};
                    b[0].re = s0.re + s1.re; b[0].im = s0.im + s1.im;
                    b[2].re = s0.re - s1.re; b[2].im = s0.im - s1.im;
                    b[1].re = d0.re + rd1.re; b[1].im = d0.im + rd1.im;
                    b[3].re = d0.re - rd1.re; b[3].im = d0.im - rd1.im;
                } else {
                    for (size_t p = 0; p < r; ++p) {
                        long double sr = 0, si = 0;
                        for (size_t q = 0; q < r; ++q) {
                            cd tw = w[((p * q) % r) * rs];
                            if (conj_tw) tw = cconj(tw);
                            sr += (long double)a[q].re * tw.re - (long double)a[q].im * tw.im;
                            si += (long double)a[q].re * tw.im + (long double)a[q].im * tw.re;
                        }
                        b[p].re = (double)sr; b[p].im = (double)si;
                    }
                }
                const size_t base = blk * Ns * r + k;
                for (size_t p = 0; p < r; ++p) dst[base + p * Ns] = b[p];
            }
        }
        Ns *= r;
        cd* t = src; src = dst; dst = t;
    }
    if (src != y) memcpy(y, src, sizeof(cd) * n);
}

/* Smooth transform of length n (all prime factors <= ORC_MAX_DIRECT_PRIME), unscaled. */
static int fft_smooth(size_t n, int conj_tw, const cd* in, cd* out) {
    cd* w = twiddle_table(n);
    cd* x = (cd*)malloc(sizeof(cd) * n);
    cd* t = (cd*)malloc(sizeof(cd) * n);
    if (!w || !x || !t) { free(w); free(x); free(t); return -2; }
    memcpy(x, in, sizeof(cd) * n);
    stockham(n, w, conj_tw, x, out, t);
    free(w); free(x); free(t);
    return 0;
}

static int fft_any(size_t n, int conj_tw, const cd* in, cd* out);

/* ------------------------------------------------------------------ */
/* Rader (src/foye_FFT_rader.hpp:142-401), FP64                        */
/* ------------------------------------------------------------------ */
/* L = n-1; a[i] = x[g^-i]; b[i] = exp(-+2 pi i g^i / n); linear convolution of length
 * M = next_smooth(2L-1) (registry; 7-smooth beyond it) through FFT_M; fold c[q] = lin[q] + lin[q+L];
 * X[0] = sum x; X[g^q] = x0 + c[q].  Unscaled. */
static int fft_rader(size_t n, int conj_tw, const cd* x, cd* out) {
    const size_t L = n - 1;
    size_t M = orc_next_smooth(2 * L - 1);
    if (M == 0) M = orc_next_7smooth(2 * L - 1);
    const size_t g = orc_find_primitive_root(n);
    const size_t ginv = orc_power_mod(g, n - 2, n);
    cd* a = (cd*)calloc(M, sizeof(cd));
    cd* b = (cd*)calloc(M, sizeof(cd));
    cd* A = (cd*)malloc(sizeof(cd) * M);
    cd* B = (cd*)malloc(sizeof(cd) * M);
    size_t* gp = (size_t*)malloc(sizeof(size_t) * L);
    if (!a || !b || !A || !B || !gp) { free(a); free(b); free(A); free(B); free(gp); return -2; }
    long double sr = x[0].re, si = x[0].im;
    size_t cur = 1, cur_inv = 1;
    for (size_t i = 0; i < L; ++i) {
        gp[i] = cur;
        a[i] = x[cur_inv];
        sr += x[cur_inv].re; si += x[cur_inv].im;
        cd w = twiddle_ld(cur, n);
        b[i] = conj_tw ? cconj(w) : w;
        cur = (size_t)mulmod(cur, g, n);
        cur_inv = (size_t)mulmod(cur_inv, ginv, n);
    }
    int rc = fft_any(M, 0, a, A);
    if (!rc) rc = fft_any(M, 0, b, B);
    if (!rc) {
        for (size_t i = 0; i < M; ++i) A[i] = cmul(A[i], B[i]);
        rc = fft_any(M, 1, A, a);          /* unscaled inverse; divide by M below */
    }
    if (!rc) {
        const double inv_m = 1.0 / (double)M;
        out[0].re = (double)sr; out[0].im = (double)si;
        for (size_t q = 0; q < L; ++q) {
            cd c = a[q];
            if (q + L < M) { c.re += a[q + L].re; c.im += a[q + L].im; }
            out[gp[q]].re = x[0].re + c.re * inv_m;
            out[gp[q]].im = x[0].im + c.im * inv_m;
        }
    }
    free(a); free(b); free(A); free(B); free(gp);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Bluestein (src/foye_FFT_bluestein.hpp:79-355), FP64                 */
/* ------------------------------------------------------------------ */
/* chirp w_n = exp(+i pi (n^2 mod 2N) / N) with exact integer reduction (:7-18);
 * a = x * conj(w) zero-padded to M; kernel h[n] = w_n at n and M-n; X = conj(w) * IFFT(FFT(a) FFT(h)).
 * M = smallest registered length >= 2N-1 (:95, :173-183), else the smallest 7-smooth one.
 * conj_tw selects the +i sign (unscaled inverse). */
static int fft_bluestein(size_t n, int conj_tw, const cd* x, cd* out) {
    if (n < 2) { if (n == 1) out[0] = x[0]; return n ? 0 : -1; }
    size_t M = orc_next_smooth(2 * n - 1);
    if (M == 0) M = orc_next_7smooth(2 * n - 1);
    cd* w = (cd*)calloc(n, sizeof(cd));
    cd* a = (cd*)calloc(M, sizeof(cd));
    cd* h = (cd*)calloc(M, sizeof(cd));
    cd* A = (cd*)malloc(sizeof(cd) * M);
    cd* H = (cd*)malloc(sizeof(cd) * M);
    if (!w || !a || !h || !A || !H) { free(w); free(a); free(h); free(A); free(H); return -2; }
    const uint64_t two_n = 2 * (uint64_t)n;
    for (size_t i = 0; i < n; ++i) {
        uint64_t sq = mulmod(i, i, two_n);
        long double ang = 3.141592653589793238462643383279502884L * (long double)sq / (long double)n;
        cd c = {(double)cosl(ang), (double)sinl(ang)};   /* exp(+i pi sq / n) */
        if (conj_tw) c = cconj(c);
        w[i] = c;
    }
    for (size_t i = 0; i < n; ++i) a[i] = cmul(x[i], cconj(w[i]));
    h[0] = w[0];
    for (size_t i = 1; i < n; ++i) { h[i] = w[i]; h[M - i] = w[i]; }
    int rc = fft_any(M, 0, a, A);
    if (!rc) rc = fft_any(M, 0, h, H);
    if (!rc) {
        for (size_t i = 0; i < M; ++i) A[i] = cmul(A[i], H[i]);
        rc = fft_any(M, 1, A, a);
    }
    if (!rc) {
        const double inv_m = 1.0 / (double)M;
        for (size_t i = 0; i < n; ++i) {
            cd v = {a[i].re * inv_m, a[i].im * inv_m};
            out[i] = cmul(v, cconj(w[i]));
        }
    }
    free(w); free(a); free(h); free(A); free(H);
    return rc;
}

/* Unscaled transform of any length; conj_tw = 1 for the +i sign. */
static int fft_any(size_t n, int conj_tw, const cd* in, cd* out) {
    if (n == 1) { out[0] = in[0]; return 0; }
    if (max_factor(n) <= ORC_MAX_DIRECT_PRIME) return fft_smooth(n, conj_tw, in, out);
    if (orc_is_prime(n)) return fft_rader(n, conj_tw, in, out);
    return fft_bluestein(n, conj_tw, in, out);
}

/* Strategy chain of foye_FFT.hpp:101-126 evaluated in FP64: smooth / mixed -> radix stages,
 * Rader-processable prime -> Rader, otherwise Bluestein (the reference's DFT fallback beyond
 * 39062 is replaced by Bluestein, which computes the same transform). */
int orc_fft(size_t n, int inverse, const double* in, double* out) {
    if (n == 0) return -1;
    const cd* x = (const cd*)in;
    cd* y = (cd*)malloc(sizeof(cd) * n);
    if (!y) return -2;
    int rc;
    int s = orc_strategy(n);
    if (s == 0 || s == 1) rc = fft_smooth(n, inverse, x, y);
    else if (orc_is_prime(n)) rc = fft_rader(n, inverse, x, y);
    else if (max_factor(n) <= ORC_MAX_DIRECT_PRIME) rc = fft_smooth(n, inverse, x, y);
    else rc = fft_bluestein(n, inverse, x, y);
    if (!rc) {
        if (inverse) {
            const double s1 = 1.0 / (double)n;
            for (size_t i = 0; i < n; ++i) { y[i].re *= s1; y[i].im *= s1; }
        }
        memcpy(out, y, sizeof(cd) * n);
    }
    free(y);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Batched / threaded drivers (used for the timed CPU baseline)        */
/* ------------------------------------------------------------------ */

typedef struct {
    size_t n, lo, hi; int inverse; int f32;
    const void* in; void* out; int rc;
} job_t;

static void* run_job(void* p) {
    job_t* j = (job_t*)p;
    j->rc = 0;
    double* xi = NULL; double* yo = NULL;
    if (j->f32) {
        xi = (double*)malloc(sizeof(double) * 2 * j->n);
        yo = (double*)malloc(sizeof(double) * 2 * j->n);
        if (!xi || !yo) { j->rc = -2; free(xi); free(yo); return NULL; }
    }
    for (size_t b = j->lo; b < j->hi && !j->rc; ++b) {
        if (j->f32) {
            const float* src = (const float*)j->in + 2 * j->n * b;
            float* dst = (float*)j->out + 2 * j->n * b;
            for (size_t i = 0; i < 2 * j->n; ++i) xi[i] = src[i];
            j->rc = orc_fft(j->n, j->inverse, xi, yo);
            for (size_t i = 0; i < 2 * j->n; ++i) dst[i] = (float)yo[i];
        } else {
            j->rc = orc_fft(j->n, j->inverse, (const double*)j->in + 2 * j->n * b,
                            (double*)j->out + 2 * j->n * b);
        }
    }
    free(xi); free(yo);
    return NULL;
}

/* `batch` contiguous transforms split over `threads` POSIX threads.  f32 != 0: float buffers
 * (converted to double per transform). */
int orc_fft_batch(size_t n, size_t batch, int inverse, const void* in, void* out, int threads, int f32) {
    if (threads < 1) threads = 1;
    if ((size_t)threads > batch) threads = batch ? (int)batch : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    job_t* jobs = (job_t*)malloc(sizeof(job_t) * threads);
    if (!th || !jobs) { free(th); free(jobs); return -2; }
    for (int t = 0; t < threads; ++t) {
        job_t j = {n, batch * t / threads, batch * (t + 1) / threads, inverse, f32, in, out, 0};
        jobs[t] = j;
        pthread_create(&th[t], NULL, run_job, &jobs[t]);
    }
    int rc = 0;
    for (int t = 0; t < threads; ++t) { pthread_join(th[t], NULL); if (jobs[t].rc) rc = jobs[t].rc; }
    free(th); free(jobs);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Seeded synthetic inputs                                             */
/* ------------------------------------------------------------------ */
/* The inputs of every configuration: element i of stream `seed` is a pure function of
 * (seed, i), so that the GPU library's generator, this one and any number of threads produce
 * the same values.  Bits: splitmix64 finalizer of seed + golden-ratio increments
 * (2i for the real part, 2i+1 for the imaginary part).  uniform: 53-bit u -> 2u - 1;
 * normal: Box-Muller, r = sqrt(-2 ln(1 - u1)), angle 2 pi u2.
 * Restated here so that the CPU baseline and the fixtures never load the product library;
 * tests/test_oracle_generator.py checks it equal to fyg_fill_random. */
static uint64_t orc_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t orc_rand_bits(uint64_t seed, uint64_t i) {
    const uint64_t phi = 0x9E3779B97F4A7C15ull;
    return orc_mix64(orc_mix64(seed + phi) + (i + 1) * phi);
}

typedef struct {
    uint64_t seed;
    int dist, f32;
    size_t lo, hi;
    void* out;
} fill_job;

static void* fill_run(void* p) {
    const fill_job* j = (const fill_job*)p;
    for (size_t i = j->lo; i < j->hi; ++i) {
        const double u1 = (double)(orc_rand_bits(j->seed, 2 * i) >> 11) * 0x1.0p-53;
        const double u2 = (double)(orc_rand_bits(j->seed, 2 * i + 1) >> 11) * 0x1.0p-53;
        double re, im;
        if (j->dist == 0) {
            re = 2.0 * u1 - 1.0;
            im = 2.0 * u2 - 1.0;
        } else {
            const double r = sqrt(-2.0 * log(1.0 - u1));
            re = r * cos(6.283185307179586 * u2);
            im = r * sin(6.283185307179586 * u2);
        }
        if (j->f32) {
            ((float*)j->out)[2 * i] = (float)re;
            ((float*)j->out)[2 * i + 1] = (float)im;
        } else {
            ((double*)j->out)[2 * i] = re;
            ((double*)j->out)[2 * i + 1] = im;
        }
    }
    return NULL;
}

/* dist: 0 uniform[-1, 1), 1 normal; f32: 1 complex<float>, 0 complex<double> */
int orc_fill_random(uint64_t seed, int dist, int f32, size_t n, void* out, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    if (n < ((size_t)1 << 16)) threads = 1;
    pthread_t th[64];
    fill_job jobs[64];
    for (int t = 0; t < threads; ++t) {
        jobs[t].seed = seed;
        jobs[t].dist = dist;
        jobs[t].f32 = f32;
        jobs[t].lo = n * (size_t)t / (size_t)threads;
        jobs[t].hi = n * (size_t)(t + 1) / (size_t)threads;
        jobs[t].out = out;
    }
    int started[64] = {0};
    for (int t = 1; t < threads; ++t) started[t] = pthread_create(&th[t], NULL, fill_run, &jobs[t]) == 0;
    fill_run(&jobs[0]);
    for (int t = 1; t < threads; ++t) {
        if (started[t]) pthread_join(th[t], NULL);
        else fill_run(&jobs[t]);   /* no thread: this range on the calling thread */
    }
    return 0;
}
