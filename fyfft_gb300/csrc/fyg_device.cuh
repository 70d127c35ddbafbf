// fyg_device.cuh -- device-side building blocks of the GB300 FFT engine.
//
// Complex helpers, fast integer division, the radix-r butterfly codelets (r = 2,3,4,5,7,8,9,16
// and the odd primes 11, 13) and the codelet constant tables.
//
// Codelets compute the forward DFT y[k] = sum_n a[n] exp(-2 pi i nk/r) in place and in natural
// order.  Inverse transforms never need a second codelet set: the engine computes
// IDFT(x) = conj(DFT(conj(x))) by conjugating at the first load and the last store of a pipeline.
//
// Reference counterparts: the butterflies of src/foye_FFT_radix{2,3,4,5,7}.hpp, the fixed-size
// micro-kernels of src/foye_FFT_microKernel.hpp:48-1388 and the batch kernel's radix-r DFTs
// (src/foye_FFT_batch_kernel.hpp:6-766).  The constants are cos/sin(2 pi m/r) computed on the
// host in long double (fyg_plan.cu) and uploaded once per device.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fyg {

template <typename T> struct vec2;
template <> struct vec2<float> { using type = float2; };
template <> struct vec2<double> { using type = double2; };
template <typename T> using cplx = typename vec2<T>::type;

template <typename T2> __device__ __forceinline__ T2 mk(decltype(T2::x) a, decltype(T2::x) b) { T2 r; r.x = a; r.y = b; return r; }
template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { return mk<T2>(a.x + b.x, a.y + b.y); }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { return mk<T2>(a.x - b.x, a.y - b.y); }
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
    return mk<T2>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
template <typename T2> __device__ __forceinline__ T2 cconj(T2 a) { return mk<T2>(a.x, -a.y); }
template <typename T2, typename T> __device__ __forceinline__ T2 cscale(T2 a, T s) { return mk<T2>(a.x * s, a.y * s); }
// -i * a
template <typename T2> __device__ __forceinline__ T2 mul_mi(T2 a) { return mk<T2>(a.y, -a.x); }

// FP32 complex add / subtract as one packed f32x2 instruction (sm_100+): both lanes are IEEE
// round-to-nearest operations.  Unlike the scalar form they are never contracted into an FMA
// with a neighbouring multiply (measured: 3-5% faster passes, rel-L2 1.69e-7 -> 1.72e-7 at 2^20).
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) {
    float2 d;
    asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n add.rn.f32x2 rd, ra, rb;\n"
        " mov.b64 {%0, %1}, rd;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
    float2 d;
    asm("{\n .reg .b64 ra, rb, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n sub.rn.f32x2 rd, ra, rb;\n"
        " mov.b64 {%0, %1}, rd;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

// Conversions between storage (TIO) and compute (T) complex types.
__device__ __forceinline__ float2 to_c(float2 v, float) { return v; }
__device__ __forceinline__ double2 to_c(float2 v, double) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_c(double2 v, double) { return v; }
__device__ __forceinline__ float2 to_c(double2 v, float) { return make_float2((float)v.x, (float)v.y); }

// q = n / d for 0 <= n < 2^31 (Granlund-Montgomery round-up multiplier; host sets m and s).
struct FastDiv {
    uint32_t d, m, s;
    __device__ __forceinline__ uint32_t div(uint32_t n) const { return (__umulhi(n, m) + n) >> s; }
};

// Codelet constants: C[m] = cos(2 pi m/r), S[m] = sin(2 pi m/r) for every codelet size r that
// needs them (odd primes, and the composite sizes for their internal twiddles).
#define FYG_CODELET_TABLES(X) \
    X(3) X(5) X(7) X(9) X(11) X(13) X(16) X(12) X(20) X(24) X(25) X(27) X(32)
template <typename T> struct CodeletConsts {
#define FYG_DECL(r) T c##r[r], s##r[r];
    FYG_CODELET_TABLES(FYG_DECL)
#undef FYG_DECL
};

// One copy per translation unit that launches kernels (no relocatable device code); each such
// unit exports an upload function that ensure_device_constants() calls once per device.
static __constant__ CodeletConsts<float> g_kf;
static __constant__ CodeletConsts<double> g_kd;

template <typename T> __device__ __forceinline__ const CodeletConsts<T>& kc();
template <> __device__ __forceinline__ const CodeletConsts<float>& kc<float>() { return g_kf; }
template <> __device__ __forceinline__ const CodeletConsts<double>& kc<double>() { return g_kd; }

// ------------------------------------------------------------------------------------------
// Codelets (forward sign).
// ------------------------------------------------------------------------------------------

template <typename T2> __device__ __forceinline__ void dft2(T2* a) {
    T2 t = a[0];
    a[0] = cadd(t, a[1]);
    a[1] = csub(t, a[1]);
}

template <typename T2> __device__ __forceinline__ void dft4_io(T2& a0, T2& a1, T2& a2, T2& a3) {
    T2 s0 = cadd(a0, a2), d0 = csub(a0, a2);
    T2 s1 = cadd(a1, a3), d1 = mul_mi(csub(a1, a3));
    a0 = cadd(s0, s1);
    a2 = csub(s0, s1);
    a1 = cadd(d0, d1);
    a3 = csub(d0, d1);
}
template <typename T2> __device__ __forceinline__ void dft4(T2* a) { dft4_io(a[0], a[1], a[2], a[3]); }

// Odd prime p: y_k = a0 + sum_n C[nk] t_n - i sum_n S[nk] d_n, y_{p-k} = ... + i ...
// with t_n = a_n + a_{p-n}, d_n = a_n - a_{p-n}.
template <int P, typename T, typename T2>
__device__ __forceinline__ void dft_odd_prime(T2* a, const T* C, const T* S) {
    constexpr int H = (P - 1) / 2;
    T2 t[H + 1], d[H + 1];
    T2 y0 = a[0];
#pragma unroll
    for (int n = 1; n <= H; ++n) {
        t[n] = cadd(a[n], a[P - n]);
        d[n] = csub(a[n], a[P - n]);
        y0 = cadd(y0, t[n]);
    }
    const T2 a0 = a[0];
    a[0] = y0;
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        T2 re = a0;
        T2 im = mk<T2>(T(0), T(0));
#pragma unroll
        for (int n = 1; n <= H; ++n) {
            const int m = (n * k) % P;
            re.x = fma(C[m], t[n].x, re.x);
            re.y = fma(C[m], t[n].y, re.y);
            im.x = fma(S[m], d[n].x, im.x);
            im.y = fma(S[m], d[n].y, im.y);
        }
        // y_k = re - i*im, y_{P-k} = re + i*im (t and d stay intact for the next k)
        a[k] = mk<T2>(re.x + im.y, re.y - im.x);
        a[P - k] = mk<T2>(re.x - im.y, re.y + im.x);
    }
}

// exp(-2 pi i e/16) for a compile-time e (0 <= e < 16)
template <typename T, typename T2> __device__ __forceinline__ T2 w16(int e) {
    const CodeletConsts<T>& K = kc<T>();
    return mk<T2>(K.c16[e & 15], -K.s16[e & 15]);
}

template <typename T, typename T2> __device__ __forceinline__ void dft8(T2* a) {
    // radix-2 split: even/odd DFT4, twiddle w8^k = w16^(2k), combine
    T2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
    T2 o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
    dft4_io(e0, e1, e2, e3);
    dft4_io(o0, o1, o2, o3);
    const T r = kc<T>().c16[2];  // cos(pi/4)
    o1 = mk<T2>(r * (o1.x + o1.y), r * (o1.y - o1.x));      // * (r, -r)
    o2 = mul_mi(o2);                                         // * -i
    o3 = mk<T2>(r * (o3.y - o3.x), -r * (o3.x + o3.y));     // * (-r, -r)
    a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
    a[1] = cadd(e1, o1); a[5] = csub(e1, o1);
    a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
    a[3] = cadd(e3, o3); a[7] = csub(e3, o3);
}

template <typename T, typename T2> __device__ __forceinline__ void dft16(T2* a) {
    // n = 4 n1 + n2, k = k1 + 4 k2: DFT4 over n1, twiddle w16^(n2 k1), DFT4 over n2
    T2 f[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        T2 x0 = a[n2], x1 = a[4 + n2], x2 = a[8 + n2], x3 = a[12 + n2];
        dft4_io(x0, x1, x2, x3);
        f[n2][0] = x0; f[n2][1] = x1; f[n2][2] = x2; f[n2][3] = x3;
    }
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
        for (int k1 = 1; k1 < 4; ++k1) f[n2][k1] = cmul(f[n2][k1], w16<T, T2>(n2 * k1));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        T2 x0 = f[0][k1], x1 = f[1][k1], x2 = f[2][k1], x3 = f[3][k1];
        dft4_io(x0, x1, x2, x3);
        a[k1] = x0; a[k1 + 4] = x1; a[k1 + 8] = x2; a[k1 + 12] = x3;
    }
}

template <typename T, typename T2> __device__ __forceinline__ void dft9(T2* a) {
    // n = 3 n1 + n2, k = k1 + 3 k2: DFT3 over n1, twiddle w9^(n2 k1), DFT3 over n2
    const CodeletConsts<T>& K = kc<T>();
    T2 f[3][3];
#pragma unroll
    for (int n2 = 0; n2 < 3; ++n2) {
        T2 x[3] = {a[n2], a[3 + n2], a[6 + n2]};
        dft_odd_prime<3, T>(x, K.c3, K.s3);
        f[n2][0] = x[0]; f[n2][1] = x[1]; f[n2][2] = x[2];
    }
#pragma unroll
    for (int n2 = 1; n2 < 3; ++n2)
#pragma unroll
        for (int k1 = 1; k1 < 3; ++k1) {
            const int e = n2 * k1;
            f[n2][k1] = cmul(f[n2][k1], mk<T2>(K.c9[e], -K.s9[e]));
        }
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
        T2 x[3] = {f[0][k1], f[1][k1], f[2][k1]};
        dft_odd_prime<3, T>(x, K.c3, K.s3);
        a[k1] = x[0]; a[k1 + 3] = x[1]; a[k1 + 6] = x[2];
    }
}

template <int R, typename T> __device__ __forceinline__ const T* kcos() {
#define FYG_SEL(r) if constexpr (R == r) return kc<T>().c##r; else
    FYG_CODELET_TABLES(FYG_SEL)
#undef FYG_SEL
    return nullptr;
}
template <int R, typename T> __device__ __forceinline__ const T* ksin() {
#define FYG_SEL(r) if constexpr (R == r) return kc<T>().s##r; else
    FYG_CODELET_TABLES(FYG_SEL)
#undef FYG_SEL
    return nullptr;
}

template <int R, typename T, typename T2> __device__ __forceinline__ void dft(T2* a);

// Composite codelet R = A*B in registers: n = B n1 + n2, k = k1 + A k2.
// DFT_A over n1, internal twiddle exp(-2 pi i n2 k1 / R), DFT_B over n2; natural-order output.
template <int A, int B, typename T, typename T2>
__device__ __forceinline__ void dft_comp(T2* a) {
    constexpr int R = A * B;
    const T* C = kcos<R, T>();
    const T* S = ksin<R, T>();
    T2 f[B][A];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
        T2 x[A];
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) x[n1] = a[B * n1 + n2];
        dft<A, T>(x);
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) f[n2][k1] = x[k1];
    }
#pragma unroll
    for (int n2 = 1; n2 < B; ++n2)
#pragma unroll
        for (int k1 = 1; k1 < A; ++k1) {
            const int e = (n2 * k1) % R;
            f[n2][k1] = cmul(f[n2][k1], mk<T2>(C[e], -S[e]));
        }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
        T2 x[B];
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) x[n2] = f[n2][k1];
        dft<B, T>(x);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) a[k1 + A * k2] = x[k2];
    }
}

// Stage radices the engine supports (host planner and kernel dispatch share this list).
#define FYG_STAGE_RADICES(X) \
    X(2) X(3) X(4) X(5) X(7) X(8) X(9) X(11) X(13) X(16) X(12) X(20) X(24) X(25) X(27) X(32)

template <int R, typename T, typename T2> __device__ __forceinline__ void dft(T2* a) {
    const CodeletConsts<T>& K = kc<T>();
    if constexpr (R == 2) dft2(a);
    else if constexpr (R == 3) dft_odd_prime<3, T>(a, K.c3, K.s3);
    else if constexpr (R == 4) dft4(a);
    else if constexpr (R == 5) dft_odd_prime<5, T>(a, K.c5, K.s5);
    else if constexpr (R == 7) dft_odd_prime<7, T>(a, K.c7, K.s7);
    else if constexpr (R == 8) dft8<T>(a);
    else if constexpr (R == 9) dft9<T>(a);
    else if constexpr (R == 11) dft_odd_prime<11, T>(a, K.c11, K.s11);
    else if constexpr (R == 13) dft_odd_prime<13, T>(a, K.c13, K.s13);
    else if constexpr (R == 16) dft16<T>(a);
    else if constexpr (R == 12) dft_comp<4, 3, T>(a);
    else if constexpr (R == 20) dft_comp<4, 5, T>(a);
    else if constexpr (R == 24) dft_comp<8, 3, T>(a);
    else if constexpr (R == 25) dft_comp<5, 5, T>(a);
    else if constexpr (R == 27) dft_comp<3, 9, T>(a);
    else if constexpr (R == 32) dft_comp<4, 8, T>(a);
}

}  // namespace fyg
