// fyg_split.cu -- the first pass of the N = m p split (p prime with a cyclic Rader convolution,
// 2 <= m <= 8), the planner's alternative to a Bluestein convolution of length >= 2N - 1:
//
//   X[k1 + m k2] = sum_{n2 < p} w_p^(n2 k2) z_k1[n2]                       (w_q = exp(-2 pi i / q))
//   z_k1[n2]     = w_N^(n2 k1) sum_{n1 < m} x[n2 + p n1] w_m^(n1 k1)
//
// (the index maps n = n2 + p n1, k = k1 + m k2; w_N^(p n1 m k2) = 1).  This kernel writes the
// z_k1 of every transform, contiguous per k1; the m length-p transforms then run as the Rader
// passes of fyg_plan.cu, whose scatter store writes X[k1 + m k2] (PassParams::split_m).  Inverse
// transforms conjugate every twiddle.  One thread per (transform, n2): the m loads (stride p)
// and the m stores are coalesced across a warp.  The twiddle table holds w_N^t for t < N, which
// both n2 k1 < N and ((n1 k1) mod m) p < N index directly.
//
// The reference has no counterpart: it runs such lengths as Bluestein convolutions up to 39062
// and as a direct DFT above (foye_FFT.hpp:162-184).
#include "fyg_internal.h"

namespace fyg {
namespace {

constexpr int kSplitThreads = 256;

// PassParams fields: in / in_offsets / ids / idist (user input), out (z, odist = N per
// transform), Rr = p with div_Rr, g.R = m, ncols = transforms x p, conj_in (inverse), tw_stage
// (the w_N^t table).
template <typename T, int M>
__global__ void __launch_bounds__(kSplitThreads) k_split(const __grid_constant__ PassParams p) {
    using T2 = cplx<T>;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= p.ncols) return;
    const uint32_t b = p.div_Rr.div((uint32_t)q);
    const uint32_t j = (uint32_t)q - b * (uint32_t)p.Rr;
    const int64_t P = p.Rr;
    const T2* x = reinterpret_cast<const T2*>(p.in) + transform_base(p.in_offsets, p.ids, b, p.idist) + j;
    T2* z = reinterpret_cast<T2*>(p.out) + (int64_t)b * p.odist + j;
    const T2* W = reinterpret_cast<const T2*>(p.tw_stage);
    const T sgn = p.conj_in ? T(-1) : T(1);
    T2 v[M], wm[M];
#pragma unroll
    for (int i = 0; i < M; ++i) v[i] = ld_data(x + i * P);
#pragma unroll
    for (int r = 1; r < M; ++r) {
        const T2 w = __ldg(W + r * P);
        wm[r] = mk<T2>(w.x, sgn * w.y);
    }
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
        T2 acc = v[0];
#pragma unroll
        for (int n1 = 1; n1 < M; ++n1) {
            const int e = (n1 * k1) % M;
            acc = e == 0 ? cadd(acc, v[n1]) : cadd(acc, cmul(v[n1], wm[e]));
        }
        if (k1) {
            const T2 w = __ldg(W + (int64_t)j * k1);
            acc = cmul(acc, mk<T2>(w.x, sgn * w.y));
        }
        z[k1 * P] = acc;
    }
}

template <typename T, int M>
cudaError_t go(const PassParams& p, unsigned grid, cudaStream_t st) {
    k_split<T, M><<<grid, kSplitThreads, 0, st>>>(p);
    return cudaGetLastError();
}

template <typename T>
cudaError_t dispatch(const PassParams& p, unsigned grid, cudaStream_t st) {
    switch (p.g.R) {
        case 2: return go<T, 2>(p, grid, st);
        case 3: return go<T, 3>(p, grid, st);
        case 4: return go<T, 4>(p, grid, st);
        case 5: return go<T, 5>(p, grid, st);
        case 6: return go<T, 6>(p, grid, st);
        case 7: return go<T, 7>(p, grid, st);
        case 8: return go<T, 8>(p, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

int split_threads() { return kSplitThreads; }

cudaError_t launch_split(int kv, const PassParams& p, unsigned grid, cudaStream_t st) {
    if (p.g.C != kSplitThreads) return cudaErrorInvalidValue;
    return kv == KV_SPLIT_F64 ? dispatch<double>(p, grid, st) : dispatch<float>(p, grid, st);
}

}  // namespace fyg
