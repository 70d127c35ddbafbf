// fyg_k_fast.cuh -- launch helpers of the register-resident kernels (fyg_fast.cuh); each
// fyg_k_fast<R>.cu translation unit instantiates the load variants of one tile shape.
#pragma once
#include "fyg_k_variant.cuh"
#include "fyg_fast.cuh"

namespace fyg {

template <class S, int LD, bool MID, bool TMA = false>
cudaError_t launch_fast_kernel(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st) {
    auto kern = k_fast<S, LD, MID, TMA>;
    const size_t smem = S::smem_bytes();
    constexpr int kMaxDev = 64;
    static bool attr_set[kMaxDev] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (smem > 48 * 1024 && dev < kMaxDev && !attr_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    static const CUtensorMap none = {};
    kern<<<grid, S::T, smem, st>>>(p, tmap ? *tmap : none);
    return cudaGetLastError();
}

// Load variant of a pass: the mid pass of a convolution always follows an earlier pass
// (inter-pass twiddle); other passes by load mode and position.  A tensor map selects the TMA
// form of the twiddle-load variants (passes after the first).
template <class S>
cudaError_t launch_fast_shape(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st) {
    constexpr bool tma_ok = S::R % 256 == 0;
    if (p.mid) {
        if (p.load_mode != LD_PLAIN || p.Ns <= 1) return cudaErrorInvalidValue;
        if constexpr (tma_ok)
            if (tmap) return launch_fast_kernel<S, FL_TWIDDLE, true, true>(p, tmap, grid, st);
        return launch_fast_kernel<S, FL_TWIDDLE, true>(p, nullptr, grid, st);
    }
    switch (p.load_mode) {
        case LD_CHIRP: return launch_fast_kernel<S, FL_CHIRP, false>(p, nullptr, grid, st);
        case LD_GATHER: return launch_fast_kernel<S, FL_GATHER, false>(p, nullptr, grid, st);
        default:
            if (p.Ns > 1) {
                if constexpr (tma_ok)
                    if (tmap) return launch_fast_kernel<S, FL_TWIDDLE, false, true>(p, tmap, grid, st);
                return launch_fast_kernel<S, FL_TWIDDLE, false>(p, nullptr, grid, st);
            }
            return launch_fast_kernel<S, FL_PLAIN, false>(p, nullptr, grid, st);
    }
}

}  // namespace fyg
