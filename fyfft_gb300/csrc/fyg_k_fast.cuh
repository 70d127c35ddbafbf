// fyg_k_fast.cuh -- launch helpers of the register-resident kernels (fyg_fast.cuh); each
// fyg_k_fast<R>.cu translation unit instantiates the load variants of one tile shape.
#pragma once
#include "fyg_k_variant.cuh"
#include "fyg_fast.cuh"

namespace fyg {

template <class S, int LD, bool MID>
cudaError_t launch_fast_kernel(const PassParams& p, unsigned grid, cudaStream_t st) {
    auto kern = k_fast<S, LD, MID>;
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
    kern<<<grid, S::T, smem, st>>>(p);
    return cudaGetLastError();
}

// Load variant of a pass: the mid pass of a convolution always follows an earlier pass
// (inter-pass twiddle); other passes by load mode and position.
template <class S> cudaError_t launch_fast_shape(const PassParams& p, unsigned grid, cudaStream_t st) {
    if (p.mid) {
        if (p.load_mode != LD_PLAIN || p.Ns <= 1) return cudaErrorInvalidValue;
        return launch_fast_kernel<S, FL_TWIDDLE, true>(p, grid, st);
    }
    switch (p.load_mode) {
        case LD_CHIRP: return launch_fast_kernel<S, FL_CHIRP, false>(p, grid, st);
        case LD_GATHER: return launch_fast_kernel<S, FL_GATHER, false>(p, grid, st);
        default:
            return p.Ns > 1 ? launch_fast_kernel<S, FL_TWIDDLE, false>(p, grid, st)
                            : launch_fast_kernel<S, FL_PLAIN, false>(p, grid, st);
    }
}

}  // namespace fyg
