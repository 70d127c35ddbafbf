// fyg_k_variant.cuh -- explicit instantiation helper for one tile-pass kernel variant.
#pragma once
#include "fyg_internal.h"
#include "fyg_kernels.cuh"

namespace fyg {

template <typename T, typename TI, typename TO, int CLASS, bool COLMAJOR, int TAG = 0>
cudaError_t launch_layout(const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st) {
    auto kern = k_pass<T, TI, TO, CLASS, COLMAJOR, TAG>;
    constexpr int kMaxDev = 64;
    static size_t smem_set[kMaxDev] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (smem > 48 * 1024 && dev < kMaxDev && smem > smem_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        smem_set[dev] = smem;
    }
    kern<<<grid, threads, smem, st>>>(p);
    return cudaGetLastError();
}

template <typename T, typename TI, typename TO, int CLASS, int TAG = 0>
cudaError_t launch_variant(const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st) {
    if (p.g.colmajor) return launch_layout<T, TI, TO, CLASS, true, TAG>(p, grid, threads, smem, st);
    return launch_layout<T, TI, TO, CLASS, false, TAG>(p, grid, threads, smem, st);
}

// Copies the codelet constants into this translation unit's __constant__ tables.
static cudaError_t upload_consts_tu(const CodeletConsts<float>& kf, const CodeletConsts<double>& kd) {
    cudaError_t e = cudaMemcpyToSymbol(g_kf, &kf, sizeof(kf));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_kd, &kd, sizeof(kd));
    return e;
}
static const bool g_consts_registered = register_const_uploader(&upload_consts_tu);

}  // namespace fyg
