// Register-resident FP32 tile-pass kernels for power-of-two tile lengths (fyg_fast.cuh).
#include "fyg_k_variant.cuh"
#include "fyg_fast.cuh"

namespace fyg {

namespace {

template <class S> cudaError_t launch_shape(const PassParams& p, unsigned grid, cudaStream_t st) {
    auto kern = k_fast<S>;
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

// R -> (P, C): 256 threads per CTA up to R = 2048
using F256 = FastShape<256, 16, 16>;
using F512 = FastShape<512, 32, 16>;
using F1024 = FastShape<1024, 32, 8>;
using F2048 = FastShape<2048, 32, 4>;
using F4096 = FastShape<4096, 32, 4>;

template <class S> bool shape_of(int* C, int* threads, size_t* smem) {
    *C = S::C;
    *threads = S::T;
    *smem = S::smem_bytes();
    return true;
}

}  // namespace

bool fast_shape(int R, int* C, int* threads, size_t* smem) {
    switch (R) {
        case 256: return shape_of<F256>(C, threads, smem);
        case 512: return shape_of<F512>(C, threads, smem);
        case 1024: return shape_of<F1024>(C, threads, smem);
        case 2048: return shape_of<F2048>(C, threads, smem);
        case 4096: return shape_of<F4096>(C, threads, smem);
        default: return false;
    }
}

cudaError_t launch_fast(const PassParams& p, unsigned grid, cudaStream_t st) {
    switch (p.g.R) {
        case 256: return launch_shape<F256>(p, grid, st);
        case 512: return launch_shape<F512>(p, grid, st);
        case 1024: return launch_shape<F1024>(p, grid, st);
        case 2048: return launch_shape<F2048>(p, grid, st);
        case 4096: return launch_shape<F4096>(p, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fyg
