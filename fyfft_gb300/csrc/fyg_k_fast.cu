// Shape table and dispatch of the register-resident FP32 kernels (fyg_fast.cuh); the kernels
// themselves are instantiated per tile length in fyg_k_fast<R>.cu.
#include "fyg_internal.h"
#include "fyg_fast.cuh"

namespace fyg {

cudaError_t launch_fast_256(const PassParams& p, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_512(const PassParams& p, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_1024(const PassParams& p, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_2048(const PassParams& p, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_4096(const PassParams& p, unsigned grid, cudaStream_t st);

namespace {
template <class S> bool shape_of(int* C, int* threads, size_t* smem) {
    *C = S::C;
    *threads = S::T;
    *smem = S::smem_bytes();
    return true;
}
}  // namespace

bool fast_shape(int R, int* C, int* threads, size_t* smem) {
    switch (R) {
        case 256: return shape_of<FastR256>(C, threads, smem);
        case 512: return shape_of<FastR512>(C, threads, smem);
        case 1024: return shape_of<FastR1024>(C, threads, smem);
        case 2048: return shape_of<FastR2048>(C, threads, smem);
        case 4096: return shape_of<FastR4096>(C, threads, smem);
        default: return false;
    }
}

cudaError_t launch_fast(const PassParams& p, unsigned grid, cudaStream_t st) {
    switch (p.g.R) {
        case 256: return launch_fast_256(p, grid, st);
        case 512: return launch_fast_512(p, grid, st);
        case 1024: return launch_fast_1024(p, grid, st);
        case 2048: return launch_fast_2048(p, grid, st);
        case 4096: return launch_fast_4096(p, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fyg
