// Register-resident kernels of tile length 2048, wide shape (512 threads, all load variants).
#include "fyg_k_fast.cuh"
namespace fyg {
cudaError_t launch_fast_2048w(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st) {
    return launch_fast_shape<FastR2048W>(p, tmap, grid, st);
}
}  // namespace fyg
