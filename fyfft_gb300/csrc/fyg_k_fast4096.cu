// Register-resident kernels of tile length 4096 (all load variants).
#include "fyg_k_fast.cuh"
namespace fyg {
cudaError_t launch_fast_4096(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st) {
    return launch_fast_shape<FastR4096>(p, tmap, grid, st);
}
}  // namespace fyg
