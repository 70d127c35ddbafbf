// Register-resident kernels of tile length 243 (all load variants).
#include "fyg_k_fast.cuh"
namespace fyg {
cudaError_t launch_fast_243(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st) {
    return launch_fast_shape<FastR243>(p, tmap, grid, st);
}
}  // namespace fyg
