// Tile-pass kernels with FP64 arithmetic on FP64 data.
#include "fyg_k_variant.cuh"
namespace fyg {
cudaError_t launch_f64(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st) {
    return launch_variant<double, double, double, 16>(p, grid, threads, smem, st);
}
}  // namespace fyg
