// Tile-pass kernels with FP32 arithmetic on FP32 data.
#include "fyg_k_variant.cuh"
namespace fyg {
cudaError_t launch_f32(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st) {
    return launch_variant<float, float, float, 16>(p, grid, threads, smem, st);
}
}  // namespace fyg
