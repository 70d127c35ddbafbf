// Tile-pass kernels with FP32 arithmetic on FP32 data, stage radices up to 32.
#include "fyg_k_variant.cuh"
namespace fyg {
cudaError_t launch_f32c32(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st) {
    return launch_variant<float, float, float, 32>(p, grid, threads, smem, st);
}
}  // namespace fyg
