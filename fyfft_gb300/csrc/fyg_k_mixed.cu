// Tile-pass kernels with FP64 arithmetic on FP32 input and/or output: the FP64 convolution
// of FP32 Rader/Bluestein plans whose length breaks the FP32 error budget.
#include "fyg_k_variant.cuh"
namespace fyg {
cudaError_t launch_mixed(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st) {
    if (kv == KV_F64_IF32_C16) return launch_variant<double, float, double, 16>(p, grid, threads, smem, st);
    if (kv == KV_F64_OF32_C16) return launch_variant<double, double, float, 16>(p, grid, threads, smem, st);
    return launch_variant<double, float, float, 16>(p, grid, threads, smem, st);
}
}  // namespace fyg
