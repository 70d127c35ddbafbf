// Tile-pass kernels with FP64 arithmetic on FP64 data.
#include "fyg_k_variant.cuh"
namespace fyg {
cudaError_t launch_f64(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st) {
    return launch_variant<double, double, double, 16>(p, grid, threads, smem, st);
}
cudaError_t upload_consts_f64(const CodeletConsts<float>& kf, const CodeletConsts<double>& kd) {
    return upload_consts_tu(kf, kd);
}
}  // namespace fyg
