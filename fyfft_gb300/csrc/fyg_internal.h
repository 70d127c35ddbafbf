// fyg_internal.h -- host-side declarations shared by the library's translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "fyg_pass.cuh"

namespace fyg {

// Tile-pass kernel variants: compute type / input type / output type and radix class; all are
// launched with at most 512 threads per CTA.
enum KernelVariant : int {
    KV_F32_C16 = 0,     // float  compute, float  I/O, stage radices <= 16
    KV_F32_C32,         // float  compute, float  I/O, stage radices <= 32
    KV_F64_C16,         // double compute, double I/O
    KV_F64_IF32_C16,    // double compute, float in,  double out
    KV_F64_OF32_C16,    // double compute, double in, float out
    KV_F64_F32IO_C16,   // double compute, float in,  float out
    KV_FAST,            // register-resident FP32 kernel of a power-of-two tile length (fyg_fast.cuh)
    KV_SPLIT_F32,       // first pass of the N = m p split (fyg_split.cu), complex<float>
    KV_SPLIT_F64,       // the same, complex<double>
    KV_COUNT
};

struct VariantInfo { int maxt, compute_bytes; };
VariantInfo variant_info(int kv);

// Launches one tile pass; sets the dynamic shared-memory attribute when needed.
cudaError_t launch_pass(int kv, const PassParams& p, unsigned grid, int threads, size_t smem,
                        cudaStream_t st, const CUtensorMap* tmap = nullptr);

// First pass of the N = m p split: g.R = m, g.C = split_threads() columns per CTA.
int split_threads();
cudaError_t launch_split(int kv, const PassParams& p, unsigned grid, cudaStream_t st);

// Register-resident kernels: the tile shape for R (false if R has none) and the launch.
bool fast_shape(int R, int wide, int* C, int* threads, size_t* smem);
int fast_points(int R);
int fast_stages(int R, int* radix, int* ns);   // returns the stage count (radix / ns per stage)
cudaError_t launch_fast(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
// Tensor map of a register-resident pass input for TMA tile loads (fyg_k_fast.cu).
cudaError_t encode_tile_map(CUtensorMap* map, const void* base, uint64_t Rr, uint64_t rows, int C, int R);
// Thread-order tables of the register-resident kernels (kind 0: inter-pass twiddles, kind 1:
// gather of src with optional conjugation and zero padding); see k_fast_table.
cudaError_t launch_fast_table(float2* out, uint64_t total, int R, int wide, int kind, uint64_t Lr, uint64_t L,
                              uint64_t Rr, const float2* src, int64_t nvalid, int conj, cudaStream_t st);

// Uploads the codelet constant tables to the current device (once per device).
cudaError_t ensure_device_constants();

// Host values of the codelet constant tables (for translation units that upload their own).
void codelet_consts(CodeletConsts<float>* kf, CodeletConsts<double>* kd);

// Every translation unit that launches kernels holds its own __constant__ codelet tables (no
// relocatable device code) and registers an uploader for them at static initialization;
// ensure_device_constants() runs all registered uploaders once per device.
using ConstUploader = cudaError_t (*)(const CodeletConsts<float>&, const CodeletConsts<double>&);
bool register_const_uploader(ConstUploader f);

// Device RNG fill (fyg_fill_random_device).
cudaError_t launch_fill_random(uint64_t seed, int dist, int dtype, size_t first, size_t n, void* out,
                               cudaStream_t st);

// Small helper kernels.
cudaError_t launch_delay(unsigned long long ns, cudaStream_t st);
cudaError_t launch_convert_d2f(const double2* in, float2* out, size_t n, cudaStream_t st);

}  // namespace fyg
