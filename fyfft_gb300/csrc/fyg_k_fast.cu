// Shape table and dispatch of the register-resident FP32 kernels (fyg_fast.cuh); the kernels
// themselves are instantiated per tile length in fyg_k_fast<R>.cu.
#include "fyg_internal.h"
#include "fyg_fast.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

namespace fyg {

cudaError_t launch_fast_256(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_512(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_1024(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_2048(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_4096(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_243(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_343(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_256w(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_512w(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_1024w(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);
cudaError_t launch_fast_2048w(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st);

namespace {
template <class S> bool shape_of(int* C, int* threads, size_t* smem) {
    *C = S::C;
    *threads = S::T;
    *smem = S::smem_bytes();
    return true;
}
}  // namespace

bool fast_shape(int R, int wide, int* C, int* threads, size_t* smem) {
    if (wide) {
        switch (R) {
            case 256: return shape_of<FastR256W>(C, threads, smem);
            case 512: return shape_of<FastR512W>(C, threads, smem);
            case 1024: return shape_of<FastR1024W>(C, threads, smem);
            case 2048: return shape_of<FastR2048W>(C, threads, smem);
            default: break;   // no wide shape: the narrow one
        }
    }
    switch (R) {
        case 256: return shape_of<FastR256>(C, threads, smem);
        case 512: return shape_of<FastR512>(C, threads, smem);
        case 1024: return shape_of<FastR1024>(C, threads, smem);
        case 2048: return shape_of<FastR2048>(C, threads, smem);
        case 4096: return shape_of<FastR4096>(C, threads, smem);
        case 243: return shape_of<FastR243>(C, threads, smem);
        case 343: return shape_of<FastR343>(C, threads, smem);
        default: return false;
    }
}

namespace {
template <class S> int stages_of(int* radix, int* ns) {
    for (int s = 0; s < S::nst(); ++s) {
        radix[s] = S::radix(s);
        ns[s] = S::ns(s);
    }
    return S::nst();
}
}  // namespace

// In-tile stage schedule of a register-resident tile length (the same for both widths).
int fast_stages(int R, int* radix, int* ns) {
    switch (R) {
        case 256: return stages_of<FastR256>(radix, ns);
        case 512: return stages_of<FastR512>(radix, ns);
        case 1024: return stages_of<FastR1024>(radix, ns);
        case 2048: return stages_of<FastR2048>(radix, ns);
        case 4096: return stages_of<FastR4096>(radix, ns);
        case 243: return stages_of<FastR243>(radix, ns);
        case 343: return stages_of<FastR343>(radix, ns);
        default: return 0;
    }
}

int fast_points(int R) {
    switch (R) {
        case 256: return FastR256::P;
        case 512: return FastR512::P;
        case 1024: return FastR1024::P;
        case 2048: return FastR2048::P;
        case 4096: return FastR4096::P;
        case 243: return FastR243::P;
        case 343: return FastR343::P;
        default: return 0;
    }
}

// Tables in the fast kernels' thread order: entry ((t P + i) T + tid) belongs to thread
// tid = g C + c of tile t, register i, i.e. point n = g + G i of column jj = t C + c.
//   kind 0: inter-pass twiddle exp(-2 pi i n jj Lr / L), from the FP64 sincospi of the exactly
//           reduced exponent, rounded once
//   kind 1: src[jj + n Rr] (conjugated if conj), zero at and above nvalid
__global__ void k_fast_table(float2* out, uint64_t total, int P, int C, int T, int kind, uint64_t Lr, uint64_t L,
                             uint64_t Rr, const float2* src, int64_t nvalid, int conj) {
    const int G = T / C;
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int tid = (int)(idx % T);
        const uint64_t q = idx / T;
        const int i = (int)(q % P);
        const uint64_t t = q / P;
        const int c = tid % C, g = tid / C;
        const uint64_t n = (uint64_t)g + (uint64_t)G * i, jj = t * C + c;
        float2 w;
        if (kind == 0) {
            const uint64_t e = (n * jj % L) * Lr % L;
            double sn, cs;
            sincospi(2.0 * (double)e / (double)L, &sn, &cs);
            w = make_float2((float)cs, (float)-sn);
        } else {
            const uint64_t gi = jj + n * Rr;
            w = (int64_t)gi < nvalid ? src[gi] : make_float2(0.f, 0.f);
            if (conj) w.y = -w.y;
        }
        out[idx] = w;
    }
}

cudaError_t launch_fast_table(float2* out, uint64_t total, int R, int wide, int kind, uint64_t Lr, uint64_t L,
                              uint64_t Rr, const float2* src, int64_t nvalid, int conj, cudaStream_t st) {
    int C = 0, T = 0;
    size_t smem = 0;
    if (!fast_shape(R, wide, &C, &T, &smem)) return cudaErrorInvalidValue;
    const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, 1u << 16);
    k_fast_table<<<blocks, 256, 0, st>>>(out, total, fast_points(R), C, T, kind, Lr, L, Rr, src, nvalid, conj);
    return cudaGetLastError();
}

// Tensor map of a pass input for the TMA loads: rows of 2 Rr floats (the Rr columns of one point
// index of one transform), `rows` rows (transforms x R), boxes of 2C floats x min(R, 256) rows.
// cuTensorMapEncodeTiled comes from the driver through the runtime's entry-point query (no
// link against the driver library).
cudaError_t encode_tile_map(CUtensorMap* map, const void* base, uint64_t Rr, uint64_t rows, int C, int R) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    });
    if (!encode) return cudaErrorNotSupported;
    if ((reinterpret_cast<uintptr_t>(base) & 15) || ((Rr * 8) & 15)) return cudaErrorInvalidValue;
    const cuuint64_t dims[2] = {2 * Rr, rows};
    const cuuint64_t strides[1] = {Rr * sizeof(float2)};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * C), (cuuint32_t)std::min(R, 256)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_fast(const PassParams& p, const CUtensorMap* tmap, unsigned grid, cudaStream_t st) {
    // wide shapes are told apart by their column count
    switch (p.g.R) {
        case 256: if (p.g.C == FastR256W::C) return launch_fast_256w(p, tmap, grid, st); break;
        case 512: if (p.g.C == FastR512W::C) return launch_fast_512w(p, tmap, grid, st); break;
        case 1024: if (p.g.C == FastR1024W::C) return launch_fast_1024w(p, tmap, grid, st); break;
        case 2048: if (p.g.C == FastR2048W::C) return launch_fast_2048w(p, tmap, grid, st); break;
        default: break;
    }
    switch (p.g.R) {
        case 256: return launch_fast_256(p, tmap, grid, st);
        case 512: return launch_fast_512(p, tmap, grid, st);
        case 1024: return launch_fast_1024(p, tmap, grid, st);
        case 2048: return launch_fast_2048(p, tmap, grid, st);
        case 4096: return launch_fast_4096(p, tmap, grid, st);
        case 243: return launch_fast_243(p, tmap, grid, st);
        case 343: return launch_fast_343(p, tmap, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fyg
