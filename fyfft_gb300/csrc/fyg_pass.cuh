// fyg_pass.cuh -- the tile-pass kernel: one Stockham radix-R pass of a length-L transform,
// executed as in-CTA FFTs of length R over a tile of C "columns".
//
// Transform-level view (the pass is one radix-R step of a self-sorting Stockham FFT over the
// whole length L, with Ns = product of the radices of the earlier passes and Rr = L/R):
//   column j in [0, Rr), k = j mod Ns
//   inputs   x[j + m*Rr]                         m in [0, R)
//   twiddle  * exp(-2 pi i m k / (Ns R))         (computed from a two-level table of w_L)
//   DFT_R over m
//   outputs  y[(j/Ns)*Ns*R + k + m'*Ns]          m' in [0, R)
// A CTA owns C consecutive columns (of one or several transforms of a batch): C-element
// contiguous segments on the strided side keep HBM access coalesced, and for a single-pass
// transform (R = L, Rr = 1) the columns are whole transforms that sit back to back in memory.
// This replaces the reference's TRANSPOSE / FUSED_TWIDDLE_TRANSPOSE / leaf-op interpreter
// (src/foye_FFT_mix_radix.hpp:16-83, :536-574) and its radix engines' bit/digit-reversal LUTs:
// Stockham indexing sorts itself.
//
// Inside the CTA the length-R DFT is again a Stockham sweep over radix-r stages: ping-ponging
// in shared memory between a coalesced load phase and a coalesced store phase (the tile kernel,
// fyg_kernels.cuh), or on points held in registers with one shared exchange per stage (the
// register-resident kernels, fyg_fast.cuh).
//
// Fusions (all selected by uniform runtime fields):
//   load  LD_PLAIN   x (optionally conjugated)
//         LD_CHIRP   Bluestein: x[n] * conj(w[n]) for n < nvalid, zero padding above
//                    (src/foye_FFT_bluestein.hpp:268-313)
//         LD_GATHER  Rader: x[gather[n]] (gather < 0 -> zero padding)  (src/foye_FFT_rader.hpp:83-102)
//   mid   after the forward in-CTA FFT: multiply by a precomputed spectrum, conjugate and run a
//         second in-CTA FFT (= the first pass of the inverse transform, which consumes exactly
//         the columns this CTA holds)  (src/foye_FFT_utility.hpp:211-263 + the IFFT_M call)
//   store ST_PLAIN   y * scale (optionally conjugated)
//         ST_CHIRP   Bluestein: w[k] * y * scale (conjugated for forward), k < nvalid
//                    (src/foye_FFT_bluestein.hpp:315-354)
//         ST_SCATTER Rader: out[scatter[k]] = (x0 + y*scale (conj for forward)) * scale2, and the
//                    DC term out[0] = (x0 + A0) * scale2  (src/foye_FFT_rader.hpp:104-140, :380-398)
#pragma once
#include "fyg_device.cuh"

namespace fyg {

constexpr int kMaxStages = 16;

enum LoadMode : int { LD_PLAIN = 0, LD_CHIRP = 1, LD_GATHER = 2 };
enum StoreMode : int { ST_PLAIN = 0, ST_CHIRP = 1, ST_SCATTER = 2 };

struct TileGeom {
    int R;          // in-CTA transform length
    int C;          // columns per tile
    int log2C;      // for the element-major layout (C a power of two)
    int colmajor;   // 1: columns are whole contiguous transforms; 0: element-major column tile
    int nst;        // in-CTA stages
    int radix[kMaxStages];
    int twmul[kMaxStages];     // R / (ns * radix): local twiddle exponent multiplier
    int twoff[kMaxStages];     // offset of the stage's block in the stage-twiddle table
    FastDiv ns[kMaxStages];    // local Ns before the stage
    FastDiv rr[kMaxStages];    // R / radix (butterflies per column)
    FastDiv divR;              // R (element index -> column, column-major order)
};

struct alignas(16) PassParams {
    TileGeom g;
    // transform-level geometry of this pass
    int64_t ncols;       // batch * Rr
    int64_t idist, odist;
    int Rr;              // L / R
    int Ns;              // product of the radices of earlier passes
    int Ns_out;          // Ns used for the output index (1 for the fused mid pass)
    int Lr;              // L / (Ns * R): inter-pass twiddle exponent multiplier
    FastDiv div_Rr, div_Ns, div_Ns_out;
    const void* in;
    void* out;
    // twiddles
    const void* tw_local;    // w_R^t, t in [0, R)                        (T2)
    const void* tw_hi;       // w_L^(i*2^tw_shift) (float: hi/lo pairs)    (T2 or float4)
    const void* tw_lo;       // w_L^j, j < 2^tw_shift
    int tw_shift;
    // modes
    int load_mode, store_mode, conj_in, conj_out;
    double scale, scale2;
    int64_t nvalid;          // Bluestein: valid length N
    const void* chirp;       // Bluestein chirp w[n] = exp(+i pi (n^2 mod 2N)/N), n < N (T2)
    const int* gather;       // Rader input map (length L, -1 = zero)
    const int* scatter;      // Rader output map (length L, -1 = skip)
    void* x0buf;             // Rader: per-transform x[0] (written by the first pass, T2)
    void* dcbuf;             // Rader: per-transform DC term of the forward convolution FFT (T2)
    int x0_from_in;          // Rader: first pass (x0 read from the input, saved to x0buf)
    int dc_capture;          // Rader: the mid pass saves the DC term to dcbuf
    int mid;                 // fused spectrum multiply + second in-CTA FFT
    const void* spectrum;    // length L (T2)
    int* err;                // device error word (bounds violations are recorded, never trapped)
    // uneven batches: transform b of this pass reads/writes the user buffers at
    // offsets[ids[b]] (elements) instead of b * idist / b * odist; null for contiguous batches
    const int64_t* in_offsets;
    const int64_t* out_offsets;
    const int* ids;
    // uneven batches: 1 when in/out is the user buffer (patched in by the persistent kernel)
    int in_user, out_user;
    // register-resident kernels (fyg_fast.cuh): tables laid out in the kernel's thread order,
    // entry ((t P + i) T + tid) for tile t of a transform, register i of thread tid; null when
    // not built.  tw_tiled: inter-pass twiddles of the first Ns/C tiles (the pattern repeats
    // with period tw_tile_period = Ns/C tiles); tab_tiled: the spectrum (mid pass), the
    // conjugated zero-padded chirp (chirp load) or the chirp (chirp store)
    const void* tw_tiled;
    const void* tab_tiled;
    int tw_tile_period;
    // register-resident kernels: 1 = tiles in reverse order (odd passes of a pipeline start on
    // the tail the previous pass left in L2)
    int reverse_tiles;
    // register-resident kernels: in-tile stage twiddles, one block per stage s >= 1 holding
    // w_R^(m k twm_s) at m ns_s + k (m < radix, k < ns_s), so that the lanes of a warp (consecutive
    // k for a fixed m) read consecutive entries
    const void* tw_stage;
    // N = m p split (m > 1): transform b of this pass is sub-transform k1 = b mod m of user
    // transform b / m, whose outputs sit at elements k1 + m k of that transform (Rader scatter
    // store); 0 otherwise
    int split_m;
};

__device__ __forceinline__ int64_t transform_base(const int64_t* offs, const int* ids, int64_t b, int64_t dist) {
    return offs ? offs[ids ? ids[b] : b] : b * dist;
}

// Output base of transform b of a pass (the N = m p split interleaves m sub-transforms).
__device__ __forceinline__ int64_t out_transform_base(const PassParams& p, int64_t b) {
    if (p.split_m > 1) {
        const int64_t u = b / p.split_m;
        return transform_base(p.out_offsets, p.ids, u, p.odist) + (b - u * p.split_m);
    }
    return transform_base(p.out_offsets, p.ids, b, p.odist);
}

// Data loads go through L2 only (ld.global.cg): every element is read once, and inside one
// persistent batch launch a scratch region can be rewritten by a later pass, so no L1 copy of
// it may survive.
__device__ __forceinline__ float2 ld_data(const float2* p) { return __ldcg(p); }
__device__ __forceinline__ double2 ld_data(const double2* p) { return __ldcg(p); }

// Per-column state: the transform b a column belongs to, its column index jj inside the pass,
// the inter-pass twiddle index k = jj mod Ns, the output column offset and the global bases.
template <typename T> struct Col {
    int64_t in_base, out_base;
    int jj, k, out_j, b, valid;
    cplx<T> x0;
};

constexpr int kMaxThreads = 512;

__host__ __device__ inline int colmajor_pitch(int R) { return R + (R >> 4) + 1; }

__host__ __device__ inline size_t tile_elems(int R, int C, int colmajor) {
    return colmajor ? (size_t)C * colmajor_pitch(R) : (size_t)R * (C + 1);
}

// Per-column output state kept in shared memory for the store phase.
template <typename T> struct ColHead {
    int64_t out_base;
    int out_j, b, valid, pad;
    cplx<T> x0;
};

// Stage schedule copied to shared memory at kernel start (parameter arrays cannot be indexed
// by a run-time stage number without a local-memory copy).
struct StageDesc {
    int radix, twm, twoff;
    FastDiv ns, rr;
};

template <typename T>
__host__ __device__ inline size_t tile_head_bytes(int C) {
    return (((size_t)kMaxStages * sizeof(StageDesc) + (size_t)C * sizeof(ColHead<T>)) + 15) & ~(size_t)15;
}
template <typename T>
__host__ __device__ inline size_t tile_smem_bytes(int R, int C, int colmajor) {
    return tile_head_bytes<T>(C) + 2 * tile_elems(R, C, colmajor) * sizeof(cplx<T>);
}

// ---- inter-pass twiddle exp(-2 pi i e / L) from the two-level table ----
__device__ __forceinline__ float2 tw_two_level(const void* hi, const void* lo, int shift, uint32_t e, float) {
    const float4 A = __ldg(reinterpret_cast<const float4*>(hi) + (e >> shift));
    const float4 B = __ldg(reinterpret_cast<const float4*>(lo) + (e & ((1u << shift) - 1)));
    // (Ah + Al)(Bh + Bl) with the small cross terms folded in before the final rounding
    const float cr = fmaf(A.x, B.z, fmaf(-A.y, B.w, fmaf(A.z, B.x, -A.w * B.y)));
    const float ci = fmaf(A.x, B.w, fmaf(A.y, B.z, fmaf(A.z, B.y, A.w * B.x)));
    return make_float2(fmaf(A.x, B.x, fmaf(-A.y, B.y, cr)), fmaf(A.x, B.y, fmaf(A.y, B.x, ci)));
}
__device__ __forceinline__ double2 tw_two_level(const void* hi, const void* lo, int shift, uint32_t e, double) {
    const double2 A = __ldg(reinterpret_cast<const double2*>(hi) + (e >> shift));
    const double2 B = __ldg(reinterpret_cast<const double2*>(lo) + (e & ((1u << shift) - 1)));
    return cmul(A, B);
}

// Column state of global column q of this pass.
template <typename T, typename TI>
__device__ __forceinline__ Col<T> make_col(const PassParams& p, int64_t q) {
    using T2 = cplx<T>;
    Col<T> ci;
    ci.valid = q < p.ncols;
    const uint32_t qq = (uint32_t)(ci.valid ? q : 0);
    const uint32_t b = p.div_Rr.div(qq);
    const uint32_t jj = qq - b * (uint32_t)p.Rr;
    ci.b = (int)b;
    ci.jj = (int)jj;
    ci.k = (int)(jj - p.div_Ns.div(jj) * (uint32_t)p.Ns);
    const uint32_t qo = p.div_Ns_out.div(jj);
    ci.out_j = (int)(qo * (uint32_t)p.Ns_out * (uint32_t)p.g.R + (jj - qo * (uint32_t)p.Ns_out));
    ci.in_base = transform_base(p.in_offsets, p.ids, b, p.idist);
    ci.out_base = out_transform_base(p, b);
    ci.x0 = mk<T2>(T(0), T(0));
    return ci;
}

}  // namespace fyg
