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
// Inside the CTA the length-R DFT is again a Stockham sweep over radix-r stages; stage 0 loads
// straight from global memory into registers (coalesced), intermediate stages exchange through
// shared memory, and the last stage stores straight to global memory.
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
    int colmajor;   // 1: smem[c*R + n] (columns are whole contiguous transforms); 0: smem[n*C + c]
    int nst;        // in-CTA stages
    int radix[kMaxStages];
    int twmul[kMaxStages];     // R / (ns * radix): local twiddle exponent multiplier
    FastDiv ns[kMaxStages];    // local Ns before the stage
    FastDiv rr[kMaxStages];    // R / radix (butterflies per column)
};

struct PassParams {
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
};

template <typename T> struct ColInfo {
    int64_t in_base, out_base;
    int jj, k, out_j, b, valid, pad;
    cplx<T> x0;
};

// Shared memory: ColInfo[C], then two R*C complex buffers (none when one stage and no mid).
template <typename T>
__host__ __device__ inline size_t pass_smem_bytes(int R, int C, int nst, int mid) {
    const size_t ci = ((size_t)C * sizeof(ColInfo<T>) + 15) & ~(size_t)15;
    const size_t nbuf = (nst > 1 || mid) ? 2 : 0;
    return ci + nbuf * (size_t)R * C * sizeof(cplx<T>);
}


// ---- inter-pass twiddle exp(-2 pi i e / L) from the two-level table ----
__device__ __forceinline__ float2 tw_two_level(const PassParams& p, uint32_t e, float) {
    const float4 A = __ldg(reinterpret_cast<const float4*>(p.tw_hi) + (e >> p.tw_shift));
    const float4 B = __ldg(reinterpret_cast<const float4*>(p.tw_lo) + (e & ((1u << p.tw_shift) - 1)));
    // (Ah + Al)(Bh + Bl) with the small cross terms folded in before the final rounding
    const float cr = fmaf(A.x, B.z, fmaf(-A.y, B.w, fmaf(A.z, B.x, -A.w * B.y)));
    const float ci = fmaf(A.x, B.w, fmaf(A.y, B.z, fmaf(A.z, B.y, A.w * B.x)));
    return make_float2(fmaf(A.x, B.x, fmaf(-A.y, B.y, cr)), fmaf(A.x, B.y, fmaf(A.y, B.x, ci)));
}
__device__ __forceinline__ double2 tw_two_level(const PassParams& p, uint32_t e, double) {
    const double2 A = __ldg(reinterpret_cast<const double2*>(p.tw_hi) + (e >> p.tw_shift));
    const double2 B = __ldg(reinterpret_cast<const double2*>(p.tw_lo) + (e & ((1u << p.tw_shift) - 1)));
    return cmul(A, B);
}

template <typename T, typename TI, typename TO>
struct PassCtx {
    using T2 = cplx<T>;
    using IN2 = cplx<TI>;
    using OUT2 = cplx<TO>;
    const PassParams& p;
    T2* sm;
    ColInfo<T>* col;

    __device__ __forceinline__ int saddr(int c, int n) const {
        return p.g.colmajor ? c * p.g.R + n : (n << p.g.log2C) + c;
    }

    // element n (in-CTA index) of column c, from global memory, with the load fusions
    __device__ __forceinline__ T2 load(int c, int n) const {
        const ColInfo<T>& ci = col[c];
        T2 v = mk<T2>(T(0), T(0));
        if (!ci.valid) return v;
        const int64_t gidx = (int64_t)ci.jj + (int64_t)n * p.Rr;
        const IN2* in = reinterpret_cast<const IN2*>(p.in);
        if (p.load_mode == LD_PLAIN) {
            v = to_c(in[ci.in_base + gidx], T());
        } else if (p.load_mode == LD_CHIRP) {
            if (gidx < p.nvalid) {
                v = to_c(in[ci.in_base + gidx], T());
                if (p.conj_in) v = cconj(v);
                v = cmul(v, cconj(__ldg(reinterpret_cast<const T2*>(p.chirp) + gidx)));
            }
            return v;
        } else {
            const int t = __ldg(p.gather + gidx);
            if (t >= 0) v = to_c(in[ci.in_base + t], T());
        }
        if (p.conj_in) v = cconj(v);
        if (p.Ns > 1 && ci.k != 0 && n != 0) {
            const uint32_t e = (uint32_t)((uint64_t)n * (uint64_t)ci.k * (uint64_t)p.Lr);
            v = cmul(v, tw_two_level(p, e, T()));
        }
        return v;
    }

    // element n of column c from shared memory after the forward FFT: * spectrum, conjugate
    __device__ __forceinline__ T2 load_mid(int c, int n, const T2* src) const {
        const ColInfo<T>& ci = col[c];
        T2 v = src[saddr(c, n)];
        if (!ci.valid) return v;
        const int64_t gidx = (int64_t)ci.jj + (int64_t)n * p.Rr;
        if (p.dc_capture && gidx == 0) {
            // Rader: the DC term of the forward convolution FFT is sum_{n>=1} x[n]
            reinterpret_cast<T2*>(p.dcbuf)[ci.b] = v;
        }
        v = cmul(v, __ldg(reinterpret_cast<const T2*>(p.spectrum) + gidx));
        return cconj(v);
    }

    __device__ __forceinline__ void store(int c, int n, T2 v) const {
        const ColInfo<T>& ci = col[c];
        if (!ci.valid) return;
        const int64_t oidx = (int64_t)ci.out_j + (int64_t)n * p.Ns_out;
        OUT2* out = reinterpret_cast<OUT2*>(p.out);
        if (p.store_mode == ST_PLAIN) {
            if (p.conj_out) v = cconj(v);
            v = cscale(v, (T)p.scale);
            out[ci.out_base + oidx] = to_c(v, TO());
        } else if (p.store_mode == ST_CHIRP) {
            if (oidx < p.nvalid) {
                v = cscale(cmul(__ldg(reinterpret_cast<const T2*>(p.chirp) + oidx), v), (T)p.scale);
                if (p.conj_out) v = cconj(v);
                out[ci.out_base + oidx] = to_c(v, TO());
            }
        } else {
            const T s2 = (T)p.scale2;
            if (oidx == 0) {
                // DC: (x0 + A0) forward, (x0 + conj(A0)) inverse; A0 saved by the mid pass
                T2 a0 = reinterpret_cast<const T2*>(p.dcbuf)[ci.b];
                if (!p.conj_out) a0 = cconj(a0);
                out[ci.out_base] = to_c(cscale(cadd(ci.x0, a0), s2), TO());
            }
            const int t = __ldg(p.scatter + oidx);
            if (t > 0) {
                v = cscale(v, (T)p.scale);
                if (p.conj_out) v = cconj(v);
                out[ci.out_base + t] = to_c(cscale(cadd(ci.x0, v), s2), TO());
            }
        }
    }
};

}  // namespace fyg
