// fyg_kernels.cuh -- the tile-pass kernel template (see fyg_pass.cuh for the pass algebra).
//
// One CTA runs one tile: C columns x R points.  Every in-CTA stage processes all R*C/r radix-r
// butterflies of the tile; a thread owns at most ceil(EPT/r) of them and keeps their operands
// in registers, so a stage is: read operands (global or shared memory) -> local twiddle ->
// codelet -> __syncthreads -> write results (shared or global memory).
#pragma once
#include "fyg_pass.cuh"

namespace fyg {

enum SrcKind { SRC_GLOBAL = 0, SRC_SMEM = 1, SRC_MID = 2 };
enum DstKind { DST_SMEM = 0, DST_GLOBAL = 1 };

template <typename T, typename TI, typename TO, int RADIX, int SRC, int DST>
__device__ __noinline__ void stage(const PassCtx<T, TI, TO> X, int s, const cplx<T>* src, cplx<T>* dst) {
    using T2 = cplx<T>;
    const TileGeom& g = X.p.g;
    const int Rr = g.R / RADIX;
    const int total = Rr * g.C;
    const FastDiv nsd = g.ns[s];
    const FastDiv rrd = g.rr[s];
    const int ns = (int)nsd.d;
    const T2* twl = reinterpret_cast<const T2*>(X.p.tw_local);
    const int twm = g.twmul[s];
    const bool colmajor = g.colmajor != 0;
    const int cmask = g.C - 1, lc = g.log2C;
#pragma unroll 1
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int c, j;
        if (colmajor) { c = (int)rrd.div((uint32_t)idx); j = idx - c * Rr; }
        else { c = idx & cmask; j = idx >> lc; }
        T2 v[RADIX];
#pragma unroll
        for (int m = 0; m < RADIX; ++m) {
            const int n = j + m * Rr;
            if constexpr (SRC == SRC_GLOBAL) v[m] = X.load(c, n);
            else if constexpr (SRC == SRC_SMEM) v[m] = src[X.saddr(c, n)];
            else v[m] = X.load_mid(c, n, src);
        }
        const int q = (int)nsd.div((uint32_t)j);
        const int k = j - q * ns;
        if (k) {
#pragma unroll
            for (int m = 1; m < RADIX; ++m) v[m] = cmul(v[m], __ldg(twl + m * k * twm));
        }
        dft<RADIX, T>(v);
        const int base = q * ns * RADIX + k;
#pragma unroll
        for (int m = 0; m < RADIX; ++m) {
            const int n = base + m * ns;
            if constexpr (DST == DST_SMEM) dst[X.saddr(c, n)] = v[m];
            else X.store(c, n, v[m]);
        }
    }
    if constexpr (DST == DST_SMEM) __syncthreads();
}

template <typename T, typename TI, typename TO, int SRC, int DST>
__device__ __forceinline__ void dispatch_stage(const PassCtx<T, TI, TO>& X, int s, const cplx<T>* src,
                                               cplx<T>* dst) {
    switch (X.p.g.radix[s]) {
        case 2: stage<T, TI, TO, 2, SRC, DST>(X, s, src, dst); break;
        case 3: stage<T, TI, TO, 3, SRC, DST>(X, s, src, dst); break;
        case 4: stage<T, TI, TO, 4, SRC, DST>(X, s, src, dst); break;
        case 5: stage<T, TI, TO, 5, SRC, DST>(X, s, src, dst); break;
        case 7: stage<T, TI, TO, 7, SRC, DST>(X, s, src, dst); break;
        case 8: stage<T, TI, TO, 8, SRC, DST>(X, s, src, dst); break;
        case 9: stage<T, TI, TO, 9, SRC, DST>(X, s, src, dst); break;
        case 11: stage<T, TI, TO, 11, SRC, DST>(X, s, src, dst); break;
        case 13: stage<T, TI, TO, 13, SRC, DST>(X, s, src, dst); break;
        case 16: stage<T, TI, TO, 16, SRC, DST>(X, s, src, dst); break;
        default:
            if (threadIdx.x == 0 && X.p.err) atomicOr(X.p.err, 1);
            break;
    }
}

// One in-CTA FFT over the tile.  Stages ping-pong between the two shared buffers bufs[0/1];
// `src` is the buffer SRC_MID reads from.  Returns the buffer the last stage wrote when
// DST == DST_SMEM.
template <typename T, typename TI, typename TO, int SRC, int DST>
__device__ __forceinline__ cplx<T>* run_fft(const PassCtx<T, TI, TO>& X, cplx<T>* const* bufs,
                                            const cplx<T>* src) {
    const int nst = X.p.g.nst;
    int w = (src == bufs[0]) ? 1 : 0;  // first buffer written
    if (nst == 1) {
        dispatch_stage<T, TI, TO, SRC, DST>(X, 0, src, bufs[w]);
        return bufs[w];
    }
    dispatch_stage<T, TI, TO, SRC, DST_SMEM>(X, 0, src, bufs[w]);
    for (int s = 1; s < nst - 1; ++s) {
        dispatch_stage<T, TI, TO, SRC_SMEM, DST_SMEM>(X, s, bufs[w], bufs[w ^ 1]);
        w ^= 1;
    }
    dispatch_stage<T, TI, TO, SRC_SMEM, DST>(X, nst - 1, bufs[w], bufs[w ^ 1]);
    return bufs[w ^ 1];
}

// Per-column setup shared by every tile kernel: (transform b, column jj) of each of the C
// columns, their global bases, the inter-pass twiddle index k and the Rader x0 term.
template <typename T, typename TI>
__device__ __forceinline__ void setup_columns(const PassParams& p, ColInfo<T>* col, int64_t q0) {
    using T2 = cplx<T>;
    for (int c = threadIdx.x; c < p.g.C; c += blockDim.x) {
        ColInfo<T> ci;
        const int64_t q = q0 + c;
        ci.valid = q < p.ncols;
        const uint32_t qq = (uint32_t)(ci.valid ? q : 0);
        const uint32_t b = p.div_Rr.div(qq);
        const uint32_t jj = qq - b * (uint32_t)p.Rr;
        ci.b = (int)b;
        ci.jj = (int)jj;
        const uint32_t qn = p.div_Ns.div(jj);
        ci.k = (int)(jj - qn * (uint32_t)p.Ns);
        const uint32_t qo = p.div_Ns_out.div(jj);
        ci.out_j = (int)(qo * (uint32_t)p.Ns_out * (uint32_t)p.g.R + (jj - qo * (uint32_t)p.Ns_out));
        ci.in_base = (int64_t)b * p.idist;
        ci.out_base = (int64_t)b * p.odist;
        ci.pad = 0;
        ci.x0 = mk<T2>(T(0), T(0));
        if (p.store_mode == ST_SCATTER && ci.valid) {
            if (p.x0_from_in) {
                ci.x0 = to_c(reinterpret_cast<const cplx<TI>*>(p.in)[ci.in_base], T());
                if (jj == 0 && p.x0buf) reinterpret_cast<T2*>(p.x0buf)[b] = ci.x0;
            } else if (p.x0buf) {
                ci.x0 = reinterpret_cast<const T2*>(p.x0buf)[b];
            }
        } else if (p.x0_from_in && p.x0buf && ci.valid && jj == 0) {
            reinterpret_cast<T2*>(p.x0buf)[b] =
                to_c(reinterpret_cast<const cplx<TI>*>(p.in)[ci.in_base], T());
        }
        col[c] = ci;
    }
}

template <typename T, typename TI, typename TO, int MAXT>
__global__ void __launch_bounds__(MAXT) k_pass(const __grid_constant__ PassParams p) {
    extern __shared__ __align__(16) unsigned char smraw[];
    using T2 = cplx<T>;
    ColInfo<T>* col = reinterpret_cast<ColInfo<T>*>(smraw);
    const size_t ci = ((size_t)p.g.C * sizeof(ColInfo<T>) + 15) & ~(size_t)15;
    T2* bufs[2] = {reinterpret_cast<T2*>(smraw + ci),
                   reinterpret_cast<T2*>(smraw + ci) + (size_t)p.g.R * p.g.C};
    setup_columns<T, TI>(p, col, (int64_t)blockIdx.x * p.g.C);
    __syncthreads();
    const PassCtx<T, TI, TO> X{p, bufs[0], col};
    if (!p.mid) {
        run_fft<T, TI, TO, SRC_GLOBAL, DST_GLOBAL>(X, bufs, bufs[1]);
    } else {
        T2* y = run_fft<T, TI, TO, SRC_GLOBAL, DST_SMEM>(X, bufs, bufs[1]);
        run_fft<T, TI, TO, SRC_MID, DST_GLOBAL>(X, bufs, y);
    }
}

}  // namespace fyg
