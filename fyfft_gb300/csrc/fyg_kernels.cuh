// fyg_kernels.cuh -- the tile-pass kernel template (see fyg_pass.cuh for the pass algebra).
//
// One CTA runs one tile: C columns x R points, held in shared memory:
//   load phase   global -> shared with the load fusions (conjugation, inter-pass twiddle,
//                Bluestein chirp and zero padding, Rader gather); batches of UNR loads per
//                thread are issued before any is consumed
//   stages       radix-r Stockham stages ping-ponging between two shared buffers, one butterfly
//                per loop iteration with its operands in registers; codelets up to radix 32
//                (composites stay in registers)
//   mid phase    (Rader/Bluestein) spectrum multiply + conjugation in place, then the stages
//                again (the first pass of the inverse transform)
//   store phase  shared -> global with the store fusions (scaling, conjugation, Bluestein chirp
//                and truncation, Rader scatter)
// The common plain load/store paths are specialized: a thread of an element-major tile always
// serves the same column (addresses and twiddle exponents advance by a constant), and a
// column-major tile of back-to-back transforms is one flat contiguous copy.  Chirp, gather and
// scatter take a general per-element path.
//
// Layouts (compile-time): element-major tiles (C consecutive columns of a multi-pass step, C a
// power of two) keep element (c, n) at n*(C+1) + c; column-major tiles (whole transforms,
// single-pass) at c*Rp + n + n/16.  The padding keeps strided shared accesses within two-way
// bank conflicts.
#pragma once
#include "fyg_pass.cuh"

namespace fyg {

// Radix classes: a kernel variant compiles the stages of one class, so its register budget is
// set by the class's largest codelet rather than by the largest codelet of the library.
#define FYG_RADICES_C16(X) X(2) X(3) X(4) X(5) X(7) X(8) X(9) X(11) X(13) X(16) X(12)
#define FYG_RADICES_C32_ONLY(X) X(20) X(24) X(25) X(27) X(32)

constexpr int LD_PLAIN_TW = 3;   // LD_PLAIN with the inter-pass twiddle (passes after the first)

template <bool COLMAJOR> struct Lay {
    int C, lc, pitch;
    __device__ __forceinline__ int at(int c, int n) const {
        if constexpr (COLMAJOR) return c * pitch + n + (n >> 4);
        else return n * pitch + c;
    }
};

// Radix-RADIX Stockham stage from one shared buffer into the other: one butterfly per loop
// iteration (operands in registers), so register use depends only on the radix.
template <typename T, int RADIX, bool COLMAJOR>
__device__ __forceinline__ void stage_pp(const cplx<T>* src, cplx<T>* dst, const Lay<COLMAJOR> L, int R,
                                         FastDiv nsd, FastDiv rrd, int twm, const cplx<T>* twl,
                                         const cplx<T>* twst) {
    using T2 = cplx<T>;
    const int Rr_l = R / RADIX;
    const int total = Rr_l * L.C;
    const int ns = (int)nsd.d;
#pragma unroll 1
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int c, j;
        if constexpr (COLMAJOR) { c = (int)rrd.div((uint32_t)idx); j = idx - c * Rr_l; }
        else { c = idx & (L.C - 1); j = idx >> L.lc; }
        T2 v[RADIX];
        if constexpr (COLMAJOR) {
#pragma unroll
            for (int m = 0; m < RADIX; ++m) v[m] = src[L.at(c, j + m * Rr_l)];
        } else {
            const T2* s0 = src + j * L.pitch + c;
            const int st = Rr_l * L.pitch;
#pragma unroll
            for (int m = 0; m < RADIX; ++m) v[m] = s0[m * st];
        }
        const int q = (int)nsd.div((uint32_t)j);
        const int k = j - q * ns;
        if (k) {
            if (twst) {
                // the stage's block of the stage-twiddle table: w_R^(m k twm) at m ns + k, so
                // that threads with consecutive k (consecutive butterflies) read consecutive
                // entries
                const cplx<T>* tw = twst + k;
#pragma unroll
                for (int m = 1; m < RADIX; ++m) v[m] = cmul(v[m], __ldg(tw + m * ns));
            } else {
                const int t = k * twm;
#pragma unroll
                for (int m = 1; m < RADIX; ++m) v[m] = cmul(v[m], __ldg(twl + m * t));
            }
        }
        dft<RADIX, T>(v);
        const int base = q * ns * RADIX + k;
        if constexpr (COLMAJOR) {
#pragma unroll
            for (int m = 0; m < RADIX; ++m) dst[L.at(c, base + m * ns)] = v[m];
        } else {
            T2* d0 = dst + base * L.pitch + c;
            const int st = ns * L.pitch;
#pragma unroll
            for (int m = 0; m < RADIX; ++m) d0[m * st] = v[m];
        }
    }
    __syncthreads();
}

// Runs the in-CTA schedule starting in bufs[w]; returns the index of the buffer holding the result.
template <typename T, int CLASS, bool COLMAJOR>
__device__ __forceinline__ int run_stages(const PassParams& p, const StageDesc* sd, cplx<T>* const* bufs, int w,
                                          const Lay<COLMAJOR> L) {
    const cplx<T>* twl = reinterpret_cast<const cplx<T>*>(p.tw_local);
    const cplx<T>* twst = reinterpret_cast<const cplx<T>*>(p.tw_stage);
    const int nst = p.g.nst, R = p.g.R;
    for (int s = 0; s < nst; ++s) {
        const StageDesc d = sd[s];
        const cplx<T>* tws = twst ? twst + d.twoff : nullptr;
        const cplx<T>* src = bufs[w];
        cplx<T>* dst = bufs[w ^ 1];
        switch (d.radix) {
#define FYG_CASE(r) case r: stage_pp<T, r, COLMAJOR>(src, dst, L, R, d.ns, d.rr, d.twm, twl, tws); break;
            FYG_RADICES_C16(FYG_CASE)
#undef FYG_CASE
#define FYG_CASE(r) \
    case r: if constexpr (CLASS >= 32) stage_pp<T, r, COLMAJOR>(src, dst, L, R, d.ns, d.rr, d.twm, twl, tws); break;
            FYG_RADICES_C32_ONLY(FYG_CASE)
#undef FYG_CASE
            default:
                if (threadIdx.x == 0 && p.err) atomicOr(p.err, 1);
                break;
        }
        w ^= 1;
    }
    return w;
}

// Column state of column c of a column-major tile (whole transforms, Rr == 1).
template <typename T>
__device__ __forceinline__ Col<T> colmajor_col(const PassParams& p, int64_t q) {
    Col<T> ci;
    ci.valid = q < p.ncols;
    ci.b = (int)q;
    ci.jj = 0;
    ci.k = 0;
    ci.out_j = 0;
    ci.in_base = ci.valid ? transform_base(p.in_offsets, p.ids, q, p.idist) : 0;
    ci.out_base = ci.valid ? out_transform_base(p, q) : 0;
    ci.x0 = mk<cplx<T>>(T(0), T(0));
    return ci;
}

// ------------------------------------------------------------------------------------------
// Load phase, general path: every load fusion, per-element column lookup.
// ------------------------------------------------------------------------------------------
template <typename T, typename TI, int MODE, int UNR, bool COLMAJOR>
__device__ __forceinline__ void load_general(const PassParams& p, cplx<T>* buf, const Lay<COLMAJOR> L, int64_t q0,
                                             const Col<T>& mc) {
    using T2 = cplx<T>;
    using IN2 = cplx<TI>;
    const IN2* gin = reinterpret_cast<const IN2*>(p.in);
    const int R = p.g.R, E = R * L.C, nthr = blockDim.x, Rr = p.Rr;
    const int conj_in = p.conj_in;
    const uint32_t Lr = (uint32_t)p.Lr;
    const int64_t nvalid = p.nvalid;
    const T2* chirp = reinterpret_cast<const T2*>(p.chirp);
    const int* gather = p.gather;
    const void* twhi = p.tw_hi;
    const void* twlo = p.tw_lo;
    const int tws = p.tw_shift;
    const FastDiv divR = p.g.divR;
    for (int e0 = threadIdx.x; e0 < E; e0 += nthr * UNR) {
        T2 u[UNR];
        int sa[UNR];
#pragma unroll
        for (int i = 0; i < UNR; ++i) {
            const int e = e0 + i * nthr;
            T2 v = mk<T2>(T(0), T(0));
            sa[i] = -1;
            if (e < E) {
                int c, n;
                Col<T> ci;
                if constexpr (COLMAJOR) {
                    c = (int)divR.div((uint32_t)e);
                    n = e - c * R;
                    ci = colmajor_col<T>(p, q0 + c);
                } else {
                    c = e & (L.C - 1);
                    n = e >> L.lc;
                    ci = mc;
                }
                sa[i] = L.at(c, n);
                if (ci.valid) {
                    const int gidx = ci.jj + n * Rr;
                    if constexpr (MODE == LD_PLAIN || MODE == LD_PLAIN_TW) {
                        v = to_c(ld_data(gin + ci.in_base + gidx), T());
                        if (conj_in) v = cconj(v);
                        if constexpr (MODE == LD_PLAIN_TW) {
                            if (ci.k != 0 && n != 0)
                                v = cmul(v, tw_two_level(twhi, twlo, tws, (uint32_t)(n * ci.k) * Lr, T()));
                        }
                    } else if constexpr (MODE == LD_CHIRP) {
                        if (gidx < nvalid) {
                            v = to_c(ld_data(gin + ci.in_base + gidx), T());
                            if (conj_in) v = cconj(v);
                            v = cmul(v, cconj(__ldg(chirp + gidx)));
                        }
                    } else {
                        const int t = __ldg(gather + gidx);
                        if (t >= 0) {
                            v = to_c(ld_data(gin + ci.in_base + t), T());
                            if (conj_in) v = cconj(v);
                        }
                    }
                }
            }
            u[i] = v;
        }
#pragma unroll
        for (int i = 0; i < UNR; ++i)
            if (sa[i] >= 0) buf[sa[i]] = u[i];
    }
}

// Load phase, element-major plain path: this thread serves column tid % C, rows g, g+G, ...
template <typename T, typename TI, bool TW, int UNR>
__device__ __forceinline__ void load_elem_plain(const PassParams& p, cplx<T>* buf, const Lay<false> L,
                                                const Col<T>& mc) {
    using T2 = cplx<T>;
    using IN2 = cplx<TI>;
    const int R = p.g.R;
    const int G = blockDim.x >> L.lc;           // threads per column
    const int g = threadIdx.x >> L.lc;
    const int c = threadIdx.x & (L.C - 1);
    const T isign = p.conj_in ? T(-1) : T(1);
    const IN2* src = reinterpret_cast<const IN2*>(p.in) + mc.in_base + mc.jj;
    const int64_t Rr = p.Rr;
    const uint32_t kL = (uint32_t)mc.k * (uint32_t)p.Lr;
    for (int n0 = g; n0 < R; n0 += G * UNR) {
        T2 u[UNR];
#pragma unroll
        for (int i = 0; i < UNR; ++i) {
            const int n = n0 + i * G;
            u[i] = mk<T2>(T(0), T(0));
            if (n < R && mc.valid) u[i] = to_c(ld_data(src + (int64_t)n * Rr), T());
        }
#pragma unroll
        for (int i = 0; i < UNR; ++i) {
            const int n = n0 + i * G;
            if (n < R) {
                T2 v = u[i];
                v.y *= isign;
                if constexpr (TW) {
                    const uint32_t e = (uint32_t)n * kL;
                    if (e) v = cmul(v, tw_two_level(p.tw_hi, p.tw_lo, p.tw_shift, e, T()));
                }
                buf[n * L.pitch + c] = v;
            }
        }
    }
}

// Load phase, column-major plain path over back-to-back transforms: a flat contiguous copy.
template <typename T, typename TI, int UNR>
__device__ __forceinline__ void load_flat_plain(const PassParams& p, cplx<T>* buf, const Lay<true> L, int64_t q0) {
    using T2 = cplx<T>;
    using IN2 = cplx<TI>;
    const int R = p.g.R, E = R * L.C, nthr = blockDim.x;
    const int64_t left = (p.ncols - q0) * (int64_t)R;
    const int Ev = left < E ? (int)left : E;
    const IN2* src = reinterpret_cast<const IN2*>(p.in) + q0 * (int64_t)R;
    const T isign = p.conj_in ? T(-1) : T(1);
    const FastDiv divR = p.g.divR;
    for (int e0 = threadIdx.x; e0 < E; e0 += nthr * UNR) {
        T2 u[UNR];
#pragma unroll
        for (int i = 0; i < UNR; ++i) {
            const int e = e0 + i * nthr;
            u[i] = mk<T2>(T(0), T(0));
            if (e < Ev) u[i] = to_c(ld_data(src + e), T());
        }
#pragma unroll
        for (int i = 0; i < UNR; ++i) {
            const int e = e0 + i * nthr;
            if (e < E) {
                const int c = (int)divR.div((uint32_t)e);
                T2 v = u[i];
                v.y *= isign;
                buf[L.at(c, e - c * R)] = v;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// Store phase
// ------------------------------------------------------------------------------------------
template <typename T, typename TO, bool COLMAJOR>
__device__ __forceinline__ void store_general(const PassParams& p, const cplx<T>* buf, const Lay<COLMAJOR> L,
                                              const ColHead<T>* head) {
    using T2 = cplx<T>;
    using OUT2 = cplx<TO>;
    OUT2* gout = reinterpret_cast<OUT2*>(p.out);
    const int R = p.g.R, E = R * L.C, nthr = blockDim.x;
    const int Ns_out = p.Ns_out;
    const int store_mode = p.store_mode, conj_out = p.conj_out;
    const T scale = (T)p.scale, scale2 = (T)p.scale2;
    const int64_t nvalid = p.nvalid;
    const T2* chirp = reinterpret_cast<const T2*>(p.chirp);
    const int* scatter = p.scatter;
    const T2* dcbuf = reinterpret_cast<const T2*>(p.dcbuf);
    const int64_t ostride = p.split_m > 1 ? p.split_m : 1;
    const bool nfast = COLMAJOR || Ns_out == 1;
    const FastDiv divR = p.g.divR;
#pragma unroll 4
    for (int e = threadIdx.x; e < E; e += nthr) {
        int c, n;
        if (nfast) { c = (int)divR.div((uint32_t)e); n = e - c * R; }
        else { c = e & (L.C - 1); n = e >> L.lc; }
        const ColHead<T> h = head[c];
        if (!h.valid) continue;
        T2 u = buf[L.at(c, n)];
        const int oidx = h.out_j + n * Ns_out;
        if (store_mode == ST_PLAIN) {
            if (conj_out) u = cconj(u);
            gout[h.out_base + oidx] = to_c(cscale(u, scale), TO());
        } else if (store_mode == ST_CHIRP) {
            if (oidx < nvalid) {
                u = cscale(cmul(__ldg(chirp + oidx), u), scale);
                if (conj_out) u = cconj(u);
                gout[h.out_base + oidx] = to_c(u, TO());
            }
        } else {
            if (oidx == 0) {
                // Rader DC: (x0 + A0) forward, (x0 + conj(A0)) inverse
                T2 a0 = dcbuf[h.b];
                if (!conj_out) a0 = cconj(a0);
                gout[h.out_base] = to_c(cscale(cadd(h.x0, a0), scale2), TO());
            }
            const int t = __ldg(scatter + oidx);
            if (t > 0) {
                u = cscale(u, scale);
                if (conj_out) u = cconj(u);
                gout[h.out_base + t * ostride] = to_c(cscale(cadd(h.x0, u), scale2), TO());
            }
        }
    }
}

// Element-major plain store.  Strided outputs (Ns_out > 1): this thread serves column tid % C.
// Contiguous outputs (Ns_out == 1): threads form C groups, group c writes column c's R outputs.
template <typename T, typename TI, typename TO>
__device__ __forceinline__ void store_elem_plain(const PassParams& p, const cplx<T>* buf, const Lay<false> L,
                                                 int64_t q0) {
    using T2 = cplx<T>;
    using OUT2 = cplx<TO>;
    const int R = p.g.R;
    const T sx = (T)p.scale, sy = p.conj_out ? -(T)p.scale : (T)p.scale;
    const int G = blockDim.x >> L.lc;
    if (p.Ns_out > 1) {
        const int g = threadIdx.x >> L.lc;
        const int c = threadIdx.x & (L.C - 1);
        const Col<T> ci = make_col<T, TI>(p, q0 + c);
        if (!ci.valid) return;
        OUT2* dst = reinterpret_cast<OUT2*>(p.out) + ci.out_base + ci.out_j;
        const int64_t ns = p.Ns_out;
#pragma unroll 4
        for (int n = g; n < R; n += G) {
            const T2 u = buf[n * L.pitch + c];
            dst[n * ns] = to_c(mk<T2>(u.x * sx, u.y * sy), TO());
        }
    } else {
        const int c = threadIdx.x / G;
        const int g = threadIdx.x - c * G;
        const Col<T> ci = make_col<T, TI>(p, q0 + c);
        if (!ci.valid) return;
        OUT2* dst = reinterpret_cast<OUT2*>(p.out) + ci.out_base + ci.out_j;
#pragma unroll 4
        for (int n = g; n < R; n += G) {
            const T2 u = buf[n * L.pitch + c];
            dst[n] = to_c(mk<T2>(u.x * sx, u.y * sy), TO());
        }
    }
}

// Column-major plain store over back-to-back transforms: a flat contiguous copy.
template <typename T, typename TO>
__device__ __forceinline__ void store_flat_plain(const PassParams& p, const cplx<T>* buf, const Lay<true> L,
                                                 int64_t q0) {
    using T2 = cplx<T>;
    using OUT2 = cplx<TO>;
    const int R = p.g.R, E = R * L.C, nthr = blockDim.x;
    const int64_t left = (p.ncols - q0) * (int64_t)R;
    const int Ev = left < E ? (int)left : E;
    OUT2* dst = reinterpret_cast<OUT2*>(p.out) + q0 * (int64_t)R;
    const T sx = (T)p.scale, sy = p.conj_out ? -(T)p.scale : (T)p.scale;
    const FastDiv divR = p.g.divR;
#pragma unroll 4
    for (int e = threadIdx.x; e < Ev; e += nthr) {
        const int c = (int)divR.div((uint32_t)e);
        const T2 u = buf[L.at(c, e - c * R)];
        dst[e] = to_c(mk<T2>(u.x * sx, u.y * sy), TO());
    }
}

// ------------------------------------------------------------------------------------------
// The kernel
// ------------------------------------------------------------------------------------------
// One tile (tile index `tile` of the pass described by p) with the CTA's threads.
template <typename T, typename TI, typename TO, int CLASS, bool COLMAJOR>
__device__ __forceinline__ void tile_body(const PassParams& p, int64_t tile, unsigned char* smraw) {
    using T2 = cplx<T>;
    using IN2 = cplx<TI>;
    const int R = p.g.R, C = p.g.C;
    StageDesc* sd = reinterpret_cast<StageDesc*>(smraw);
    ColHead<T>* head = reinterpret_cast<ColHead<T>*>(smraw + kMaxStages * sizeof(StageDesc));
    T2* bufs[2];
    bufs[0] = reinterpret_cast<T2*>(smraw + tile_head_bytes<T>(C));
    bufs[1] = bufs[0] + tile_elems(R, C, COLMAJOR);
    Lay<COLMAJOR> L;
    L.C = C;
    L.lc = p.g.log2C;
    L.pitch = COLMAJOR ? colmajor_pitch(R) : C + 1;
    const int64_t q0 = tile * C;
    const IN2* gin = reinterpret_cast<const IN2*>(p.in);
    const int E = R * C;
    const int nthr = blockDim.x;
    constexpr int UNR = sizeof(T) == 4 ? 16 : 8;
    const bool plain_in = p.load_mode == LD_PLAIN;
    const bool plain_out = p.store_mode == ST_PLAIN;
    const bool flat_in = COLMAJOR && plain_in && p.idist == R && !p.in_offsets;
    const bool flat_out = COLMAJOR && plain_out && p.odist == R && !p.out_offsets;

    // ---- stage schedule; per-column head for the general paths (output base, validity, x0) ----
    if (threadIdx.x < kMaxStages) {
        const int s = threadIdx.x;
        StageDesc d;
        // unrolled selects keep the parameter reads at constant offsets
#pragma unroll
        for (int t = 0; t < kMaxStages; ++t)
            if (t == s) {
                d.radix = p.g.radix[t];
                d.twm = p.g.twmul[t];
                d.twoff = p.g.twoff[t];
                d.ns = p.g.ns[t];
                d.rr = p.g.rr[t];
            }
        sd[s] = d;
    }
    const bool need_head = !(plain_out && (flat_out || !COLMAJOR)) || p.x0_from_in;
    if (need_head) {
        for (int c = threadIdx.x; c < C; c += nthr) {
            const Col<T> ci = COLMAJOR ? colmajor_col<T>(p, q0 + c) : make_col<T, TI>(p, q0 + c);
            T2 x0 = mk<T2>(T(0), T(0));
            if (ci.valid && (p.store_mode == ST_SCATTER || (p.x0_from_in && p.x0buf))) {
                x0 = p.x0_from_in ? to_c(ld_data(gin + ci.in_base), T())
                                 : ld_data(reinterpret_cast<const T2*>(p.x0buf) + ci.b);
                if (p.x0_from_in && p.x0buf && ci.jj == 0) reinterpret_cast<T2*>(p.x0buf)[ci.b] = x0;
            }
            ColHead<T> h;
            h.out_base = ci.out_base;
            h.out_j = ci.out_j;
            h.b = ci.b;
            h.valid = ci.valid;
            h.pad = 0;
            h.x0 = x0;
            head[c] = h;
        }
    }

    // ---- load phase ----
    T2* buf = bufs[0];
    {
        Col<T> mc;
        if constexpr (!COLMAJOR) mc = make_col<T, TI>(p, q0 + (threadIdx.x & (C - 1)));
        if constexpr (COLMAJOR) {
            if (flat_in) load_flat_plain<T, TI, UNR>(p, buf, L, q0);
            else if (p.load_mode == LD_CHIRP) load_general<T, TI, LD_CHIRP, UNR, true>(p, buf, L, q0, mc);
            else if (p.load_mode == LD_GATHER) load_general<T, TI, LD_GATHER, UNR, true>(p, buf, L, q0, mc);
            else load_general<T, TI, LD_PLAIN, UNR, true>(p, buf, L, q0, mc);
        } else {
            if (p.load_mode == LD_CHIRP) load_general<T, TI, LD_CHIRP, UNR, false>(p, buf, L, q0, mc);
            else if (p.load_mode == LD_GATHER) load_general<T, TI, LD_GATHER, UNR, false>(p, buf, L, q0, mc);
            else if (p.Ns > 1) load_elem_plain<T, TI, true, UNR>(p, buf, L, mc);
            else load_elem_plain<T, TI, false, UNR>(p, buf, L, mc);
        }
    }
    __syncthreads();

    int w = run_stages<T, CLASS, COLMAJOR>(p, sd, bufs, 0, L);
    buf = bufs[w];

    if (p.mid) {
        // spectrum multiply + conjugation (the inverse is computed as conj(F(conj(.)))); the
        // forward output is in natural order: element n of column c is global index jj + n Rr
        const T2* spec = reinterpret_cast<const T2*>(p.spectrum);
        T2* dcbuf = reinterpret_cast<T2*>(p.dcbuf);
        const FastDiv divR = p.g.divR;
        Col<T> mc;
        if constexpr (!COLMAJOR) mc = make_col<T, TI>(p, q0 + (threadIdx.x & (C - 1)));
        for (int e = threadIdx.x; e < E; e += nthr) {
            int c, n;
            Col<T> ci;
            if constexpr (COLMAJOR) {
                c = (int)divR.div((uint32_t)e);
                n = e - c * R;
                ci = colmajor_col<T>(p, q0 + c);
            } else {
                c = e & (C - 1);
                n = e >> L.lc;
                ci = mc;
            }
            const int sa = L.at(c, n);
            T2 u = buf[sa];
            if (ci.valid) {
                const int gidx = ci.jj + n * p.Rr;
                if (p.dc_capture && gidx == 0) dcbuf[ci.b] = u;
                u = cconj(cmul(u, __ldg(spec + gidx)));
            }
            buf[sa] = u;
        }
        __syncthreads();
        w = run_stages<T, CLASS, COLMAJOR>(p, sd, bufs, w, L);
        buf = bufs[w];
    }

    // ---- store phase ----
    if constexpr (COLMAJOR) {
        if (flat_out) store_flat_plain<T, TO>(p, buf, L, q0);
        else store_general<T, TO, true>(p, buf, L, head);
    } else {
        if (plain_out) store_elem_plain<T, TI, TO>(p, buf, L, q0);
        else store_general<T, TO, false>(p, buf, L, head);
    }
}

// TAG only distinguishes instantiations made by different translation units.
template <typename T, typename TI, typename TO, int CLASS, bool COLMAJOR, int TAG = 0>
__global__ void __launch_bounds__(kMaxThreads) k_pass(const __grid_constant__ PassParams p) {
    extern __shared__ __align__(16) unsigned char smraw[];
    tile_body<T, TI, TO, CLASS, COLMAJOR>(p, (int64_t)blockIdx.x, smraw);
}

}  // namespace fyg
