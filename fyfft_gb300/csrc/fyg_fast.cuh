// fyg_fast.cuh -- register-resident tile-pass kernels for power-of-two tile lengths (FP32).
//
// Same pass algebra as fyg_pass.cuh (one radix-R Stockham step of a length-L transform over C
// consecutive columns), with the in-CTA length-R DFT organised around registers instead of
// shared-memory sweeps:
//   * a column is served by G = R/P threads; thread g of column c owns the P points
//     n = g + G*i (i < P) and keeps them in registers for the whole pass;
//   * stage s (radix r = min(P, R/P^s), ns = P^s) is P/r butterflies per thread whose operands
//     are exactly those registers (j = g + G*b, inputs j + m*R/r = g + G*(b + m*P/r)), so the
//     global load feeds the first butterflies directly and the last stage leaves output point
//     n = g + G*i in register i (Stockham order is natural order at the end);
//   * between stages the outputs go through one shared buffer (column-major, padded so that
//     both the strided writes and the unit-stride reads are free of bank conflicts);
//   * the store is direct and coalesced across the tile's columns when the output stride
//     Ns_out > 1, and a flat copy through shared memory when Ns_out = 1 (the tile's columns are
//     then back to back in memory).
// Columns per tile C and points per thread P are chosen per R so that a CTA has 256 threads and
// two CTAs fit on an SM (<= 128 registers per thread, one shared buffer): one CTA's loads
// overlap the other's butterflies.
//
// Fusions: conjugation and the inter-pass twiddle (two-level table), the Bluestein chirp with
// zero padding or the Rader gather at the load; the fused mid pass of a convolution (spectrum
// multiply, conjugation, second in-CTA DFT = first inverse pass, Rader DC capture); scaling,
// conjugation, the Bluestein output chirp with truncation or the Rader scatter with the x0 and
// DC terms at the store.  Uneven batches use the generic kernel (fyg_kernels.cuh).
#pragma once
#include <cuda.h>   // CUtensorMap (an opaque, 64-byte aligned descriptor passed by value)

#include "fyg_pass.cuh"

namespace fyg {

// Shape of a fast tile: R points per column, P registers-points per thread (every stage radix
// divides P), C columns per tile, TWB: group size of the inter-pass twiddle factorization
// (fast_twiddle, used when no thread-order table was built).
template <int R_, int P_, int C_, int TWB_ = 4> struct FastShape {
    static constexpr int R = R_, P = P_, C = C_, TWB = TWB_;
    static_assert(P % TWB == 0, "twiddle groups must tile the registers");
    static constexpr int G = R / P;            // threads per column
    static constexpr int T = C * G;            // threads per CTA
    __host__ __device__ static constexpr int pad(int n) { return n >> 5; }
    // pitch of a column: >= R + R/32 and = 16/C (mod 16) (8-byte words; 1 for C >= 16), so
    // the columns met by a half-warp start in different banks
    static constexpr int Rp = ((R + (R >> 5) + 15) & ~15) + (C >= 16 ? 1 : 16 / C);
    __host__ __device__ static constexpr int nst() {
        int s = 0;
        for (int rem = R; rem > 1; rem /= (rem < P ? rem : P)) ++s;
        return s;
    }
    __host__ __device__ static constexpr int radix(int s) {
        int rem = R;
        for (int t = 0; t < s; ++t) rem /= (rem < P ? rem : P);
        return rem < P ? rem : P;
    }
    __host__ __device__ static constexpr int ns(int s) {
        int v = 1;
        for (int t = 0; t < s; ++t) v *= radix(t);
        return v;
    }
    // offset of stage s's block in the stage-twiddle table (blocks of radix(s) * ns(s) entries
    // for s = 1 .. nst-1)
    __host__ __device__ static constexpr int stage_off(int s) {
        int o = 0;
        for (int t = 1; t < s; ++t) o += radix(t) * ns(t);
        return o;
    }
    static constexpr size_t smem_bytes() { return (size_t)C * Rp * sizeof(float2); }
};

// The shapes in use: 256 threads per CTA (two CTAs per SM) up to R = 2048; 243 = 27 * 9 and
// 343 = 7 * 7 * 7 for powers of three and seven (C divides their column counts 3^k / 7^k).
// Wide shapes: 512 threads per CTA (one CTA per SM, the same 16 warps) with twice the columns,
// so that every row segment a tile reads or writes is 64-256 contiguous bytes instead of 32-128
// (FYG_FLAG_WIDE_TILES; the autotuner measures both).
using FastR256 = FastShape<256, 16, 16>;
using FastR512 = FastShape<512, 32, 16>;
using FastR1024 = FastShape<1024, 32, 8>;
using FastR2048 = FastShape<2048, 32, 4>;
using FastR4096 = FastShape<4096, 32, 4>;
using FastR243 = FastShape<243, 27, 27, 3>;
using FastR343 = FastShape<343, 7, 7, 7>;
using FastR256W = FastShape<256, 16, 32>;
using FastR512W = FastShape<512, 32, 32>;
using FastR1024W = FastShape<1024, 32, 16>;
using FastR2048W = FastShape<2048, 32, 8>;

template <class S> __device__ __forceinline__ int fast_addr(int c, int n) { return c * S::Rp + n + S::pad(n); }

// A thread's own points n = g + G i sit at own_base + own_off(i): the padding (g + G i) >> 5
// splits into a per-thread part and a compile-time part when G is a multiple or a divisor of 32
// (then g < G never carries into the padding); other shapes use fast_addr.
template <class S> struct Own {
    static constexpr bool linear = (S::G % 32 == 0) || (32 % S::G == 0);
    __device__ static __forceinline__ int base(int c, int g) {
        return c * S::Rp + g + ((S::G % 32 == 0) ? (g >> 5) : 0);
    }
    __host__ __device__ static constexpr int off(int i) {
        return S::G * i + ((S::G % 32 == 0) ? i * (S::G / 32) : ((S::G * i) >> 5));
    }
};

// One in-CTA Stockham stage over the thread's registers.  Non-final stages write their outputs
// to shared memory and read the next stage's operands back (two barriers: the buffer is shared
// by consecutive exchanges).
template <class S, int ST>
__device__ __forceinline__ void fast_stage(float2 (&v)[S::P], float2* sm, int c, int g, const float2* twl) {
    constexpr int r = S::radix(ST), ns = S::ns(ST), nb = S::P / r;
    constexpr bool last = ST == S::nst() - 1;
    // outputs base + m ns: linear in m (one per-thread address, compile-time offsets) when ns is
    // a multiple of 32, or ns == 1 with r dividing 32 (base = j r stays inside a 32-point block)
    constexpr bool wlin = (ns % 32 == 0) || (ns == 1 && 32 % r == 0);
    constexpr int wstride = ns % 32 == 0 ? ns + ns / 32 : 1;
#pragma unroll
    for (int b = 0; b < nb; ++b) {
        float2 x[r];
#pragma unroll
        for (int m = 0; m < r; ++m) x[m] = v[b + m * nb];
        const int j = g + S::G * b;
        const int k = j % ns;
        if constexpr (ST > 0) {
            // w_R^(m k twm) from this stage's block: lanes with consecutive k read consecutive
            // entries (entries with k = 0 are 1)
            const float2* tw = twl + S::stage_off(ST) + k;
#pragma unroll
            for (int m = 1; m < r; ++m) x[m] = cmul(x[m], __ldg(tw + m * ns));
        }
        dft<r, float>(x);
        if constexpr (last) {
#pragma unroll
            for (int m = 0; m < r; ++m) v[b + m * nb] = x[m];
        } else {
            const int base = (j - k) * r + k;   // (j / ns) * ns * r + k
            if constexpr (wlin) {
                float2* w = sm + fast_addr<S>(c, base);
#pragma unroll
                for (int m = 0; m < r; ++m) w[m * wstride] = x[m];
            } else {
#pragma unroll
                for (int m = 0; m < r; ++m) sm[fast_addr<S>(c, base + m * ns)] = x[m];
            }
        }
    }
    if constexpr (!last) {
        __syncthreads();
        if constexpr (Own<S>::linear) {
            const float2* rd = sm + Own<S>::base(c, g);
#pragma unroll
            for (int i = 0; i < S::P; ++i) v[i] = rd[Own<S>::off(i)];
        } else {
#pragma unroll
            for (int i = 0; i < S::P; ++i) v[i] = sm[fast_addr<S>(c, g + S::G * i)];
        }
        __syncthreads();
    }
}

template <class S, int ST>
__device__ __forceinline__ void fast_stages_from(float2 (&v)[S::P], float2* sm, int c, int g, const float2* twl) {
    if constexpr (ST < S::nst()) {
        fast_stage<S, ST>(v, sm, c, g, twl);
        fast_stages_from<S, ST + 1>(v, sm, c, g, twl);
    }
}

// L2 residency: the thread-order tables are read by every transform of a batch, the streamed
// data once; table reads carry an evict-last policy so the tables stay in L2 while the batch
// streams through it (measured: Bluestein 999983 -2.6%, 131074 -4%; evict-first data loads
// were slower and are not used).
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float2 ld_table(const float2* ptr, uint64_t pol) {
    float2 v;
    asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(ptr), "l"(pol));
    return v;
}

// Data load that reads memory only where `pred` holds and yields zero elsewhere: a predicated
// load in inline PTX, so that the zero padding of a Bluestein input issues no memory request
// (clamping the index to the last element made every padded load of a transform hit one L2
// line) while all of a thread's loads stay in flight together (no branch).
__device__ __forceinline__ float2 ld_data_if(const float2* ptr, bool pred) {
    float2 v;
    asm("{\n .reg .pred q;\n setp.ne.u32 q, %3, 0;\n mov.b32 %0, 0;\n mov.b32 %1, 0;\n"
        " @q ld.global.cg.v2.f32 {%0, %1}, [%2];\n}"
        : "=f"(v.x), "=f"(v.y)
        : "l"(ptr), "r"((unsigned)pred));
    return v;
}

// ---- TMA tile loads (cp.async.bulk.tensor) ----
// One thread arms an mbarrier with the tile's byte count and issues the 2D tensor loads of the
// C columns x R rows of the tile (boxes of 2C floats x 256 rows) into shared memory; every thread
// waits on the barrier's phase.  The wait is bounded (globaltimer, 2 s): on expiry the kernel
// records an error bit and carries on with whatever the buffer holds, so no thread leaves a
// barrier the others still reach.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t mb, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mb), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mb, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t mb) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mb)
        : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mb, uint32_t parity) {
    const uint64_t t0 = global_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n selp.u32 %0, 1, 0, q;\n}"
            : "=r"(done)
            : "r"(mb), "r"(parity)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > 2000000000ull) return false;
    }
}

// Load variants, compiled as separate kernels so that each gets its own register allocation.
enum FastLoad : int {
    FL_PLAIN = 0,     // x (conjugated for inverses): first passes
    FL_TWIDDLE = 1,   // x * w_L^(n k Lr): passes after the first
    FL_CHIRP = 2,     // Bluestein: x[n] conj(w[n]) for n < N, zero padding above
    FL_GATHER = 3     // Rader: x[gather[n]], zero where gather < 0; x[0] saved
};

// Inter-pass twiddles of the thread's points n_i = g + G i, i = B a + b:
// w^(n_i k Lr) = w^((g + G B a) k Lr) * w^(b G k Lr), i.e. P/B + B - 1 two-level lookups instead
// of P, and one extra complex product per point (about one more rounding).
template <int P, int G, int B>
__device__ __forceinline__ void fast_twiddle(float2 (&v)[P], const PassParams& p, int g, uint32_t kL) {
    float2 wb[B];
    wb[0] = make_float2(1.f, 0.f);
#pragma unroll
    for (int b = 1; b < B; ++b) wb[b] = tw_two_level(p.tw_hi, p.tw_lo, p.tw_shift, (uint32_t)(b * G) * kL, 0.f);
#pragma unroll
    for (int a = 0; a < P / B; ++a) {
        const uint32_t ea = (uint32_t)(g + G * B * a) * kL;
        const float2 wa = ea ? tw_two_level(p.tw_hi, p.tw_lo, p.tw_shift, ea, 0.f) : make_float2(1.f, 0.f);
#pragma unroll
        for (int b = 0; b < B; ++b) v[a * B + b] = cmul(v[a * B + b], b ? cmul(wa, wb[b]) : wa);
    }
}

// TMA: the data of a FL_PLAIN / FL_TWIDDLE load arrive by tensor copies (tmap describes the pass
// input as rows of 2 Rr floats, one row per point of a transform) instead of per-thread loads.
template <class S, int LD, bool MID, bool TMA = false>
__global__ void __launch_bounds__(S::T, (S::T <= 384 ? 2 : 1))
    k_fast(const __grid_constant__ PassParams p, const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ __align__(128) unsigned char smraw[];
    float2* sm = reinterpret_cast<float2*>(smraw);
    constexpr int P = S::P, G = S::G, C = S::C, R = S::R;
    const int c = threadIdx.x % C;
    const int g = threadIdx.x / C;
    // all C columns of a tile belong to one transform (Rr is a multiple of C)
    const unsigned tile = p.reverse_tiles ? gridDim.x - 1 - blockIdx.x : blockIdx.x;
    const Col<float> ci = make_col<float, float>(p, (int64_t)tile * C + c);
    const float2* twl = reinterpret_cast<const float2*>(p.tw_stage);
    const int Rr = p.Rr;
    const uint64_t keep = l2_keep_policy();

    // ---- load: register i <- x[jj + n Rr], n = g + G i ----
    float2 v[P];
    const float2* src = reinterpret_cast<const float2*>(p.in) + ci.in_base + ci.jj;
    if constexpr (LD == FL_CHIRP) {
        // predicated loads: the zero padding above N reads nothing; all loads of the thread are
        // in flight together (branching loads were measured to serialize)
        const float2* chirp = reinterpret_cast<const float2*>(p.chirp);
        const int nlast = (int)p.nvalid - 1;
        const float2* xb = reinterpret_cast<const float2*>(p.in) + ci.in_base;
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const int gidx = ci.jj + (g + G * i) * Rr;
            v[i] = ld_data_if(xb + gidx, gidx <= nlast);
        }
        const float isign = p.conj_in ? -1.f : 1.f;
        if (p.tab_tiled) {
            // conj(chirp) in thread order, zero above N (the padded data are zero already)
            const float2* tab = reinterpret_cast<const float2*>(p.tab_tiled) + (size_t)(ci.jj / C) * (P * S::T) + threadIdx.x;
#pragma unroll
            for (int i = 0; i < P; ++i) v[i] = cmul(make_float2(v[i].x, v[i].y * isign), ld_table(tab + i * S::T, keep));
        } else {
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int gidx = ci.jj + (g + G * i) * Rr;
                const float2 u = cmul(make_float2(v[i].x, v[i].y * isign), cconj(__ldg(chirp + min(gidx, nlast))));
                v[i] = gidx <= nlast ? u : make_float2(0.f, 0.f);
            }
        }
    } else if constexpr (LD == FL_GATHER) {
        const float2* base = reinterpret_cast<const float2*>(p.in) + ci.in_base;
        const int* gather = p.gather;
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const int t = __ldg(gather + ci.jj + (g + G * i) * Rr);
            v[i] = ld_data_if(base + t, t >= 0);
        }
        if (p.conj_in) {
#pragma unroll
            for (int i = 0; i < P; ++i) v[i].y = -v[i].y;
        }
        if (p.x0_from_in && p.x0buf && ci.jj == 0 && g == 0)
            reinterpret_cast<float2*>(p.x0buf)[ci.b] = ld_data(base);
    } else {
        if constexpr (TMA) {
            // the tile lands in the exchange buffer as [point][column] (C float2 per row), so
            // that thread (c, g) reads point g + G i at (g + G i) C + c: consecutive threads,
            // consecutive words
            static_assert(R % 256 == 0 || R < 256, "TMA boxes hold 256 rows");
            constexpr int box_rows = R < 256 ? R : 256;
            __shared__ __align__(8) uint64_t mbar;
            const uint32_t mb = smem_u32(&mbar);
            if (threadIdx.x == 0) mbar_init(mb, 1);
            __syncthreads();
            if (threadIdx.x == 0) {
                mbar_expect_tx(mb, (uint32_t)(C * R * sizeof(float2)));
                const int x = 2 * (ci.jj - c);      // first column of the tile, in floats
                const int y = ci.b * R;             // first row: point 0 of this transform
#pragma unroll 1
                for (int k = 0; k < R / box_rows; ++k)
                    tma_load_2d(smem_u32(sm + (size_t)k * box_rows * C), &tmap, x, y + k * box_rows, mb);
            }
            if (!mbar_wait_bounded(mb, 0) && p.err) atomicOr(p.err, 4);
#pragma unroll
            for (int i = 0; i < P; ++i) v[i] = sm[(g + G * i) * C + c];
            __syncthreads();   // the buffer is the exchange buffer of the first stage
        } else {
#pragma unroll
            for (int i = 0; i < P; ++i) v[i] = ld_data(src + (g + G * i) * Rr);
        }
        if (p.conj_in) {
#pragma unroll
            for (int i = 0; i < P; ++i) v[i].y = -v[i].y;
        }
        if constexpr (LD == FL_TWIDDLE) {
            if (p.tw_tiled) {
                const float2* tw = reinterpret_cast<const float2*>(p.tw_tiled) +
                                   (size_t)((ci.jj / C) % p.tw_tile_period) * (P * S::T) + threadIdx.x;
#pragma unroll
                for (int i = 0; i < P; ++i) v[i] = cmul(v[i], ld_table(tw + i * S::T, keep));
            } else if (ci.k) {
                fast_twiddle<P, G, S::TWB>(v, p, g, (uint32_t)ci.k * (uint32_t)p.Lr);
            }
        }
    }

    fast_stages_from<S, 0>(v, sm, c, g, twl);

    if constexpr (MID) {
        // forward output point n of this column is global index jj + n Rr of the convolution
        const float2* spec = reinterpret_cast<const float2*>(p.spectrum);
        // Rader: the DC term of the forward convolution FFT (global index 0 = register 0 of
        // thread 0 of column 0)
        if (p.dc_capture && ci.jj == 0 && g == 0) reinterpret_cast<float2*>(p.dcbuf)[ci.b] = v[0];
        if (p.tab_tiled) {
            const float2* tab = reinterpret_cast<const float2*>(p.tab_tiled) + (size_t)(ci.jj / C) * (P * S::T) + threadIdx.x;
#pragma unroll
            for (int i = 0; i < P; ++i) v[i] = cconj(cmul(v[i], ld_table(tab + i * S::T, keep)));
        } else {
#pragma unroll
            for (int i = 0; i < P; ++i) v[i] = cconj(cmul(v[i], __ldg(spec + ci.jj + (g + G * i) * Rr)));
        }
        fast_stages_from<S, 0>(v, sm, c, g, twl);
    }

    // ---- store ----
    const float scale = (float)p.scale;
    // no scaling and no conjugation (every pass but a transform's last): plain copies
    const bool unit = p.scale == 1.0 && !p.conj_out;
    if (p.Ns_out == 1) {
        // the tile's C columns are C consecutive length-R runs of the output: flat copy
        const float sy = p.conj_out ? -scale : scale;
        if constexpr (Own<S>::linear) {
            float2* wr = sm + Own<S>::base(c, g);
#pragma unroll
            for (int i = 0; i < P; ++i) wr[Own<S>::off(i)] = v[i];
        } else {
#pragma unroll
            for (int i = 0; i < P; ++i) sm[fast_addr<S>(c, g + G * i)] = v[i];
        }
        __syncthreads();
        const int64_t jj0 = ci.jj - c;
        float2* dst = reinterpret_cast<float2*>(p.out) + ci.out_base + jj0 * R;
        if (unit) {
#pragma unroll 4
            for (int e = threadIdx.x; e < C * R; e += S::T) dst[e] = sm[fast_addr<S>(e / R, e % R)];
        } else {
#pragma unroll 4
            for (int e = threadIdx.x; e < C * R; e += S::T) {
                const float2 u = sm[fast_addr<S>(e / R, e % R)];
                dst[e] = make_float2(u.x * scale, u.y * sy);
            }
        }
    } else {
        float2* dst = reinterpret_cast<float2*>(p.out) + ci.out_base + ci.out_j;
        const int ns = p.Ns_out;
        if (p.store_mode == ST_CHIRP) {
            // clamped unconditional table loads, predicated stores (see the chirp load)
            const float2* chirp = reinterpret_cast<const float2*>(p.chirp);
            const int nlast = (int)p.nvalid - 1;
            const float sy = p.conj_out ? -scale : scale;
            // the last pass has out_j = jj and Ns_out = Rr: table entry (tile, i, thread)
            const float2* tab = reinterpret_cast<const float2*>(p.tab_tiled) + (size_t)(ci.jj / C) * (P * S::T) + threadIdx.x;
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int oidx = ci.out_j + (g + G * i) * ns;
                const float2 w = p.tab_tiled ? ld_table(tab + i * S::T, keep) : __ldg(chirp + min(oidx, nlast));
                const float2 u = cmul(w, v[i]);
                if (oidx <= nlast) dst[(g + G * i) * ns] = make_float2(u.x * scale, u.y * sy);
            }
        } else if (p.store_mode == ST_SCATTER) {
            // Rader: out[scatter[k]] = (x0 + y*scale (conjugated forward)) * scale2, and the DC
            // term out[0] = (x0 + A0) * scale2 with A0 the forward convolution's DC term
            float2* obase = reinterpret_cast<float2*>(p.out) + ci.out_base;
            const int64_t os = p.split_m > 1 ? p.split_m : 1;
            const float2 x0 = ld_data(reinterpret_cast<const float2*>(p.x0buf) + ci.b);
            const float scale2 = (float)p.scale2;
            const int* scatter = p.scatter;
#pragma unroll
            for (int i = 0; i < P; ++i) {
                const int oidx = ci.out_j + (g + G * i) * ns;
                if (oidx == 0) {
                    float2 a0 = ld_data(reinterpret_cast<const float2*>(p.dcbuf) + ci.b);
                    if (!p.conj_out) a0.y = -a0.y;
                    obase[0] = cscale(cadd(x0, a0), scale2);
                }
                const int t = __ldg(scatter + oidx);
                if (t > 0) {
                    float2 u = cscale(v[i], scale);
                    if (p.conj_out) u.y = -u.y;
                    obase[t * os] = cscale(cadd(x0, u), scale2);
                }
            }
        } else if (unit) {
#pragma unroll
            for (int i = 0; i < P; ++i) dst[(g + G * i) * ns] = v[i];
        } else {
            const float sy = p.conj_out ? -scale : scale;
#pragma unroll
            for (int i = 0; i < P; ++i) dst[(g + G * i) * ns] = make_float2(v[i].x * scale, v[i].y * sy);
        }
    }
}

}  // namespace fyg
