// fyg_plan.cu -- planner and executor of the GB300 FFT library, and the plan part of the C ABI.
//
// Plan construction replaces fy::fft::FFT1D_C2C_invoker's constructor (foye_FFT.hpp:101-126):
// the strategy is chosen once, the stage schedule is derived from N's factorization, and all
// tables (twiddles, chirp, Rader permutations, convolution spectra) are computed once, on the
// host in long double (spectra: FP64 GPU FFT of the long-double kernel) and uploaded, or on the
// device from FP64 sincospi (the thread-order tables of the register-resident kernels).
// Each pass runs the register-resident kernel of its tile length when there is one
// (fyg_fast.cuh: FP32, 256-4096 / 243 / 343 points), else the shared-memory tile kernel.
//
// GPU strategies:
//   single    N <= one CTA's capacity and 13-smooth: one tile pass, several transforms per CTA
//             (replaces the smooth registry's radix engines and micro-kernels,
//             src/foye_FFT_radix_wrap.hpp:6-124, src/foye_FFT_radix{2,3,4,5,7}.hpp,
//             src/foye_FFT_microKernel.hpp, and the batch kernel src/foye_FFT_batch_kernel.hpp)
//   multi     13-smooth N above that: 2-3 Stockham passes of radix <= 4096 with the inter-pass
//             twiddle fused into the next pass's load (replaces the mixed-radix planner and
//             executor, src/foye_FFT_mix_radix.hpp:253-574)
//   rader     prime N with 13-smooth N-1: cyclic convolution of length N-1; other primes up to
//             the reference's Rader limit (39064): zero-padded linear convolution of 7-smooth
//             length M >= 2N-3 (src/foye_FFT_rader.hpp:142-401)
//   bluestein everything else: chirp-z with M >= 2N-1, the next power of two for FP32 when
//             M >= 65536 (register-resident passes), else 7-smooth (src/foye_FFT_bluestein.hpp:79-355)
// The reference's O(N^2) DFT fallback (src/foye_FFT_dft.hpp) is never used.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>

#include "fyg_host.h"

namespace fyg {

cudaError_t launch_f32(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st);
cudaError_t launch_f32c32(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st);
cudaError_t launch_f64(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st);
cudaError_t launch_mixed(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st);
cudaError_t launch_scale_copy(const void* in, void* out, size_t n, int dtype, double scale, int conj,
                              cudaStream_t st);

VariantInfo variant_info(int kv) {
    return {512, (kv == KV_F32_C16 || kv == KV_F32_C32 || kv == KV_FAST || kv == KV_SPLIT_F32) ? 8 : 16};
}

cudaError_t launch_pass(int kv, const PassParams& p, unsigned grid, int threads, size_t smem, cudaStream_t st,
                        const CUtensorMap* tmap) {
    if (kv == KV_FAST) return launch_fast(p, tmap, grid, st);
    if (kv == KV_SPLIT_F32 || kv == KV_SPLIT_F64) return launch_split(kv, p, grid, st);
    if (kv == KV_F32_C16) return launch_f32(kv, p, grid, threads, smem, st);
    if (kv == KV_F32_C32) return launch_f32c32(kv, p, grid, threads, smem, st);
    if (kv == KV_F64_C16) return launch_f64(kv, p, grid, threads, smem, st);
    return launch_mixed(kv, p, grid, threads, smem, st);
}

DevBuf::~DevBuf() {
    if (ptr) cudaFree(ptr);
}

int DevBuf::alloc(size_t n) {
    if (ptr) { cudaFree(ptr); ptr = nullptr; bytes = 0; }
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
        ptr = nullptr;
        cudaGetLastError();
        return set_error(FYG_ERR_ALLOC, "cudaMalloc(" + std::to_string(n) + ") failed: " + cudaGetErrorString(e));
    }
    bytes = n;
    return FYG_OK;
}

int DevBuf::upload(const void* host, size_t n) {
    int rc = alloc(n);
    if (rc) return rc;
    cudaError_t e = cudaMemcpy(ptr, host, n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "table upload");
    return FYG_OK;
}

// ------------------------------------------------------------------------------------------
// Table cache
// ------------------------------------------------------------------------------------------

namespace {
struct TableCache {
    std::mutex mu;
    std::map<std::string, std::shared_ptr<DevBuf>> map;
    uint64_t hits = 0, misses = 0;
};
// Heap-allocated and never destroyed: entries can outlive the CUDA runtime at process exit
// (fyg_plan_cache_clear releases what no plan uses).
TableCache& table_cache() {
    static TableCache* c = new TableCache();
    return *c;
}
}  // namespace

int cached_table(fyg_plan* pl, const std::string& key, const std::function<int(DevBuf&)>& build, const void** out) {
    const std::string k = "dev" + std::to_string(pl->device) + ":" + key;
    TableCache& tc = table_cache();
    {
        std::lock_guard<std::mutex> lk(tc.mu);
        auto it = tc.map.find(k);
        if (it != tc.map.end()) {
            ++tc.hits;
            pl->tables.push_back(it->second);
            *out = it->second->ptr;
            return FYG_OK;
        }
        ++tc.misses;
    }
    // built without the lock: building a spectrum creates (and caches) a sub-plan
    auto buf = std::make_shared<DevBuf>();
    const int rc = build(*buf);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(tc.mu);
        auto ins = tc.map.emplace(k, buf);
        if (!ins.second) buf = ins.first->second;   // built concurrently by another thread
    }
    pl->tables.push_back(buf);
    *out = buf->ptr;
    return FYG_OK;
}

FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    uint32_t s = 0;
    while ((1ull << s) < d) ++s;
    const uint64_t m = ((1ull << 32) * ((1ull << s) - d)) / d + 1;
    f.m = (uint32_t)m;
    f.s = s;
    return f;
}

// ------------------------------------------------------------------------------------------
// Number theory and the reference's strategy chain
// ------------------------------------------------------------------------------------------

static bool is_prime(uint64_t n) {
    if (n < 2) return false;
    if (n < 4) return true;
    if (n % 2 == 0 || n % 3 == 0) return false;
    for (uint64_t i = 5; i * i <= n; i += 6)
        if (n % i == 0 || n % (i + 2) == 0) return false;
    return true;
}

static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((unsigned __int128)a * b % m); }

static uint64_t powmod(uint64_t b, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    b %= m;
    while (e) {
        if (e & 1) r = mulmod(r, b, m);
        b = mulmod(b, b, m);
        e >>= 1;
    }
    return r;
}

static uint64_t primitive_root(uint64_t p) {
    if (p == 2) return 1;
    std::vector<uint64_t> f;
    uint64_t m = p - 1;
    for (uint64_t q = 2; q * q <= m; ++q)
        if (m % q == 0) { f.push_back(q); while (m % q == 0) m /= q; }
    if (m > 1) f.push_back(m);
    for (uint64_t g = 2; g < p; ++g) {
        bool ok = true;
        for (uint64_t q : f) if (powmod(g, (p - 1) / q, p) == 1) { ok = false; break; }
        if (ok) return g;
    }
    return 0;
}

// largest prime factor of n (1 for n == 1)
static uint64_t max_prime_factor(uint64_t n) {
    uint64_t best = 1;
    for (uint64_t q = 2; q * q <= n; ++q)
        while (n % q == 0) { best = q; n /= q; }
    if (n > 1) best = std::max(best, n);
    return best;
}

bool is_smooth(uint64_t n, uint64_t b) { return n >= 1 && max_prime_factor(n) <= b; }

static uint64_t next_smooth7(uint64_t n) {
    for (uint64_t m = std::max<uint64_t>(n, 1);; ++m)
        if (is_smooth(m, 7)) return m;
}

// The 38 lengths the reference's smooth registry supports directly (pure powers of 2, 3, 5, 7
// in its radix engines; src/foye_FFT_radix_wrap.hpp:87-98).  Needed to answer
// acquired_execution_strategy() exactly as the reference does.
static bool ref_directly_supported(uint64_t n) {
    auto pure_power = [](uint64_t n, uint64_t b, uint64_t maxv) {
        if (n < b || n > maxv) return false;
        while (n % b == 0) n /= b;
        return n == 1;
    };
    return pure_power(n, 2, 65536) || pure_power(n, 3, 59049) || pure_power(n, 5, 78125) ||
           pure_power(n, 7, 16807);
}

// foye_FFT.hpp:162-184 with src/foye_FFT_mix_radix.hpp:618-643 (every 7-smooth length is
// mixed-radix processable), src/foye_FFT_rader.hpp:403-423 (non-registered prime with
// 2n-3 <= 78125) and src/foye_FFT_bluestein.hpp:188-215 (n <= 39062).
static int ref_strategy(uint64_t n) {
    if (n < 2) return -1;
    if (ref_directly_supported(n)) return FYG_STRATEGY_KERNEL_DIRECT;
    if (is_smooth(n, 7)) return FYG_STRATEGY_MIX_RADIX;
    if (is_prime(n) && n <= 78125 && 2 * n - 3 <= 78125) return FYG_STRATEGY_RADER;
    if (n <= 39062) return FYG_STRATEGY_BLUESTEIN;
    return FYG_STRATEGY_DFT;
}

// N = m p with 2 <= m <= 8 and p prime, p - 1 13-smooth: m cyclic Rader transforms of length p
// after one pass of length-m DFTs (fyg_split.cu) move about N points per pass, where a Bluestein
// convolution moves 2N to 4N.  Returns m (0: no split) for lengths above 8192, whose Bluestein
// convolution (length >= 2N - 1 > 16384) takes more than one pass.
static uint64_t split_factor(uint64_t n) {
    if (n <= 8192 || is_smooth(n, 13) || is_prime(n)) return 0;
    for (uint64_t m = 2; m <= 8; ++m)
        if (n % m == 0 && is_prime(n / m) && is_smooth(n / m - 1, 13)) return m;
    return 0;
}

// ------------------------------------------------------------------------------------------
// Capacities and schedules
// ------------------------------------------------------------------------------------------

constexpr size_t kSmemLimit = 232448;  // 227 KB dynamic shared memory per CTA on sm_100/103

size_t smem_for(int cb, int R, int C, bool colmajor) {
    return cb == 8 ? tile_smem_bytes<float>(R, C, colmajor) : tile_smem_bytes<double>(R, C, colmajor);
}

int tile_class(int cb, int rmax) { return (cb == 8 && rmax > 16) ? 32 : 16; }

// Stage radices the kernels implement (FYG_STAGE_RADICES), and the largest one per compute type
// (a radix-r butterfly keeps 2r values in registers).
static const int kRadices[] = {
#define FYG_LIST(r) r,
    FYG_STAGE_RADICES(FYG_LIST)
#undef FYG_LIST
};
// Plans of uneven batches cap the stage radix at 16 so the persistent kernel compiles only the
// smaller codelets (lower register pressure); set for the duration of such a plan's creation.
static thread_local int t_radix_cap = 0;
// Uneven-batch group plans (FYG_FLAG_SMALL_TILES): stage-radix cap and single-pass tile cap
// (bytes of shared memory), 0 = defaults (16, 100 KB); set around a batch's plan creation.
static thread_local int t_batch_radix_cap = 0;
static thread_local size_t t_batch_single_cap = 0;
static int max_radix(int cb) {
    const int r = cb == 8 ? 32 : 16;
    return t_radix_cap ? std::min(r, t_radix_cap) : r;
}

// Radix schedule of an in-CTA transform of length R: fewest stages, then the smallest largest
// radix (register pressure), then larger radices first.  Empty if R is not representable.
std::vector<int> radices_for(int R, int cb) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, std::vector<int>> memo;
    const int rmax = max_radix(cb);
    const int key = cb * 1000 + rmax;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = memo.find({R, key});
        if (it != memo.end()) return it->second;
    }
    // best[d] = (stages, largest radix) for every divisor d of R
    std::map<int, std::pair<int, int>> best;
    std::map<int, int> choice;
    std::vector<int> divs;
    for (int d = 1; d <= R; ++d) if (R % d == 0) divs.push_back(d);
    best[1] = {0, 0};
    for (int d : divs) {
        if (d == 1) continue;
        std::pair<int, int> bd = {1 << 20, 0};
        int bc = 0;
        for (int r : kRadices) {
            if (r > rmax || d % r) continue;
            auto it = best.find(d / r);
            if (it == best.end() || it->second.first >= (1 << 20)) continue;
            std::pair<int, int> cand = {it->second.first + 1, std::max(it->second.second, r)};
            if (cand < bd || (cand == bd && r > bc)) { bd = cand; bc = r; }
        }
        best[d] = bd;
        choice[d] = bc;
    }
    std::vector<int> out;
    if (best[R].first < (1 << 20) && best[R].first <= kMaxStages) {
        for (int d = R; d > 1; d /= choice[d]) out.push_back(choice[d]);
        std::sort(out.begin(), out.end(), std::greater<int>());
    }
    std::lock_guard<std::mutex> lk(mu);
    memo[{R, key}] = out;
    return out;
}

// Columns per element-major tile: 8 (64 B fp32 segments) while two CTAs still fit on an SM,
// else 4; 0 if not even 4 columns fit.
int multi_C(int cb, int R) {
    if (tile_fits(cb, R, 8, false) && smem_for(cb, R, 8, false) <= kSmemLimit / 2) return 8;
    if (tile_fits(cb, R, 4, false)) return 4;
    return 0;
}

bool tile_fits(int cb, int R, int C, bool colmajor) {
    const std::vector<int> r = radices_for(R, cb);
    if (r.empty()) return false;
    return smem_for(cb, R, C, colmajor) <= kSmemLimit;
}

// Split L into P >= 2 pass radices whose C-column tiles fit in shared memory: fewest passes,
// then fewest in-CTA stages, then the most balanced split.  For convolution pipelines the last
// forward radix also runs the fused mid pass (two buffers).
// Schedule overrides of fyg_plan_create_ex (0 = planner default), set for the duration of one
// plan's creation.
static thread_local uint64_t t_max_pass_r = 0;
static thread_local uint64_t t_conv_len = 0;
static thread_local int t_order = 0;  // 1: reversed pass order
static thread_local size_t t_idist = 0, t_odist = 0;  // user layout of the next plan (0: contiguous)
static thread_local int t_cols = 0;   // single-pass: transforms per CTA (threads per transform = T/C)
static thread_local int t_threads = 0;  // single-pass: thread policy of single_pass_threads

bool split_passes(uint64_t L, int cb, bool conv, std::vector<int>& out) {
    std::vector<int> divs;
    const int dmax = t_max_pass_r ? (int)std::min<uint64_t>(t_max_pass_r, 4096) : 4096;
    for (int d = 4; d <= dmax && (uint64_t)d <= L; ++d)
        if (L % d == 0 && multi_C(cb, d)) divs.push_back(d);
    if (divs.empty()) return false;
    const int Rmax = divs.back();
    for (int P = 2; P <= 6; ++P) {
        double best = 1e30;
        std::vector<int> best_f, cur;
        const double target = std::log((double)L) / P;
        std::function<void(uint64_t, int)> rec = [&](uint64_t rem, int left) {
            if (left == 1) {
                if (rem > (uint64_t)Rmax || rem < 2) return;
                if (!multi_C(cb, (int)rem)) return;
                cur.push_back((int)rem);
                {
                    double cost = 0;
                    for (int f : cur)
                        cost += (double)radices_for(f, cb).size() + 0.25 * std::fabs(std::log((double)f) - target);
                    if (cost < best) { best = cost; best_f = cur; }
                }
                cur.pop_back();
                return;
            }
            for (int d : divs) {
                if (rem % d) continue;
                if ((double)(rem / d) > std::pow((double)Rmax, left - 1)) continue;
                cur.push_back(d);
                rec(rem / d, left - 1);
                cur.pop_back();
            }
        };
        rec(L, P);
        if (!best_f.empty()) {
            out = best_f;
            return true;
        }
    }
    return false;
}

void fill_geom(TileGeom& g, int R, int C, bool colmajor, const std::vector<int>& rad) {
    std::memset(&g, 0, sizeof(g));
    g.R = R;
    g.C = C;
    int lc = 0;
    while ((1 << lc) < C) ++lc;
    g.log2C = lc;
    g.colmajor = colmajor ? 1 : 0;
    g.nst = (int)rad.size();
    int ns = 1, off = 0;
    for (size_t s = 0; s < rad.size(); ++s) {
        g.radix[s] = rad[s];
        g.ns[s] = make_fastdiv((uint32_t)ns);
        g.twmul[s] = R / (ns * rad[s]);
        g.rr[s] = make_fastdiv((uint32_t)(R / rad[s]));
        g.twoff[s] = off;                       // stage 0 has no twiddles and no block
        if (s > 0) off += rad[s] * ns;
        ns *= rad[s];
    }
    g.divR = make_fastdiv((uint32_t)R);
}

// ------------------------------------------------------------------------------------------
// Tables
// ------------------------------------------------------------------------------------------

static const long double kTwoPiL = 6.283185307179586476925286766559005768L;

// exp(-2 pi i t/n) in long double with exact integer reduction of t
void twiddle_ld(uint64_t t, uint64_t n, long double* c, long double* s) {
    t %= n;
    // reduce to the first octant-friendly form: angle = 2 pi t / n, t < n
    const long double a = kTwoPiL * (long double)t / (long double)n;
    *c = cosl(a);
    *s = -sinl(a);
}

// Host images of the twiddle tables (shared by plans and by the allocation-free entry point).
std::vector<unsigned char> host_local_table(int R, int cb) {
    std::vector<unsigned char> out((size_t)R * 2 * cb);
    for (int t = 0; t < R; ++t) {
        long double c, s;
        twiddle_ld(t, R, &c, &s);
        if (cb == 8) reinterpret_cast<float2*>(out.data())[t] = make_float2((float)c, (float)s);
        else reinterpret_cast<double2*>(out.data())[t] = make_double2((double)c, (double)s);
    }
    return out;
}

// two-level table of w_L: hi[i] = w^(i 2^s), lo[j] = w^j; float tables hold (hi, lo) pairs
void host_two_level(uint64_t L, int cb, std::vector<unsigned char>& hi, std::vector<unsigned char>& lo, int* shift) {
    int s = 0;
    while ((1ull << (2 * s)) < L) ++s;  // 2^s ~ sqrt(L)
    if (s < 1) s = 1;
    const uint64_t B = 1ull << s, nhi = (L + B - 1) / B;
    auto pack = [](long double c, long double sn) {
        const float ch = (float)c, sh = (float)sn;
        return make_float4(ch, sh, (float)(c - (long double)ch), (float)(sn - (long double)sh));
    };
    const size_t es = cb == 8 ? sizeof(float4) : sizeof(double2);
    hi.assign(nhi * es, 0);
    lo.assign(B * es, 0);
    for (uint64_t i = 0; i < nhi + B; ++i) {
        const bool h = i < nhi;
        const uint64_t t = h ? i * B : i - nhi;
        long double c, sn;
        twiddle_ld(t, L, &c, &sn);
        unsigned char* dst = h ? hi.data() + i * es : lo.data() + (i - nhi) * es;
        if (cb == 8) *reinterpret_cast<float4*>(dst) = pack(c, sn);
        else *reinterpret_cast<double2*>(dst) = make_double2((double)c, (double)sn);
    }
    *shift = s;
}

static int upload_local_table(fyg_plan* pl, int R, int cb, const void** dptr) {
    return cached_table(pl, "local:" + std::to_string(R) + ":" + std::to_string(cb), [&](DevBuf& b) {
        const std::vector<unsigned char> h = host_local_table(R, cb);
        return b.upload(h.data(), h.size());
    }, dptr);
}

// one buffer: the hi table, then the lo table (both 16-byte entries)
static int upload_two_level(fyg_plan* pl, uint64_t L, int cb, const void** hi, const void** lo, int* shift) {
    std::vector<unsigned char> th, tl;
    size_t hi_bytes = 0;
    int s = 0;
    host_two_level(L, cb, th, tl, &s);   // cheap next to the plan's other work: O(sqrt L) entries
    hi_bytes = th.size();
    const void* base = nullptr;
    const int rc = cached_table(pl, "twolevel:" + std::to_string(L) + ":" + std::to_string(cb), [&](DevBuf& b) {
        std::vector<unsigned char> all(th);
        all.insert(all.end(), tl.begin(), tl.end());
        return b.upload(all.data(), all.size());
    }, &base);
    if (rc) return rc;
    *hi = base;
    *lo = static_cast<const unsigned char*>(base) + hi_bytes;
    *shift = s;
    return FYG_OK;
}

// ------------------------------------------------------------------------------------------
// Pipelines
// ------------------------------------------------------------------------------------------

struct ConvTables {
    const void* chirp = nullptr;
    const int* gather = nullptr;
    const int* scatter = nullptr;
    const void* spectrum = nullptr;
    std::string src_key;      // identifies the transform these tables belong to (cache keys)
};

struct PipeSpec {
    int kind;                 // GS_*
    uint64_t L;               // algorithm length
    std::vector<int> prad;    // pass radices (size 1 for single-pass)
    int C;                    // columns per tile (single-pass: transforms per CTA)
    int threads = 0;          // single-pass: thread policy (single_pass_threads)
};

// The N = m p split: a first pass (fyg_split.cu) ahead of a Rader pipeline of length p over m
// times the batch, whose scatter store interleaves the m transforms of each user transform.
struct SplitSpec {
    uint64_t m = 1;              // 1: no split
    uint64_t p = 0;              // length of the Rader transforms
    const void* tw = nullptr;    // w_N^t, t < N (user element type)
};

int pick_variant(int compute_cb, int tin_cb, int tout_cb, int cls) {
    if (compute_cb == 8) return cls <= 16 ? KV_F32_C16 : KV_F32_C32;
    if (tin_cb == 16 && tout_cb == 16) return KV_F64_C16;
    if (tin_cb == 8 && tout_cb == 16) return KV_F64_IF32_C16;
    if (tin_cb == 16 && tout_cb == 8) return KV_F64_OF32_C16;
    return KV_F64_F32IO_C16;
}

// about 16 elements per thread
int threads_for(int R, int C, int maxt) {
    int t = (R * C + 15) / 16;
    t = (t + 31) / 32 * 32;
    t = std::max(t, 64);
    return std::min(t, maxt);
}

// Single-pass tiles (whole transforms per CTA).
// Transforms per CTA: `requested` (the autotuner's choice) or about 4096 (FP32) / 2048 (FP64)
// points per CTA; at most the batch and 256, and 1 when C transforms would not fit in shared
// memory.
int single_pass_cols(int cb, int L, size_t batch, int requested) {
    int C = requested ? requested : std::max(1, (cb == 8 ? 4096 : 2048) / L);
    C = (int)std::min<uint64_t>((uint64_t)C, batch);
    C = std::max(std::min(C, 256), 1);
    if (smem_for(cb, L, C, true) > kSmemLimit) C = 1;
    return C;
}

// Threads per CTA of a single-pass tile: `requested` policy 0 = about 16 points per thread
// (throughput: many CTAs per SM), 1 = one thread per butterfly of the stage with the most
// butterflies (latency: the few CTAs of a small batch finish each stage in one step).
int single_pass_threads(int L, int C, const std::vector<int>& rad, int requested) {
    if (requested == 1 && !rad.empty()) {
        const int rmin = *std::min_element(rad.begin(), rad.end());
        int t = (L / rmin) * C;
        t = (t + 31) / 32 * 32;
        return std::max(64, std::min(t, kMaxThreads));
    }
    return threads_for(L, C, kMaxThreads);
}

// Whether a 13-smooth length runs as one tile pass (whole transform per CTA) within `cap`
// bytes of shared memory.
bool single_pass_fits(int cb, uint64_t n, size_t cap) {
    return is_smooth(n, 13) && n <= 16384 && tile_fits(cb, (int)n, 1, true) && smem_for(cb, (int)n, 1, true) <= cap;
}

static int build_pipeline(fyg_plan* pl, const PipeSpec& ps, bool inverse,
                          const std::map<int, const void*>& local_tabs, const void* tw_hi,
                          const void* tw_lo, int tw_shift, const ConvTables& ct, const SplitSpec& sp,
                          std::vector<PassDesc>& out) {
    out.clear();
    const int P = (int)ps.prad.size();
    const bool conv = ps.kind == GS_RADER || ps.kind == GS_BLUESTEIN;
    const int K = conv ? 2 * P - 1 : P;
    const int cb = pl->compute_bytes;
    const int io_cb = pl->dtype == FYG_C32 ? 8 : 16;
    const uint64_t n = pl->n, L = ps.L;
    uint64_t ns_fwd = 1, ns_inv = 1;
    for (int i = 0; i < K; ++i) {
        PassDesc d;
        std::memset(&d.p, 0, sizeof(d.p));
        PassParams& p = d.p;
        const bool first = i == 0, last = i == K - 1;
        const bool mid = conv && i == P - 1;
        int R;
        uint64_t Ns;
        if (i < P) { R = ps.prad[i]; Ns = ns_fwd; ns_fwd *= R; }
        else { R = ps.prad[K - 1 - i]; Ns = ns_inv; ns_inv *= R; }
        if (mid) ns_inv = R;  // the mid pass also performs the first inverse pass (radix R, Ns 1)
        const bool single = (P == 1);
        const int C = single ? ps.C : multi_C(cb, R);
        const std::vector<int> rad = radices_for(R, cb);
        fill_geom(p.g, R, C, single, rad);
        // stage twiddles of the tile kernel's in-CTA schedule, one block per stage s >= 1:
        // w_R^(m k twm_s) at twoff_s + m ns_s + k
        {
            std::string key = "gstage:" + std::to_string(R) + ":" + std::to_string(cb);
            for (int r : rad) key += ":" + std::to_string(r);
            int rc = cached_table(pl, key, [&](DevBuf& b) {
                std::vector<unsigned char> t;
                uint64_t ns = 1;
                auto put = [&](long double c, long double sn) {
                    if (cb == 8) {
                        const float2 v = make_float2((float)c, (float)sn);
                        t.insert(t.end(), (const unsigned char*)&v, (const unsigned char*)&v + sizeof(v));
                    } else {
                        const double2 v = make_double2((double)c, (double)sn);
                        t.insert(t.end(), (const unsigned char*)&v, (const unsigned char*)&v + sizeof(v));
                    }
                };
                for (size_t st = 0; st < rad.size(); ++st) {
                    const uint64_t r = (uint64_t)rad[st], twm = (uint64_t)R / (ns * r);
                    if (st > 0)
                        for (uint64_t m = 0; m < r; ++m)
                            for (uint64_t k = 0; k < ns; ++k) {
                                long double c, sn;
                                twiddle_ld(m * k * twm, (uint64_t)R, &c, &sn);
                                put(c, sn);
                            }
                    ns *= r;
                }
                if (t.empty()) put(1.0L, 0.0L);
                return b.upload(t.data(), t.size());
            }, &p.tw_stage);
            if (rc) return rc;
        }
        p.Rr = (int)(L / R);
        p.Ns = (int)Ns;
        p.Ns_out = mid ? 1 : (int)Ns;
        p.Lr = (int)(L / (Ns * R));
        p.div_Rr = make_fastdiv((uint32_t)p.Rr);
        p.div_Ns = make_fastdiv((uint32_t)p.Ns);
        p.div_Ns_out = make_fastdiv((uint32_t)p.Ns_out);
        p.tw_local = local_tabs.at(R);
        p.tw_hi = tw_hi;
        p.tw_lo = tw_lo;
        p.tw_shift = tw_shift;
        p.scale = 1.0;
        p.scale2 = 1.0;
        p.nvalid = (int64_t)n;
        p.mid = mid ? 1 : 0;
        p.spectrum = ct.spectrum;
        p.chirp = ct.chirp;
        p.gather = ct.gather;
        p.scatter = ct.scatter;
        p.err = reinterpret_cast<int*>(pl->errword.ptr);
        const bool split = sp.m > 1;
        d.in_role = first ? (split ? ROLE_S2 : ROLE_IN) : ((i - 1) % 2 == 0 ? ROLE_S0 : ROLE_S1);
        d.out_role = last ? ROLE_OUT : (i % 2 == 0 ? ROLE_S0 : ROLE_S1);
        d.in_elem_bytes = (d.in_role == ROLE_IN || d.in_role == ROLE_S2) ? io_cb : cb;
        d.out_elem_bytes = d.out_role == ROLE_OUT ? io_cb : cb;
        p.idist = d.in_role == ROLE_IN ? (int64_t)pl->idist : d.in_role == ROLE_S2 ? (int64_t)sp.p : (int64_t)L;
        p.odist = d.out_role == ROLE_OUT ? (int64_t)pl->odist : (int64_t)L;
        d.in_len = d.in_role == ROLE_IN ? (int64_t)n : d.in_role == ROLE_S2 ? (int64_t)sp.p : (int64_t)L;
        d.out_len = d.out_role == ROLE_OUT ? (int64_t)(split ? sp.p : n) : (int64_t)L;
        d.bmul = (int)sp.m;
        if (last && split) p.split_m = (int)sp.m;
        // load / store fusions
        p.load_mode = LD_PLAIN;
        p.store_mode = ST_PLAIN;
        if (first) {
            p.conj_in = inverse ? 1 : 0;
            if (ps.kind == GS_BLUESTEIN) p.load_mode = LD_CHIRP;
            if (ps.kind == GS_RADER) { p.load_mode = LD_GATHER; p.x0_from_in = 1; }
        }
        if (mid && ps.kind == GS_RADER) p.dc_capture = 1;
        if (last) {
            if (ps.kind == GS_BLUESTEIN) {
                p.store_mode = ST_CHIRP;
                p.conj_out = inverse ? 0 : 1;
                p.scale = inverse ? 1.0 / ((double)L * (double)n) : 1.0 / (double)L;
            } else if (ps.kind == GS_RADER) {
                p.store_mode = ST_SCATTER;
                p.conj_out = inverse ? 0 : 1;
                p.scale = 1.0 / (double)L;
                p.scale2 = inverse ? 1.0 / (double)n : 1.0;
            } else {
                p.conj_out = inverse ? 1 : 0;
                p.scale = inverse ? 1.0 / (double)n : 1.0;
            }
        }
        const int rmax = *std::max_element(rad.begin(), rad.end());
        const int cls = tile_class(cb, rmax);
        d.threads = single ? single_pass_threads(R, C, rad, ps.threads) : threads_for(R, C, kMaxThreads);
        d.kv = pick_variant(cb, (int)d.in_elem_bytes, (int)d.out_elem_bytes, cls);
        d.smem = smem_for(cb, R, C, single);
        // register-resident kernel for the tile lengths it is compiled for (FP32; not for the
        // tiles of uneven batches, which run inside the generic persistent kernel); the
        // inter-pass twiddle table needs C | Ns
        int fc = 0, ft = 0, wide = 0;
        size_t fsm = 0;
        auto shape_ok = [&](int w) {
            return fast_shape(R, w, &fc, &ft, &fsm) && (L / R) % (uint64_t)fc == 0 && (p.Ns <= 1 || p.Ns % fc == 0);
        };
        // the wide shape (FYG_FLAG_WIDE_TILES) where its column count divides the pass, else
        // the narrow one
        const bool want_fast = pl->dtype == FYG_C32 && cb == 8 && !single &&
                               !(pl->flags & (FYG_FLAG_SMALL_TILES | FYG_FLAG_GENERIC_KERNELS)) &&
                               !(p.mid && (p.load_mode != LD_PLAIN || p.Ns <= 1));
        bool fast = false;
        if (want_fast && (pl->flags & FYG_FLAG_WIDE_TILES) && shape_ok(1)) { fast = true; wide = 1; }
        else if (want_fast && shape_ok(0)) fast = true;
        if (fast) {
            fill_geom(p.g, R, fc, false, rad);
            p.reverse_tiles = i & 1;   // measured 0.3-2% faster than one order for all passes
            // in-tile stage twiddles, one block per stage s >= 1: w_R^(m k twm) at m ns + k
            {
                int srad[kMaxStages], sns[kMaxStages];
                const int nst = fast_stages(R, srad, sns);
                int rc = cached_table(pl, "stagetw:" + std::to_string(R), [&](DevBuf& b) {
                    std::vector<float2> t;
                    for (int st = 1; st < nst; ++st) {
                        const uint64_t twm = (uint64_t)R / ((uint64_t)sns[st] * (uint64_t)srad[st]);
                        for (int m = 0; m < srad[st]; ++m)
                            for (int k = 0; k < sns[st]; ++k) {
                                long double c, sn;
                                twiddle_ld((uint64_t)m * (uint64_t)k * twm, (uint64_t)R, &c, &sn);
                                t.push_back(make_float2((float)c, (float)sn));
                            }
                    }
                    if (t.empty()) t.push_back(make_float2(1.f, 0.f));
                    return b.upload(t.data(), t.size() * sizeof(float2));
                }, &p.tw_stage);
                if (rc) return rc;
            }
            d.kv = KV_FAST;
            d.threads = ft;
            d.smem = fsm;
            // thread-order tables (shared by the forward and inverse pipelines)
            // keyed by content: the source table's own key (which transform's chirp or spectrum)
            // and the tile geometry
            auto tiled = [&](const std::string& key, uint64_t total, int kind, const void* src, int64_t nvalid,
                             int conj, const void** outp) -> int {
                return cached_table(pl, "tiled:" + key, [&](DevBuf& b) {
                    int rc = b.alloc(total * sizeof(float2));
                    if (rc) return rc;
                    cudaError_t e = launch_fast_table(static_cast<float2*>(b.ptr), total, R, wide, kind, (uint64_t)p.Lr,
                                                      L, (uint64_t)p.Rr, static_cast<const float2*>(src), nvalid, conj,
                                                      0);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
                    return e == cudaSuccess ? FYG_OK : cuda_error(e, "thread-order table");
                }, outp);
            };
            const std::string sh = std::to_string(R) + "x" + std::to_string(fc) + ":" + std::to_string(Ns) + ":" +
                                   std::to_string(L) + ":" + ct.src_key;
            int rc = FYG_OK;
            if (p.Ns > 1 && p.load_mode == LD_PLAIN) {
                rc = tiled("tw:" + sh, Ns * (uint64_t)R, 0, nullptr, 0, 0, &p.tw_tiled);
                p.tw_tile_period = (int)(Ns / (uint64_t)fc);
            }
            if (!rc && p.mid) rc = tiled("spec:" + sh, L, 1, ct.spectrum, (int64_t)L, 0, &p.tab_tiled);
            else if (!rc && p.load_mode == LD_CHIRP) rc = tiled("chin:" + sh, L, 1, ct.chirp, (int64_t)n, 1, &p.tab_tiled);
            else if (!rc && p.store_mode == ST_CHIRP && p.Ns_out == p.Rr)
                rc = tiled("chout:" + sh, L, 1, ct.chirp, (int64_t)n, 0, &p.tab_tiled);
            if (rc) return rc;
        }
        // TMA tile loads for register-resident passes that read a scratch buffer of the plan
        // (its address is fixed; power-of-two tiles, boxes of 256 rows).  By default only for
        // tiles of 4 columns (32-byte rows: R = 2048, 4096), where they measured faster than
        // per-thread loads (Bluestein 999983 x 64 mid pass 0.809 -> 0.733 ms); on 8-column tiles
        // they measured slower (2^20 x 64 second pass 0.216 -> 0.240 ms).
        // FYG_FLAG_TMA_LOADS: every eligible pass; FYG_FLAG_NO_TMA_LOADS: none.
        const bool tma_wanted = !(pl->flags & FYG_FLAG_NO_TMA_LOADS) &&
                                ((pl->flags & FYG_FLAG_TMA_LOADS) || (d.kv == KV_FAST && p.g.C <= 4));
        if (tma_wanted && d.kv == KV_FAST && p.load_mode == LD_PLAIN && p.Ns > 1 &&
            (d.in_role == ROLE_S0 || d.in_role == ROLE_S1) && (R % 256 == 0)) {
            const void* base = d.in_role == ROLE_S0 ? pl->scratch0.ptr : pl->scratch1.ptr;
            if (encode_tile_map(&d.tmap, base, (uint64_t)p.Rr, (uint64_t)pl->chunk * sp.m * (uint64_t)R, p.g.C, R) ==
                cudaSuccess)
                d.tma = true;
            else
                cudaGetLastError();
        }
        if (d.smem > kSmemLimit)
            return set_error(FYG_ERR_UNSUPPORTED, "tile of " + std::to_string(R) + "x" + std::to_string(C) +
                                                      " exceeds shared memory");
        out.push_back(d);
    }
    if (sp.m > 1) {
        // the split pass: user input -> scratch2 (m length-p transforms per user transform)
        PassDesc d;
        std::memset(&d.p, 0, sizeof(d.p));
        PassParams& p = d.p;
        p.g.R = (int)sp.m;
        p.g.C = split_threads();
        p.Rr = (int)sp.p;
        p.div_Rr = make_fastdiv((uint32_t)sp.p);
        p.idist = (int64_t)pl->idist;
        p.odist = (int64_t)n;
        p.conj_in = inverse ? 1 : 0;
        p.tw_stage = sp.tw;
        p.scale = p.scale2 = 1.0;
        p.err = reinterpret_cast<int*>(pl->errword.ptr);
        d.in_role = ROLE_IN;
        d.out_role = ROLE_S2;
        d.in_elem_bytes = d.out_elem_bytes = io_cb;
        d.in_len = d.out_len = (int64_t)n;
        d.kv = pl->dtype == FYG_C32 ? KV_SPLIT_F32 : KV_SPLIT_F64;
        d.threads = split_threads();
        d.smem = 0;
        out.insert(out.begin(), d);
    }
    return FYG_OK;
}

// FP64 transform of a host vector on the GPU (used to precompute convolution spectra).
static int gpu_fft_f64(size_t n, const std::vector<double2>& h, std::vector<double2>& H);

// Spectrum of a convolution kernel: FP64 GPU FFT of the long-double kernel, rounded once to the
// compute type.
static int upload_spectrum(DevBuf& b, const std::vector<double2>& kernel_time, int cb) {
    const size_t M = kernel_time.size();
    std::vector<double2> H;
    int rc = gpu_fft_f64(M, kernel_time, H);
    if (rc) return rc;
    if (cb == 8) {
        std::vector<float2> Hf(M);
        for (size_t i = 0; i < M; ++i) Hf[i] = make_float2((float)H[i].x, (float)H[i].y);
        return b.upload(Hf.data(), M * sizeof(float2));
    }
    return b.upload(H.data(), M * sizeof(double2));
}

// The schedule of a plan, without touching the GPU: strategy, algorithm length, the N = m p
// split factor, pass radices, and for single-pass lengths the transforms per CTA.  Sets
// pl->strategy, split_m, L, conv_fp64 and compute_bytes from pl->n, dtype, flags and batch (and
// the schedule options of plan_create_opts).  n >= 2.
static int plan_spec(fyg_plan* pl, PipeSpec& ps, uint64_t& nt, uint64_t& split_m) {
    const uint64_t n = pl->n;
    const int io_cb = pl->dtype == FYG_C32 ? 8 : 16;
    ps.C = 1;
    // nt: length of the transforms the Rader / Bluestein passes compute (N / m for the split)
    nt = n;
    split_m = 1;
    const size_t single_cap = (pl->flags & FYG_FLAG_SMALL_TILES)
                                  ? (t_batch_single_cap ? std::min(t_batch_single_cap, kSmemLimit) : (100u << 10))
                                  : kSmemLimit;
    if (single_pass_fits(io_cb, n, single_cap)) {
        ps.kind = GS_SINGLE;
        ps.L = n;
        ps.prad = {(int)n};
    } else if (is_smooth(n, 13)) {
        ps.kind = GS_MULTI;
        ps.L = n;
    } else if (is_prime(n) && (is_smooth(n - 1, 13) || 2 * n - 3 <= 78125)) {
        ps.kind = GS_RADER;
        const uint64_t Lc = n - 1;
        ps.L = is_smooth(Lc, 13) ? Lc : next_smooth7(2 * Lc - 1);
        if (t_conv_len) {
            if (!(t_conv_len == Lc && is_smooth(Lc, 13)) && !(t_conv_len >= 2 * Lc - 1 && is_smooth(t_conv_len, 7)))
                return set_error(FYG_ERR_INVALID_ARG, "Rader convolution length must be N-1 (13-smooth) or 7-smooth >= 2N-3");
            ps.L = t_conv_len;
        }
    } else if (!t_conv_len && !(pl->flags & FYG_FLAG_SMALL_TILES) && (split_m = split_factor(n)) > 1) {
        // N = m p: the first pass (fyg_split.cu) leaves m length-p transforms per transform,
        // which run as a cyclic Rader pipeline over m times the batch
        ps.kind = GS_RADER;
        nt = n / split_m;
        ps.L = nt - 1;
    } else {
        split_m = 1;
        ps.kind = GS_BLUESTEIN;
        ps.L = next_smooth7(2 * n - 1);
        // FP32 multi-pass convolutions: the power-of-two length runs on the register-resident
        // kernels, which more than make up for up to twice the points
        uint64_t m2 = 1;
        while (m2 < 2 * n - 1) m2 <<= 1;
        if (pl->dtype == FYG_C32 && m2 >= 65536 &&
            !(pl->flags & (FYG_FLAG_CONV_FP64 | FYG_FLAG_SMALL_TILES | FYG_FLAG_GENERIC_KERNELS)))
            ps.L = m2;
        if (t_conv_len) {
            if (t_conv_len < 2 * n - 1 || !is_smooth(t_conv_len, 7))
                return set_error(FYG_ERR_INVALID_ARG, "Bluestein convolution length must be 7-smooth and >= 2N-1");
            ps.L = t_conv_len;
        }
    }
    pl->strategy = split_m > 1 ? GS_SPLIT : ps.kind;
    pl->split_m = split_m;
    pl->L = ps.L;
    const bool conv = ps.kind == GS_RADER || ps.kind == GS_BLUESTEIN;
    if (conv && pl->dtype == FYG_C32) {
        if (pl->flags & FYG_FLAG_CONV_FP64) pl->conv_fp64 = 1;
        else pl->conv_fp64 = 0;
    }
    pl->compute_bytes = (pl->dtype == FYG_C64 || pl->conv_fp64) ? 16 : 8;
    const int cb = pl->compute_bytes;
    if (ps.kind != GS_SINGLE) {
        if (conv && ps.L <= 16384 && tile_fits(cb, (int)ps.L, 1, true) &&
            smem_for(cb, (int)ps.L, 1, true) <= single_cap) {
            ps.prad = {(int)ps.L};
        } else if (!split_passes(ps.L, cb, conv, ps.prad)) {
            return set_error(FYG_ERR_UNSUPPORTED, "no pass decomposition for length " + std::to_string(ps.L));
        } else if (t_order) {
            std::reverse(ps.prad.begin(), ps.prad.end());
            for (int R : ps.prad)
                if (!tile_fits(cb, R, multi_C(cb, R), false) || (conv && R == ps.prad.back() && !multi_C(cb, R)))
                    return set_error(FYG_ERR_UNSUPPORTED, "reversed pass order does not fit shared memory");
        }
    }
    if (ps.prad.size() == 1) {
        ps.C = single_pass_cols(cb, (int)ps.L, pl->batch, t_cols);
        ps.threads = t_threads;
    }
    return FYG_OK;
}

static int make_plan(fyg_plan* pl) {
    const uint64_t n = pl->n;
    const int io_cb = pl->dtype == FYG_C32 ? 8 : 16;
    PipeSpec ps;
    ps.C = 1;
    ConvTables ct;

    if (n == 1) {
        pl->strategy = GS_COPY;
        pl->L = 1;
        pl->compute_bytes = io_cb;
        return FYG_OK;
    }
    // ---- strategy and pass schedule ----
    uint64_t nt = n, split_m = 1;
    int rc = plan_spec(pl, ps, nt, split_m);
    if (rc) return rc;
    const bool conv = ps.kind == GS_RADER || ps.kind == GS_BLUESTEIN;
    const int cb = pl->compute_bytes;
    const int P = (int)ps.prad.size();
    // ---- chunking: keep the scratch of one chunk L2-resident ----
    const int K = conv ? 2 * P - 1 : P;
    if (K == 1 && split_m == 1) pl->chunk = pl->batch;
    else {
        // Whole batch per pass unless a scratch buffer would exceed 4 GB: measured on GB300, an
        // L2-sized chunk (8-128 MB) is 1.1-1.5x slower than one launch per pass over the batch,
        // because the tile kernels are issue-bound, not HBM-bound.  FYG_CHUNK_MB overrides.
        uint64_t chunk_mb = 4096;
        if (const char* e = std::getenv("FYG_CHUNK_MB")) chunk_mb = std::max<uint64_t>(1, std::strtoull(e, nullptr, 10));
        const uint64_t chunk_elems = (chunk_mb << 20) / cb;
        uint64_t c = std::max<uint64_t>(1, chunk_elems / (ps.L * split_m));
        if (pl->flags & FYG_FLAG_NO_L2_CHUNK) c = pl->batch;
        pl->chunk = (size_t)std::min<uint64_t>(c, pl->batch);
    }
    // column indices are 32-bit inside the kernels
    const uint64_t maxRr = ps.L / *std::min_element(ps.prad.begin(), ps.prad.end());
    if ((uint64_t)pl->chunk * split_m * std::max<uint64_t>(maxRr, split_m > 1 ? nt : 1) >= (1ull << 31) ||
        ps.L >= (1ull << 31))
        return set_error(FYG_ERR_INVALID_LENGTH, "length/batch too large for 32-bit tile indexing");

    rc = pl->errword.alloc(16);
    if (rc) return rc;
    cudaMemset(pl->errword.ptr, 0, 16);
    // ---- tables ----
    std::map<int, const void*> local_tabs;
    for (int R : ps.prad)
        if (!local_tabs.count(R)) {
            const void* d = nullptr;
            rc = upload_local_table(pl, R, cb, &d);
            if (rc) return rc;
            local_tabs[R] = d;
        }
    const void *tw_hi = nullptr, *tw_lo = nullptr;
    int tw_shift = 1;
    if (P > 1) {
        rc = upload_two_level(pl, ps.L, cb, &tw_hi, &tw_lo, &tw_shift);
        if (rc) return rc;
    }
    const std::string cbs = std::to_string(cb);
    if (ps.kind == GS_BLUESTEIN) {
        // chirp w[k] = exp(+i pi (k^2 mod 2N) / N), exact integer reduction, long double
        const uint64_t twoN = 2 * n, M = ps.L;
        std::vector<long double> wc, ws;
        auto chirp_ld = [&]() {
            if (!wc.empty()) return;
            wc.resize(n);
            ws.resize(n);
            for (uint64_t k = 0; k < n; ++k) {
                const uint64_t sq = mulmod(k, k, twoN);
                const long double a = kTwoPiL * 0.5L * (long double)sq / (long double)n;
                wc[k] = cosl(a);
                ws[k] = sinl(a);
            }
        };
        ct.src_key = "B" + std::to_string(n) + ":" + std::to_string(M) + ":" + cbs;
        rc = cached_table(pl, "chirp:" + std::to_string(n) + ":" + cbs, [&](DevBuf& b) {
            chirp_ld();
            if (cb == 8) {
                std::vector<float2> c(n);
                for (uint64_t k = 0; k < n; ++k) c[k] = make_float2((float)wc[k], (float)ws[k]);
                return b.upload(c.data(), n * sizeof(float2));
            }
            std::vector<double2> c(n);
            for (uint64_t k = 0; k < n; ++k) c[k] = make_double2((double)wc[k], (double)ws[k]);
            return b.upload(c.data(), n * sizeof(double2));
        }, &ct.chirp);
        if (rc) return rc;
        // the convolution kernel: the chirp and its mirror image, zero in between
        rc = cached_table(pl, "spectrum:" + ct.src_key, [&](DevBuf& b) {
            chirp_ld();
            std::vector<double2> kt(M, make_double2(0, 0));
            kt[0] = make_double2((double)wc[0], (double)ws[0]);
            for (uint64_t k = 1; k < n; ++k) {
                kt[k] = make_double2((double)wc[k], (double)ws[k]);
                kt[M - k] = kt[k];
            }
            return upload_spectrum(b, kt, cb);
        }, &ct.spectrum);
        if (rc) return rc;
    } else if (ps.kind == GS_RADER) {
        const uint64_t Lc = nt - 1, M = ps.L, g = primitive_root(nt), ginv = powmod(g, nt - 2, nt);
        std::vector<uint64_t> gp(Lc);
        std::vector<int> gi(Lc);
        uint64_t cur = 1, curi = 1;
        for (uint64_t i = 0; i < Lc; ++i) {
            gp[i] = cur;
            gi[i] = (int)curi;
            cur = mulmod(cur, g, nt);
            curi = mulmod(curi, ginv, nt);
        }
        ct.src_key = "R" + std::to_string(nt) + ":" + std::to_string(M) + ":" + cbs;
        // gather (M ints) then scatter (M ints)
        const void* maps = nullptr;
        rc = cached_table(pl, "rader:" + std::to_string(nt) + ":" + std::to_string(M), [&](DevBuf& b) {
            std::vector<int> gs(2 * M, -1);
            for (uint64_t i = 0; i < Lc; ++i) gs[i] = gi[i];
            int* scatter = gs.data() + M;
            if (M == Lc) {
                for (uint64_t q = 0; q < Lc; ++q) scatter[q] = (int)gp[q];
            } else {
                // zero-padded linear convolution; outputs q in [L-1, 2L-1) carry the cyclic result
                for (uint64_t q = Lc - 1; q < 2 * Lc - 1; ++q) scatter[q] = (int)gp[q % Lc];
            }
            return b.upload(gs.data(), 2 * M * sizeof(int));
        }, &maps);
        if (rc) return rc;
        ct.gather = static_cast<const int*>(maps);
        ct.scatter = static_cast<const int*>(maps) + M;
        // the convolution kernel w^(g^p), periodically extended for the zero-padded form
        rc = cached_table(pl, "spectrum:" + ct.src_key, [&](DevBuf& b) {
            std::vector<double2> kt(M, make_double2(0, 0));
            for (uint64_t m = 0; m < M; ++m) {
                long double c, sn;
                twiddle_ld(gp[m % Lc], nt, &c, &sn);
                kt[m] = make_double2((double)c, (double)sn);
            }
            return upload_spectrum(b, kt, cb);
        }, &ct.spectrum);
        if (rc) return rc;
        rc = pl->x0buf.alloc(pl->chunk * split_m * cb);
        if (!rc) rc = pl->dcbuf.alloc(pl->chunk * split_m * cb);
        if (rc) return rc;
    }
    // ---- scratch ----
    if (K >= 2) {
        rc = pl->scratch0.alloc(pl->chunk * split_m * ps.L * cb);
        if (!rc && K >= 3) rc = pl->scratch1.alloc(pl->chunk * split_m * ps.L * cb);
        if (rc) return rc;
    }
    const void* split_tw = nullptr;
    if (split_m > 1) {
        // the split pass's output (user element type) and its table w_N^t, t < N
        rc = pl->scratch2.alloc(pl->chunk * n * io_cb);
        if (!rc)
            rc = cached_table(pl, "splittw:" + std::to_string(n) + ":" + std::to_string(io_cb), [&](DevBuf& b) {
                std::vector<unsigned char> t(n * io_cb);
                for (uint64_t k = 0; k < n; ++k) {
                    long double c, sn;
                    twiddle_ld(k, n, &c, &sn);
                    if (io_cb == 8) reinterpret_cast<float2*>(t.data())[k] = make_float2((float)c, (float)sn);
                    else reinterpret_cast<double2*>(t.data())[k] = make_double2((double)c, (double)sn);
                }
                return b.upload(t.data(), t.size());
            }, &split_tw);
        if (rc) return rc;
    }
    const SplitSpec sp{split_m, nt, split_tw};
    rc = build_pipeline(pl, ps, false, local_tabs, tw_hi, tw_lo, tw_shift, ct, sp, pl->fwd);
    if (!rc) rc = build_pipeline(pl, ps, true, local_tabs, tw_hi, tw_lo, tw_shift, ct, sp, pl->inv);
    return rc;
}

// ------------------------------------------------------------------------------------------
// Execution
// ------------------------------------------------------------------------------------------

// Runs the pipeline over transforms [b_begin, b_end) of the batch (in/out are the batch bases).
// offs / ids (uneven batches): transform b of the user buffers starts at element offs[ids[b]]
// instead of b * idist (whole batch in one chunk).
static int run_pipeline(fyg_plan* pl, const std::vector<PassDesc>& pipe, const void* in, void* out,
                        double final_scale_mul, cudaStream_t st, size_t b_begin = 0, size_t b_end = SIZE_MAX,
                        const int64_t* offs = nullptr, const int* ids = nullptr) {
    const int io_cb = pl->dtype == FYG_C32 ? 8 : 16;
    b_end = std::min(b_end, pl->batch);
    for (size_t c0 = b_begin; c0 < b_end; c0 += pl->chunk) {
        const size_t nb = std::min(pl->chunk, b_end - c0);
        for (size_t i = 0; i < pipe.size(); ++i) {
            const PassDesc& d = pipe[i];
            PassParams p = d.p;
            auto resolve = [&](int role) -> void* {
                switch (role) {
                    case ROLE_IN: return (void*)((const char*)in + c0 * pl->idist * io_cb);
                    case ROLE_OUT: return (void*)((char*)out + c0 * pl->odist * io_cb);
                    case ROLE_S0: return pl->scratch0.ptr;
                    case ROLE_S2: return pl->scratch2.ptr;
                    default: return pl->scratch1.ptr;
                }
            };
            p.in = resolve(d.in_role);
            p.out = resolve(d.out_role);
            if (offs) {
                if (d.in_role == ROLE_IN) { p.in = in; p.in_offsets = offs; p.ids = ids; }
                if (d.out_role == ROLE_OUT) { p.out = out; p.out_offsets = offs; p.ids = ids; }
            }
            p.ncols = (int64_t)nb * d.bmul * p.Rr;
            p.x0buf = pl->x0buf.ptr;
            p.dcbuf = pl->dcbuf.ptr;
            if (i + 1 == pipe.size()) {
                if (p.store_mode == ST_SCATTER) p.scale2 *= final_scale_mul;
                else p.scale *= final_scale_mul;
            }
            const unsigned grid = (unsigned)((p.ncols + p.g.C - 1) / p.g.C);
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (pl->profile && &pipe == &pl->fwd) {
                if (pl->prof_pool_used + 2 > pl->prof_pool.size()) {
                    for (int k = 0; k < 64; ++k) {
                        cudaEvent_t ev;
                        if (cudaEventCreate(&ev) != cudaSuccess) return cuda_error(cudaGetLastError(), "event");
                        pl->prof_pool.push_back(ev);
                    }
                }
                e0 = pl->prof_pool[pl->prof_pool_used++];
                e1 = pl->prof_pool[pl->prof_pool_used++];
                cudaEventRecord(e0, st);
            }
            cudaError_t e = launch_pass(d.kv, p, grid, d.threads, d.smem, st, d.tma ? &d.tmap : nullptr);
            if (e != cudaSuccess) return cuda_error(e, "tile pass launch");
            if (e0) {
                cudaEventRecord(e1, st);
                pl->prof_pending.push_back({(int)i, {e0, e1}});
            }
        }
    }
    return FYG_OK;
}

// 1: device memory of device `dev` or managed memory; 0: host memory; -1: device memory of
// another device (its kernels would fault without peer access: rejected)
static int device_ptr_kind(const void* ptr, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (a.type == cudaMemoryTypeManaged) return 1;
    if (a.type == cudaMemoryTypeDevice) return a.device == dev ? 1 : -1;
    return 0;
}

// Host input and output: the batch is cut into chunks; chunk i's host->device copy (copy-in
// stream), its kernels (the caller's stream) and its device->host copy (copy-out stream) are
// ordered by events, so copies in both directions overlap the kernels of neighbouring chunks.
// Returns when the output is in host memory.
// Bytes of a user buffer: the last transform's start plus one transform.
static size_t span_bytes(const fyg_plan* pl, size_t dist) {
    const size_t cb = pl->dtype == FYG_C32 ? 8 : 16;
    return ((pl->batch - 1) * dist + pl->n) * cb;
}

// Copies transforms [b0, b0 + nb) of a user layout (rows of n elements, `dist` apart), leaving
// the gaps between transforms untouched: one 1D copy when the rows are back to back.
static cudaError_t copy_rows(void* dst, const void* src, const fyg_plan* pl, size_t dist, size_t b0, size_t nb,
                             cudaMemcpyKind kind, cudaStream_t st) {
    const size_t cb = pl->dtype == FYG_C32 ? 8 : 16;
    const size_t off = b0 * dist * cb, w = pl->n * cb, pitch = dist * cb;
    char* d = static_cast<char*>(dst) + off;
    const char* s = static_cast<const char*>(src) + off;
    if (pitch == w) return cudaMemcpyAsync(d, s, nb * w, kind, st);
    return cudaMemcpy2DAsync(d, pitch, s, pitch, w, nb, kind, st);
}

static int ensure_staging(fyg_plan* pl) {
    const size_t need = std::max(span_bytes(pl, pl->idist), span_bytes(pl, pl->odist));
    if (pl->stage_in_bytes >= need) return FYG_OK;
    int rc = pl->stage_in.alloc(need);
    if (!rc) rc = pl->stage_out.alloc(need);
    if (rc) return rc;
    pl->stage_in_bytes = need;
    return FYG_OK;
}

// async: return after enqueueing; the output is in host memory once the plan's copy-out stream
// has finished (fyg_plan_join orders it into a caller stream), and the host input is read by the
// copy stream without waiting for earlier work on the caller's stream (the caller has it
// ready), so consecutive calls of different plans pipeline their copies and kernels.  Otherwise
// the copy-in waits for earlier work on the caller's stream and the call returns when the output
// is in host memory.
// Asynchronous calls of one host thread on one device keep their copies in call order: each
// call's first copy-in waits for the previous call's last copy-in, and likewise for copy-outs, so
// the copy engines serve the transforms first in, first out (concurrent copy streams of many
// plans were measured to slow the first transforms and with them the whole pipeline).
// The two events of a (host thread, device) pair live as long as the thread: they are created on
// its first asynchronous call and deliberately not destroyed at thread exit, when the CUDA
// context may already be gone (two events per thread and device).
namespace {
struct CopyChain {
    cudaEvent_t h2d = nullptr, d2h = nullptr;
};
thread_local std::map<int, CopyChain> t_chain;
}  // namespace

static int execute_host_overlapped(fyg_plan* pl, const void* in, void* out, bool inverse, double scale_mul,
                                   cudaStream_t st, bool async) {
    int rc = ensure_staging(pl);
    if (rc) return rc;
    // chunks of about 64 MB, at least 2 and at most 16 (FYG_HOST_CHUNK_MB and FYG_HOST_CHUNKS
    // override the size and the cap), whole transforms, at least one L2 chunk of the plan each.
    // Every copy costs the copy engines a few microseconds of set-up: on the precision sweep's
    // pipelined host calls this measured 8.38 ms per step against 8.6-8.7 ms with 8 chunks per
    // call whatever its size, and 9.3-10.1 ms with 16-32 chunks.
    size_t want = 16, chunk_mb = 64;
    if (const char* e = std::getenv("FYG_HOST_CHUNKS")) want = std::max<size_t>(1, std::strtoull(e, nullptr, 10));
    if (const char* e = std::getenv("FYG_HOST_CHUNK_MB")) chunk_mb = std::min<size_t>(std::strtoull(e, nullptr, 10), 1u << 20);
    if (chunk_mb) {
        const size_t bytes = pl->n * pl->batch * (pl->dtype == FYG_C32 ? 8 : 16);
        want = std::min(want, std::max<size_t>(2, (bytes + (chunk_mb << 20) - 1) / (chunk_mb << 20)));
    }
    size_t cb = std::max<size_t>((pl->batch + want - 1) / want, 1);
    if (pl->chunk < pl->batch) cb = std::max(cb, pl->chunk) / pl->chunk * pl->chunk;
    const size_t nch = (pl->batch + cb - 1) / cb;
    if (!pl->s_h2d) {
        cudaError_t e = cudaStreamCreateWithFlags(&pl->s_h2d, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&pl->s_d2h, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_error(e, "staging streams");
    }
    while (pl->stage_ev.size() < 2 * nch + 1) {
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_error(e, "staging events");
        pl->stage_ev.push_back(ev);
    }
    if (!pl->ev_in_free) {
        cudaError_t e = cudaEventCreateWithFlags(&pl->ev_in_free, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->ev_out_free, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_error(e, "staging events");
    }
    cudaEvent_t start = pl->stage_ev[2 * nch];
    auto chk = [&](cudaError_t e, const char* what) { return e == cudaSuccess ? FYG_OK : cuda_error(e, what); };
    // the staging buffers of this plan: its previous call's kernels may still read stage_in and
    // its previous copy-out may still read stage_out (waits on never-recorded events are no-ops)
    rc = chk(cudaStreamWaitEvent(pl->s_h2d, pl->ev_in_free, 0), "wait");
    if (!rc) rc = chk(cudaStreamWaitEvent(st, pl->ev_out_free, 0), "wait");
    if (!async && !rc) {
        // ordered after earlier work on the caller's stream
        rc = chk(cudaEventRecord(start, st), "event");
        if (!rc) rc = chk(cudaStreamWaitEvent(pl->s_h2d, start, 0), "wait");
    }
    CopyChain* chain = nullptr;
    if (async && !rc) {
        chain = &t_chain[pl->device];
        if (!chain->h2d) {
            cudaError_t e = cudaEventCreateWithFlags(&chain->h2d, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&chain->d2h, cudaEventDisableTiming);
            if (e != cudaSuccess) return cuda_error(e, "copy chain events");
        }
        rc = chk(cudaStreamWaitEvent(pl->s_h2d, chain->h2d, 0), "wait");
        if (!rc) rc = chk(cudaStreamWaitEvent(pl->s_d2h, chain->d2h, 0), "wait");
    }
    const char* hin = static_cast<const char*>(in);
    char* hout = static_cast<char*>(out);
    char* sin = static_cast<char*>(pl->stage_in.ptr);
    char* sout = static_cast<char*>(pl->stage_out.ptr);
    for (size_t i = 0; i < nch && !rc; ++i) {
        const size_t b0 = i * cb, nb = std::min(cb, pl->batch - b0);
        cudaEvent_t ev_in = pl->stage_ev[2 * i], ev_done = pl->stage_ev[2 * i + 1];
        rc = chk(copy_rows(sin, hin, pl, pl->idist, b0, nb, cudaMemcpyHostToDevice, pl->s_h2d), "host->device staging");
        if (!rc) rc = chk(cudaEventRecord(ev_in, pl->s_h2d), "event");
        if (!rc) rc = chk(cudaStreamWaitEvent(st, ev_in, 0), "wait");
        if (!rc) rc = run_pipeline(pl, inverse ? pl->inv : pl->fwd, sin, sout, scale_mul, st, b0, b0 + nb);
        if (!rc) rc = chk(cudaEventRecord(ev_done, st), "event");
        if (!rc) rc = chk(cudaStreamWaitEvent(pl->s_d2h, ev_done, 0), "wait");
        if (!rc)
            rc = chk(copy_rows(hout, sout, pl, pl->odist, b0, nb, cudaMemcpyDeviceToHost, pl->s_d2h),
                     "device->host staging");
    }
    if (!rc) rc = chk(cudaEventRecord(pl->ev_in_free, st), "event");
    if (!rc) rc = chk(cudaEventRecord(pl->ev_out_free, pl->s_d2h), "event");
    if (chain && !rc) {
        rc = chk(cudaEventRecord(chain->h2d, pl->s_h2d), "event");
        if (!rc) rc = chk(cudaEventRecord(chain->d2h, pl->s_d2h), "event");
    }
    // async: the copy-outs complete on the plan's copy-out stream (fyg_plan_join or a device
    // synchronize waits for them); the caller's stream runs on, so the next call's kernels are
    // not held behind this call's copies
    if (async) return rc;
    // drain both copy streams before returning (the host buffers are the caller's)
    const cudaError_t e1 = cudaStreamSynchronize(pl->s_h2d);
    const cudaError_t e2 = cudaStreamSynchronize(pl->s_d2h);
    if (!rc) rc = chk(e1, "stream synchronize");
    if (!rc) rc = chk(e2, "stream synchronize");
    return rc;
}

static int execute_dir(fyg_plan* pl, const void* in, void* out, bool inverse, double scale_mul, cudaStream_t st,
                       bool async = false) {
    if (!pl) return set_error(FYG_ERR_NULL_PTR, "null plan");
    if (!in || !out) return set_error(FYG_ERR_NULL_PTR, "null buffer");
    const int io_cb = pl->dtype == FYG_C32 ? 8 : 16;
    if (((uintptr_t)in % io_cb) || ((uintptr_t)out % io_cb))
        return set_error(FYG_ERR_MISALIGNED, "buffers must be aligned to the complex element size");
    if (in == out && pl->idist != pl->odist)
        return set_error(FYG_ERR_INVALID_ARG, "in-place execution needs equal input and output distances");
    // the plan's device for the duration of the call; the caller's device again on every return
    struct DeviceScope {
        int prev = 0, dev;
        explicit DeviceScope(int d) : dev(d) {
            cudaGetDevice(&prev);
            if (prev != dev) cudaSetDevice(dev);
        }
        ~DeviceScope() {
            if (prev != dev) cudaSetDevice(prev);
        }
    } scope(pl->device);
    const size_t bytes = pl->n * pl->batch * io_cb;
    const int kin = device_ptr_kind(in, pl->device), kout = device_ptr_kind(out, pl->device);
    if (kin < 0 || kout < 0)
        return set_error(FYG_ERR_INVALID_ARG, "buffers on another device than the plan's");
    const bool din = kin > 0, dout = kout > 0;
    if (!din && !dout && pl->strategy != GS_COPY && pl->batch >= 2 && bytes >= (8u << 20))
        return execute_host_overlapped(pl, in, out, inverse, scale_mul, st, async);
    const void* din_p = in;
    void* dout_p = out;
    int rc = FYG_OK;
    if (!din || !dout) {
        rc = ensure_staging(pl);
        if (rc) return rc;
        if (!din) {
            cudaError_t e = copy_rows(pl->stage_in.ptr, in, pl, pl->idist, 0, pl->batch, cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) return cuda_error(e, "host->device staging");
            din_p = pl->stage_in.ptr;
        }
        if (!dout) dout_p = pl->stage_out.ptr;
    }
    if (pl->strategy == GS_COPY) {
        cudaError_t e = launch_scale_copy(din_p, dout_p, pl->batch, pl->dtype, scale_mul, 0, st);
        if (e != cudaSuccess) return cuda_error(e, "copy");
    } else {
        rc = run_pipeline(pl, inverse ? pl->inv : pl->fwd, din_p, dout_p, scale_mul, st);
        if (rc) return rc;
    }
    if (!dout) {
        cudaError_t e = copy_rows(out, dout_p, pl, pl->odist, 0, pl->batch, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return cuda_error(e, "device->host staging");
    }
    if ((!din || !dout) && !async) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_error(e, "stream synchronize");
    }
    return FYG_OK;
}

static int gpu_fft_f64(size_t n, const std::vector<double2>& h, std::vector<double2>& H) {
    fyg_plan* sub = nullptr;
    const uint64_t keep_r = t_max_pass_r, keep_m = t_conv_len;
    const int keep_order = t_order;
    const size_t keep_idist = t_idist, keep_odist = t_odist;
    t_order = 0;
    t_idist = t_odist = 0;
    const int keep_cap = t_radix_cap, keep_cols = t_cols, keep_threads = t_threads;
    t_max_pass_r = t_conv_len = 0;
    t_radix_cap = t_cols = t_threads = 0;
    int rc = fyg_plan_create(n, FYG_C64, 1, 0, &sub);
    t_max_pass_r = keep_r;
    t_conv_len = keep_m;
    t_order = keep_order;
    t_idist = keep_idist;
    t_odist = keep_odist;
    t_radix_cap = keep_cap;
    t_cols = keep_cols;
    t_threads = keep_threads;
    if (rc) return rc;
    DevBuf a, b;
    rc = a.upload(h.data(), n * sizeof(double2));
    if (!rc) rc = b.alloc(n * sizeof(double2));
    if (!rc) rc = execute_dir(sub, a.ptr, b.ptr, false, 1.0, 0);
    if (!rc) {
        H.resize(n);
        cudaError_t e = cudaMemcpy(H.data(), b.ptr, n * sizeof(double2), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_error(e, "spectrum download");
    }
    fyg_plan_destroy(sub);
    return rc;
}

}  // namespace fyg

// ------------------------------------------------------------------------------------------
// C ABI (plans)
// ------------------------------------------------------------------------------------------

using namespace fyg;

fyg_plan::~fyg_plan() {
    // pending asynchronous host executions still use the staging buffers and copy streams
    if (s_h2d) cudaStreamSynchronize(s_h2d);
    if (s_d2h) cudaStreamSynchronize(s_d2h);
    if (ev_in_free) cudaEventSynchronize(ev_in_free);
    if (ev_in_free) cudaEventDestroy(ev_in_free);
    if (ev_out_free) cudaEventDestroy(ev_out_free);
    for (cudaEvent_t e : prof_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : stage_ev) cudaEventDestroy(e);
    if (s_h2d) cudaStreamDestroy(s_h2d);
    if (s_d2h) cudaStreamDestroy(s_d2h);
}

namespace fyg {
// Enqueues a plan's whole batch on `st` with its user transforms at packed offsets (device
// tables offs[ids[b]]); used by the branch form of uneven batches.
int run_plan_offsets(fyg_plan* pl, const void* in, void* out, const int64_t* offs, const int* ids, int direction,
                     cudaStream_t st) {
    if (pl->chunk != pl->batch) return set_error(FYG_ERR_UNSUPPORTED, "offset execution needs one chunk");
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != pl->device) cudaSetDevice(pl->device);
    const int rc = run_pipeline(pl, direction == FYG_INVERSE ? pl->inv : pl->fwd, in, out, 1.0, st, 0, SIZE_MAX,
                                offs, ids);
    if (dev != pl->device) cudaSetDevice(dev);
    return rc;
}

void set_plan_layout(size_t idist, size_t odist) {
    t_idist = idist;
    t_odist = odist;
}

void set_batch_tile_options(int radix_cap, size_t single_cap_bytes) {
    t_batch_radix_cap = radix_cap;
    t_batch_single_cap = single_cap_bytes;
}

// plan creation with explicit schedule options (0 = default); used by the autotuner
int plan_create_opts(size_t n, int dtype, size_t batch, int flags, uint64_t max_pass_radix, uint64_t conv_length,
                     int cols, int order, int threads, fyg_plan** out) {
    t_max_pass_r = max_pass_radix;
    t_conv_len = conv_length;
    t_cols = cols;
    t_order = order;
    t_threads = threads;
    const int rc = fyg_plan_create(n, dtype, batch, flags & ~FYG_FLAG_AUTOTUNED, out);
    t_max_pass_r = 0;
    t_conv_len = 0;
    t_cols = 0;
    t_order = 0;
    t_threads = 0;
    return rc;
}
}  // namespace fyg

extern "C" {

int fyg_plan_create_layout(size_t n, int dtype, size_t batch, size_t idist, size_t odist, int flags, fyg_plan** out) {
    clear_error();
    if (idist && idist < n) return set_error(FYG_ERR_INVALID_ARG, "idist must be 0 or >= n");
    if (odist && odist < n) return set_error(FYG_ERR_INVALID_ARG, "odist must be 0 or >= n");
    if (n == 1 && ((idist && idist != 1) || (odist && odist != 1)))
        return set_error(FYG_ERR_UNSUPPORTED, "strided layouts need n >= 2");
    set_plan_layout(idist, odist);
    const int rc = fyg_plan_create(n, dtype, batch, flags, out);
    set_plan_layout(0, 0);
    return rc;
}

int fyg_plan_create_ex(size_t n, int dtype, size_t batch, int flags, size_t max_pass_radix, size_t conv_length,
                       fyg_plan** out) {
    return plan_create_opts(n, dtype, batch, flags & ~FYG_FLAG_AUTOTUNED, max_pass_radix, conv_length, 0, 0, 0, out);
}


int fyg_plan_create(size_t n, int dtype, size_t batch, int flags, fyg_plan** out) {
    clear_error();
    if (flags & FYG_FLAG_AUTOTUNED) {
        TuneChoice tc;
        if (tune_lookup(n, dtype, &tc))
            return plan_create_opts(n, dtype, batch, flags | (tc.wide ? FYG_FLAG_WIDE_TILES : 0), tc.max_pass_radix,
                                    tc.conv_length, tc.cols, tc.order, tc.threads, out);
        flags &= ~FYG_FLAG_AUTOTUNED;
    }
    if (!out) return set_error(FYG_ERR_NULL_PTR, "out is null");
    *out = nullptr;
    if (n < 1) return set_error(FYG_ERR_INVALID_LENGTH, "length must be >= 1");
    if (batch < 1) return set_error(FYG_ERR_INVALID_ARG, "batch must be >= 1");
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "dtype must be FYG_C32 or FYG_C64");
    if (n >= (1ull << 31)) return set_error(FYG_ERR_INVALID_LENGTH, "length must be < 2^31");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    e = ensure_device_constants();
    if (e != cudaSuccess) return cuda_error(e, "codelet constants");
    auto* pl = new fyg_plan();
    pl->n = n;
    pl->batch = batch;
    pl->idist = t_idist ? t_idist : n;
    pl->odist = t_odist ? t_odist : n;
    pl->dtype = dtype;
    pl->flags = flags;
    pl->device = dev;
    t_radix_cap = (flags & FYG_FLAG_SMALL_TILES) ? (t_batch_radix_cap ? t_batch_radix_cap : 16) : 0;
    int rc = make_plan(pl);
    t_radix_cap = 0;
    if (rc) {
        delete pl;
        return rc;
    }
    *out = pl;
    return FYG_OK;
}

int fyg_plan_destroy(fyg_plan* plan) {
    delete plan;
    return FYG_OK;
}

int fyg_plan_launches(const fyg_plan* plan, int* launches) {
    if (!plan || !launches) return set_error(FYG_ERR_NULL_PTR, "null argument");
    const size_t chunks = (plan->batch + plan->chunk - 1) / plan->chunk;
    *launches = plan->strategy == GS_COPY ? 1 : (int)(plan->fwd.size() * chunks);
    return FYG_OK;
}

int fyg_plan_describe(const fyg_plan* plan, char* buf, size_t len) {
    if (!plan || !buf || len == 0) return set_error(FYG_ERR_NULL_PTR, "null argument");
    static const char* kLoad[] = {"plain", "chirp", "gather"};
    static const char* kStore[] = {"plain", "chirp", "scatter"};
    std::string s;
    for (size_t i = 0; i < plan->fwd.size(); ++i) {
        const PassDesc& d = plan->fwd[i];
        char line[256];
        std::snprintf(line, sizeof(line),
                      "pass %zu: kernel=%s R=%d C=%d threads=%d smem=%zu Ns=%d Ns_out=%d load=%s%s store=%s%s\n", i,
                      d.kv == KV_FAST ? "fast" : (d.kv == KV_SPLIT_F32 || d.kv == KV_SPLIT_F64) ? "split" : "generic", d.p.g.R, d.p.g.C, d.threads, d.smem, d.p.Ns, d.p.Ns_out,
                      kLoad[d.p.load_mode], d.p.Ns > 1 ? "+twiddle" : "", kStore[d.p.store_mode],
                      d.p.mid ? " mid" : "");
        s += line;
    }
    if (s.size() + 1 > len) return set_error(FYG_ERR_INVALID_ARG, "description buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return FYG_OK;
}

int fyg_plan_profile(fyg_plan* plan, int enable) {
    if (!plan) return set_error(FYG_ERR_NULL_PTR, "null plan");
    plan->profile = enable != 0;
    plan->prof_ms.assign(plan->fwd.size(), 0.0);
    plan->prof_launches.assign(plan->fwd.size(), 0);
    plan->prof_pending.clear();
    plan->prof_pool_used = 0;
    return FYG_OK;
}

int fyg_plan_profile_read(fyg_plan* plan, double* total_ms, int64_t* launches, int64_t* bytes_per_launch,
                          int max_passes, int* n_passes) {
    if (!plan) return set_error(FYG_ERR_NULL_PTR, "null plan");
    const int np = (int)plan->fwd.size();
    if (plan->prof_ms.size() != (size_t)np) {
        plan->prof_ms.assign(np, 0.0);
        plan->prof_launches.assign(np, 0);
    }
    for (auto& pe : plan->prof_pending) {
        cudaError_t e = cudaEventSynchronize(pe.second.second);
        if (e != cudaSuccess) return cuda_error(e, "profile event");
        float ms = 0;
        cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
        plan->prof_ms[pe.first] += ms;
        plan->prof_launches[pe.first] += 1;
    }
    plan->prof_pending.clear();
    plan->prof_pool_used = 0;
    for (int i = 0; i < np && i < max_passes; ++i) {
        const PassDesc& d = plan->fwd[i];
        // elements one launch reads and writes: a full sweep of the chunk's transforms, counted
        // at the length actually stored on each side (N for user buffers, L for scratch)
        const int64_t nb = (int64_t)plan->chunk * d.bmul;
        if (total_ms) total_ms[i] = plan->prof_ms[i];
        if (launches) launches[i] = plan->prof_launches[i];
        if (bytes_per_launch) bytes_per_launch[i] = nb * (d.in_len * d.in_elem_bytes + d.out_len * d.out_elem_bytes);
    }
    if (n_passes) *n_passes = np;
    return FYG_OK;
}

int fyg_execute(fyg_plan* plan, const void* in, void* out, int direction, void* stream) {
    clear_error();
    if (direction != FYG_FORWARD && direction != FYG_INVERSE)
        return set_error(FYG_ERR_INVALID_ARG, "direction must be FYG_FORWARD or FYG_INVERSE");
    return execute_dir(plan, in, out, direction == FYG_INVERSE, 1.0, (cudaStream_t)stream);
}

int fyg_execute_async(fyg_plan* plan, const void* in, void* out, int direction, void* stream) {
    clear_error();
    if (direction != FYG_FORWARD && direction != FYG_INVERSE)
        return set_error(FYG_ERR_INVALID_ARG, "direction must be FYG_FORWARD or FYG_INVERSE");
    return execute_dir(plan, in, out, direction == FYG_INVERSE, 1.0, (cudaStream_t)stream, true);
}

int fyg_plan_join(fyg_plan* plan, void* stream) {
    if (!plan) return set_error(FYG_ERR_NULL_PTR, "null plan");
    if (!plan->ev_out_free) return FYG_OK;   // no asynchronous host execution yet
    const cudaError_t e = cudaStreamWaitEvent((cudaStream_t)stream, plan->ev_out_free, 0);
    return e == cudaSuccess ? FYG_OK : cuda_error(e, "join");
}

int fyg_execute_adjoint(fyg_plan* plan, const void* g, void* out, double scale, void* stream) {
    clear_error();
    if (!plan) return set_error(FYG_ERR_NULL_PTR, "null plan");
    // F^H g = N * IFFT(g): the inverse pipeline with its 1/N replaced by `scale`
    return execute_dir(plan, g, out, true, scale * (double)plan->n, (cudaStream_t)stream);
}

int fyg_plan_cache_stats(size_t* entries, size_t* bytes, uint64_t* hits, uint64_t* misses) {
    TableCache& tc = table_cache();
    std::lock_guard<std::mutex> lk(tc.mu);
    size_t b = 0;
    for (auto& kv : tc.map) b += kv.second->bytes;
    if (entries) *entries = tc.map.size();
    if (bytes) *bytes = b;
    if (hits) *hits = tc.hits;
    if (misses) *misses = tc.misses;
    return FYG_OK;
}

int fyg_plan_cache_clear(void) {
    TableCache& tc = table_cache();
    std::lock_guard<std::mutex> lk(tc.mu);
    for (auto it = tc.map.begin(); it != tc.map.end();) {
        if (it->second.use_count() == 1) it = tc.map.erase(it);   // no live plan holds it
        else ++it;
    }
    return FYG_OK;
}

int fyg_plan_status(fyg_plan* plan, void* stream, int* status) {
    if (!plan || !status) return set_error(FYG_ERR_NULL_PTR, "null argument");
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != plan->device) cudaSetDevice(plan->device);
    int word = 0;
    cudaError_t e = cudaMemcpyAsync(&word, plan->errword.ptr, sizeof(int), cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(plan->errword.ptr, 0, sizeof(int), (cudaStream_t)stream);
    if (dev != plan->device) cudaSetDevice(dev);
    if (e != cudaSuccess) return cuda_error(e, "plan status");
    *status = word;
    return FYG_OK;
}

int fyg_strategy(size_t n) { return ref_strategy(n); }

int fyg_gpu_strategy(size_t n) {
    if (n < 2) return -1;
    if (is_smooth(n, 7)) return ref_directly_supported(n) ? FYG_STRATEGY_KERNEL_DIRECT : FYG_STRATEGY_MIX_RADIX;
    if (is_smooth(n, 13)) return FYG_STRATEGY_MIX_RADIX;
    if (is_prime(n) && (is_smooth(n - 1, 13) || 2 * n - 3 <= 78125)) return FYG_STRATEGY_RADER;
    if (split_factor(n)) return FYG_STRATEGY_RADER;   // m Rader transforms after the split pass
    return FYG_STRATEGY_BLUESTEIN;
}

int fyg_plan_schedule(size_t n, int dtype, int flags, int* strategy, size_t* conv_length, int* split_m,
                      int* pass_radices, int max_passes, int* npasses) {
    clear_error();
    if (n < 1) return set_error(FYG_ERR_INVALID_LENGTH, "length must be >= 1");
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "dtype must be FYG_C32 or FYG_C64");
    if (n >= (1ull << 31)) return set_error(FYG_ERR_INVALID_LENGTH, "length must be < 2^31");
    // a host-only plan object: plan_spec allocates nothing and makes no CUDA call
    auto pl = std::make_unique<fyg_plan>();
    pl->n = n;
    pl->batch = 1;
    pl->idist = pl->odist = n;
    pl->dtype = dtype;
    pl->flags = flags & ~FYG_FLAG_AUTOTUNED;
    int st = GS_COPY;
    size_t L = 1;
    uint64_t m = 1;
    std::vector<int> rad;
    if (n >= 2) {
        PipeSpec ps;
        uint64_t nt = n;
        t_radix_cap = (pl->flags & FYG_FLAG_SMALL_TILES) ? (t_batch_radix_cap ? t_batch_radix_cap : 16) : 0;
        const int rc = plan_spec(pl.get(), ps, nt, m);
        t_radix_cap = 0;
        if (rc) return rc;
        st = pl->strategy;
        L = ps.L;
        rad = ps.prad;
    }
    if (strategy) *strategy = st;
    if (conv_length) *conv_length = L;
    if (split_m) *split_m = (int)m;
    if (pass_radices)
        for (int i = 0; i < (int)rad.size() && i < max_passes; ++i) pass_radices[i] = rad[i];
    if (npasses) *npasses = (int)rad.size();
    return FYG_OK;
}

int fyg_plan_info(const fyg_plan* plan, size_t* conv_length, int* passes, int* strategy) {
    if (!plan) return set_error(FYG_ERR_NULL_PTR, "null plan");
    if (conv_length) *conv_length = plan->L;
    if (passes) *passes = (int)plan->fwd.size();
    if (strategy) *strategy = plan->strategy;
    return FYG_OK;
}

const char* fyg_last_error_string(void) { return last_error(); }

int fyg_fill_random(uint64_t seed, int dist, int dtype, size_t n_complex, void* out) {
    return fyg_fill_random_at(seed, dist, dtype, 0, n_complex, out);
}

int fyg_fill_random_at(uint64_t seed, int dist, int dtype, size_t first, size_t n_complex, void* out) {
    if (!out && n_complex) return set_error(FYG_ERR_NULL_PTR, "null buffer");
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "bad dtype");
    fill_random_host(seed, dist, dtype, first, n_complex, out);
    return FYG_OK;
}

int fyg_fill_random_device(uint64_t seed, int dist, int dtype, size_t n_complex, void* out, void* stream) {
    return fyg_fill_random_device_at(seed, dist, dtype, 0, n_complex, out, stream);
}

int fyg_fill_random_device_at(uint64_t seed, int dist, int dtype, size_t first, size_t n_complex, void* out,
                              void* stream) {
    if (!out && n_complex) return set_error(FYG_ERR_NULL_PTR, "null buffer");
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "bad dtype");
    cudaError_t e = launch_fill_random(seed, dist, dtype, first, n_complex, out, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_error(e, "fill_random_device");
    return FYG_OK;
}

const char* fyg_version(void) { return "fyfft-gb300 0.1 (sm_103a)"; }

}  // extern "C"
