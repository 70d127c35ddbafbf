// fyg_host.h -- host-side plan structures of the GB300 FFT library.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <memory>
#include <map>
#include <string>
#include <vector>

#include "../../include/fygpu.h"
#include "fyg_internal.h"

struct fyg_plan;

namespace fyg {

int set_error(int code, const std::string& msg);
void clear_error();
const char* last_error();
int cuda_error(cudaError_t e, const char* what);
void fill_random_host(uint64_t seed, int dist, int dtype, size_t first, size_t n, void* out);

FastDiv make_fastdiv(uint32_t d);

// Planner building blocks (fyg_plan.cu), shared with the allocation-free entry point.
bool is_smooth(uint64_t n, uint64_t b);
std::vector<int> radices_for(int R, int cb = 8);
bool tile_fits(int cb, int R, int C, bool colmajor);
int multi_C(int cb, int R);
bool split_passes(uint64_t L, int cb, bool conv, std::vector<int>& out);
void fill_geom(TileGeom& g, int R, int C, bool colmajor, const std::vector<int>& rad);
size_t smem_for(int cb, int R, int C, bool colmajor);
int tile_class(int cb, int rmax);
int pick_variant(int compute_cb, int tin_cb, int tout_cb, int cls);
int threads_for(int R, int C, int maxt);
int single_pass_cols(int cb, int L, size_t batch, int requested);
int single_pass_threads(int L, int C, const std::vector<int>& rad, int requested);
bool single_pass_fits(int cb, uint64_t n, size_t cap);
void twiddle_ld(uint64_t t, uint64_t n, long double* c, long double* s);
std::vector<unsigned char> host_local_table(int R, int cb);

// Autotuner (fyg_autotune.cu): measured schedule choice per (dtype, length), cached in JSON.
struct TuneChoice {
    uint64_t max_pass_radix = 0, conv_length = 0;
    int cols = 0;
    int order = 0;       // 1: reversed pass order (the fused mid pass takes the other radix)
    int threads = 0;     // single-pass thread policy (single_pass_threads)
    int wide = 0;        // 1: FYG_FLAG_WIDE_TILES
    double ms = 0;
};
bool tune_lookup(size_t n, int dtype, TuneChoice* out);
// Autotune cache entries by key (the batch autotuner stores its choice under "batch..." keys).
bool tune_lookup_key(const std::string& key, TuneChoice* out);
int tune_store_key(const std::string& key, const TuneChoice& choice, const char* cache_path);
// Options of uneven-batch group plans for plans created next on this thread (0 = defaults).
void set_batch_tile_options(int radix_cap, size_t single_cap_bytes);
int plan_create_opts(size_t n, int dtype, size_t batch, int flags, uint64_t max_pass_radix, uint64_t conv_length,
                     int cols, int order, int threads, fyg_plan** out);
// A plan's whole batch with its user transforms at element offsets offs[ids[b]] (device tables).
int run_plan_offsets(fyg_plan* pl, const void* in, void* out, const int64_t* offs, const int* ids, int direction,
                     cudaStream_t st);
// Layout of the user buffers of plans created next on this thread (0 = contiguous).
void set_plan_layout(size_t idist, size_t odist);
void host_two_level(uint64_t L, int cb, std::vector<unsigned char>& hi, std::vector<unsigned char>& lo, int* shift);

// GPU-side strategy of a plan (what actually runs).
enum GpuStrategy : int {
    GS_SINGLE = 0,      // one tile pass (whole transform in one CTA)
    GS_MULTI = 1,       // multi-pass Stockham (four-step generalised), fused inter-pass twiddles
    GS_RADER = 2,       // Rader: cyclic (or zero-padded) convolution of length N-1
    GS_BLUESTEIN = 3,   // Bluestein chirp-z convolution
    GS_COPY = 4,        // n == 1
    GS_SPLIT = 5,       // N = m p: length-m DFTs and twiddles, then m Rader transforms of length p
};

// Owned device allocation.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf();
    int alloc(size_t n);      // returns FYG_OK / FYG_ERR_ALLOC
    int upload(const void* host, size_t n);
};

// Buffer roles a pass reads from / writes to.
// ROLE_S2: the split strategy's buffer between its first pass and the Rader passes.
enum Role : int { ROLE_IN = 0, ROLE_OUT = 1, ROLE_S0 = 2, ROLE_S1 = 3, ROLE_S2 = 4 };

struct PassDesc {
    PassParams p;          // in/out/ncols/x0buf/dcbuf filled at execution
    int in_role, out_role;
    int kv;                // kernel variant
    int threads;
    size_t smem;
    int64_t in_elem_bytes, out_elem_bytes;
    int64_t in_len = 0, out_len = 0;   // elements per transform read / written
    int bmul = 1;          // transforms of this pass per user transform (m for the split's Rader passes)
    bool tma = false;      // register-resident pass whose input arrives by TMA tile loads
    CUtensorMap tmap;      // (FYG_FLAG_TMA_LOADS; the input is a scratch buffer of the plan)
};

// Process-wide cache of read-only plan tables (twiddles, chirps, Rader index maps, convolution
// spectra, thread-order tables), keyed by device and content.  A plan holds shared references
// to the tables it uses, so plans of the same length (and the autotuner's candidates) build
// each table once.  Returns the table's device pointer in *out; `build` fills a fresh buffer
// on a miss (with the plan's device current).
int cached_table(fyg_plan* pl, const std::string& key, const std::function<int(DevBuf&)>& build, const void** out);

}  // namespace fyg

// The opaque plan type of the C ABI.
struct fyg_plan {
    size_t n = 0, batch = 0;
    size_t idist = 0, odist = 0;   // elements between the starts of consecutive user transforms
    int dtype = FYG_C32;
    int flags = 0;
    int device = 0;
    int strategy = 0;         // fyg::GpuStrategy
    int conv_fp64 = 0;        // Rader/Bluestein convolution runs in FP64
    size_t L = 0;             // algorithm length: n (plain) or the convolution length
    size_t chunk = 1;         // transforms per chunk (L2-resident scratch)
    int compute_bytes = 8;    // bytes of one compute complex
    std::vector<fyg::PassDesc> fwd, inv;
    // device tables
    std::vector<std::shared_ptr<fyg::DevBuf>> tables;   // read-only, shared through the table cache
    fyg::DevBuf scratch0, scratch1, scratch2, x0buf, dcbuf, errword;
    size_t split_m = 1;       // GS_SPLIT: N = split_m * p
    fyg::DevBuf stage_in, stage_out;   // staging for host pointers
    size_t stage_in_bytes = 0;
    // host-pointer execution: copy-in and copy-out streams and per-chunk events, so that the
    // copies of one batch chunk overlap the kernels of the previous one
    cudaStream_t s_h2d = nullptr, s_d2h = nullptr;
    std::vector<cudaEvent_t> stage_ev;
    // recorded when this plan's last call finished reading stage_in (its kernels) and stage_out
    // (its copy-out): the next call's copy-in and kernels wait on them
    cudaEvent_t ev_in_free = nullptr, ev_out_free = nullptr;
    // instrumentation: event pairs per launch, accumulated per forward pass
    bool profile = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_pending;
    std::vector<double> prof_ms;
    std::vector<int64_t> prof_launches;
    std::vector<cudaEvent_t> prof_pool;
    size_t prof_pool_used = 0;
    ~fyg_plan();
};
