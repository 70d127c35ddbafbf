// fyg_noalloc.cu -- an entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc.  A host application that owns every byte of device
// memory (it sizes one pool at start-up and hands each plugin only its input and output
// buffers) cannot let a plugin allocate behind its back: the allocation may fail at an
// unpredictable point or push the application over its memory budget.  A loop with a latency
// budget cannot take the device-wide synchronization that cudaMalloc / cudaFree may cause.
// fyg_execute_noalloc serves them with the multi-pass tile-pass kernel (the kernel that needs
// scratch for its pass intermediates): the scratch and the twiddle tables live in one
// file-scope __device__ array of fixed size that every GPU loading this library holds until the
// process exits.
//
// Limits: plain (13-smooth) lengths only; pass intermediates of at most kNoAllocScratchBytes
// (n * batch * element size, twice that for three or more passes) and twiddle tables of at most
// kNoAllocTableBytes; device pointers of the current device only.  The first call on a device
// sets up: it looks up the array's device address with cudaGetSymbolAddress and copies this
// file's codelet constants (both synchronous host calls, no allocation), so that first call
// should come before any stream capture.  The twiddle tables
// are computed on the device by a small kernel into the array (no host copy) whenever the
// length or the element type differs from the previous call's on that device.  All calls
// share the array and it keeps the last call's contents: two calls that overlap on the GPU
// (e.g. on different streams without ordering) race.  The intermediates need no clearing
// (every pass writes all of its output before the next pass reads it).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "fyg_host.h"
#include "fyg_k_variant.cuh"

namespace fyg {

constexpr size_t kNoAllocTableBytes = 4u << 20;     // twiddle tables of one call
constexpr size_t kNoAllocScratchBytes = 16u << 20;  // pass intermediates of one call
constexpr size_t kNoAllocBytes = kNoAllocTableBytes + kNoAllocScratchBytes;

static __device__ __align__(256) unsigned char g_noalloc[kNoAllocBytes];

namespace {

constexpr int kMaxDev = 64;
std::mutex g_mu;
unsigned char* g_base[kMaxDev] = {};   // device address of g_noalloc, per device
uint64_t g_tab_key[kMaxDev] = {};      // (n, element size) whose tables the array holds, 0 = none

constexpr int kMaxPasses = 6;

// Where one call's tables sit in the table region (byte offsets) and what they hold.
struct TableLayout {
    int passes;
    int R[kMaxPasses];            // pass radix of each local table (distinct radices only)
    size_t local_off[kMaxPasses];
    int nlocal;
    int local_of_pass[kMaxPasses];
    uint64_t L;                   // transform length of the two-level table (0: none)
    int shift;                    // 2^shift ~ sqrt(L)
    uint64_t nhi, nlo;
    size_t hi_off, lo_off;
    int cb;                       // 8: FP32 tables, 16: FP64
    size_t bytes;
};

// exp(-2 pi i e / m) from the FP64 sincospi of the exactly reduced exponent
__device__ __forceinline__ void tw_fp64(uint64_t e, uint64_t m, double* c, double* s) {
    double sn, cs;
    sincospi(2.0 * (double)(e % m) / (double)m, &sn, &cs);
    *c = cs;
    *s = -sn;
}

// Every entry of the call's tables, grid-stride: the local tables w_R^t, then the two-level
// table of w_L (hi[i] = w^(i 2^shift), lo[j] = w^j); FP32 two-level entries are (hi, lo) float
// pairs of each component, FP64 entries plain.
__global__ void k_noalloc_tables(unsigned char* tab, TableLayout t) {
    uint64_t total = t.nhi + t.nlo;
    for (int k = 0; k < t.nlocal; ++k) total += (uint64_t)t.R[k];
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t rem = idx;
        int k = 0;
        while (k < t.nlocal && rem >= (uint64_t)t.R[k]) rem -= (uint64_t)t.R[k++];
        double c, s;
        if (k < t.nlocal) {
            tw_fp64(rem, (uint64_t)t.R[k], &c, &s);
            unsigned char* dst = tab + t.local_off[k];
            if (t.cb == 8) reinterpret_cast<float2*>(dst)[rem] = make_float2((float)c, (float)s);
            else reinterpret_cast<double2*>(dst)[rem] = make_double2(c, s);
            continue;
        }
        const bool hi = rem < t.nhi;
        const uint64_t i = hi ? rem : rem - t.nhi;
        tw_fp64(hi ? i << t.shift : i, t.L, &c, &s);
        unsigned char* dst = tab + (hi ? t.hi_off : t.lo_off);
        if (t.cb == 8) {
            const float ch = (float)c, sh = (float)s;
            reinterpret_cast<float4*>(dst)[i] = make_float4(ch, sh, (float)(c - (double)ch), (float)(s - (double)sh));
        } else {
            reinterpret_cast<double2*>(dst)[i] = make_double2(c, s);
        }
    }
}

// Once per device, with that device current: the array's device address and this file's
// codelet constants.  No allocation.
int noalloc_setup(unsigned char** base) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev >= kMaxDev) return set_error(FYG_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(scratch)");
        CodeletConsts<float> kf;
        CodeletConsts<double> kd;
        codelet_consts(&kf, &kd);
        e = upload_consts_tu(kf, kd);
        if (e != cudaSuccess) return cuda_error(e, "codelet constants");
        g_base[dev] = static_cast<unsigned char*>(ptr);
    }
    *base = g_base[dev];
    return FYG_OK;
}

cudaError_t launch_tagged(int cb, int cls, const PassParams& p, unsigned grid, int threads, size_t smem,
                          cudaStream_t st) {
    if (cb == 16) return launch_variant<double, double, double, 16, 1>(p, grid, threads, smem, st);
    if (cls > 16) return launch_variant<float, float, float, 32, 1>(p, grid, threads, smem, st);
    return launch_variant<float, float, float, 16, 1>(p, grid, threads, smem, st);
}

// Device memory of device `dev`, or managed memory.
bool device_pointer(const void* ptr, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace fyg

using namespace fyg;

extern "C" int fyg_execute_noalloc(size_t n, size_t batch, int dtype, int direction, const void* in, void* out,
                                   void* stream) {
    clear_error();
    if (!in || !out) return set_error(FYG_ERR_NULL_PTR, "null buffer");
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "dtype must be FYG_C32 or FYG_C64");
    if (direction != FYG_FORWARD && direction != FYG_INVERSE)
        return set_error(FYG_ERR_INVALID_ARG, "direction must be FYG_FORWARD or FYG_INVERSE");
    if (batch < 1) return set_error(FYG_ERR_INVALID_ARG, "batch must be >= 1");
    if (n < 2 || n >= (1ull << 31) || !is_smooth(n, 13))
        return set_error(FYG_ERR_INVALID_LENGTH, "allocation-free path: length must be 13-smooth and >= 2");
    const int cb = dtype == FYG_C32 ? 8 : 16;
    if (((uintptr_t)in % cb) || ((uintptr_t)out % cb))
        return set_error(FYG_ERR_MISALIGNED, "buffers must be aligned to the complex element size");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cuda_error(cudaGetLastError(), "cudaGetDevice");
    if (!device_pointer(in, dev) || !device_pointer(out, dev))
        return set_error(FYG_ERR_INVALID_ARG,
                         "allocation-free path: in and out must be device pointers of the current device");
    const cudaStream_t st = (cudaStream_t)stream;

    // ---- schedule (the planner's rules for a plain plan) ----
    std::vector<int> prad;
    if (single_pass_fits(cb, n, (size_t)-1)) prad = {(int)n};
    else if (!split_passes(n, cb, false, prad))
        return set_error(FYG_ERR_UNSUPPORTED, "no pass decomposition for length " + std::to_string(n));
    const int P = (int)prad.size();
    if (P > kMaxPasses) return set_error(FYG_ERR_UNSUPPORTED, "allocation-free path: too many passes");
    const size_t nbuf = P >= 3 ? 2 : (P == 2 ? 1 : 0);
    const size_t inter = (size_t)n * batch * cb;
    if (nbuf * inter > kNoAllocScratchBytes)
        return set_error(FYG_ERR_INVALID_LENGTH,
                         "allocation-free path: n * batch * element size (x2 for 3+ passes) must be <= " +
                             std::to_string(kNoAllocScratchBytes) + " bytes");
    if (P > 1 && (uint64_t)(n / *std::min_element(prad.begin(), prad.end())) * batch >= (1ull << 31))
        return set_error(FYG_ERR_INVALID_LENGTH, "allocation-free path: too many columns");

    unsigned char* base = nullptr;
    int rc = noalloc_setup(&base);
    if (rc) return rc;
    unsigned char* tab = base;
    unsigned char* scratch0 = base + kNoAllocTableBytes;
    unsigned char* scratch1 = scratch0 + inter;

    // ---- table layout; the tables are written on the device when the array holds another
    //      length's ----
    TableLayout tl;
    std::memset(&tl, 0, sizeof(tl));
    tl.passes = P;
    tl.cb = cb;
    size_t off = 0;
    auto place = [&](size_t bytes) {
        const size_t at = (off + 255) & ~(size_t)255;
        off = at + bytes;
        return at;
    };
    for (int i = 0; i < P; ++i) {
        int same = -1;
        for (int k = 0; k < tl.nlocal; ++k) if (tl.R[k] == prad[i]) same = k;
        if (same < 0) {
            same = tl.nlocal++;
            tl.R[same] = prad[i];
            tl.local_off[same] = place((size_t)prad[i] * 2 * cb);
        }
        tl.local_of_pass[i] = same;
    }
    if (P > 1) {
        int sh = 0;
        while ((1ull << (2 * sh)) < n) ++sh;   // 2^shift ~ sqrt(n), as the plans' tables
        if (sh < 1) sh = 1;
        tl.L = n;
        tl.shift = sh;
        tl.nlo = 1ull << sh;
        tl.nhi = (n + tl.nlo - 1) / tl.nlo;
        const size_t es = cb == 8 ? sizeof(float4) : sizeof(double2);
        tl.hi_off = place(tl.nhi * es);
        tl.lo_off = place(tl.nlo * es);
    }
    tl.bytes = off;
    if (tl.bytes > kNoAllocTableBytes)
        return set_error(FYG_ERR_INVALID_LENGTH, "allocation-free path: twiddle tables exceed the table region");
    const uint64_t key = ((uint64_t)n << 5) | (uint64_t)cb;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_tab_key[dev] != key) {
            uint64_t total = tl.nhi + tl.nlo;
            for (int k = 0; k < tl.nlocal; ++k) total += (uint64_t)tl.R[k];
            const unsigned blocks = (unsigned)std::min<uint64_t>((total + 255) / 256, 1024);
            k_noalloc_tables<<<blocks, 256, 0, st>>>(tab, tl);
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                g_tab_key[dev] = 0;
                return cuda_error(e, "allocation-free table kernel");
            }
            g_tab_key[dev] = key;
        }
    }
    std::vector<const void*> local(P, nullptr);
    for (int i = 0; i < P; ++i) local[i] = tab + tl.local_off[tl.local_of_pass[i]];
    const void* tw_hi = P > 1 ? (const void*)(tab + tl.hi_off) : nullptr;
    const void* tw_lo = P > 1 ? (const void*)(tab + tl.lo_off) : nullptr;
    const int tw_shift = P > 1 ? tl.shift : 1;

    // ---- passes: in -> scratch0 -> scratch1 -> ... -> out ----
    const bool inverse = direction == FYG_INVERSE;
    uint64_t Ns = 1;
    for (int i = 0; i < P; ++i) {
        PassParams p;
        std::memset(&p, 0, sizeof(p));
        const int R = prad[i];
        const bool single = P == 1;
        const int C = single ? single_pass_cols(cb, R, batch, 0) : multi_C(cb, R);
        const std::vector<int> rad = radices_for(R, cb);
        fill_geom(p.g, R, C, single, rad);
        p.Rr = (int)(n / R);
        p.Ns = (int)Ns;
        p.Ns_out = (int)Ns;
        p.Lr = (int)(n / (Ns * R));
        p.div_Rr = make_fastdiv((uint32_t)p.Rr);
        p.div_Ns = make_fastdiv((uint32_t)p.Ns);
        p.div_Ns_out = make_fastdiv((uint32_t)p.Ns_out);
        p.ncols = (int64_t)batch * p.Rr;
        p.idist = p.odist = (int64_t)n;
        p.in = i == 0 ? in : (i % 2 == 1 ? (const void*)scratch0 : (const void*)scratch1);
        p.out = i == P - 1 ? out : (i % 2 == 0 ? (void*)scratch0 : (void*)scratch1);
        p.tw_local = local[i];
        p.tw_hi = tw_hi;
        p.tw_lo = tw_lo;
        p.tw_shift = tw_shift;
        p.load_mode = LD_PLAIN;
        p.store_mode = ST_PLAIN;
        p.conj_in = (i == 0 && inverse) ? 1 : 0;
        p.conj_out = (i == P - 1 && inverse) ? 1 : 0;
        p.scale = (i == P - 1 && inverse) ? 1.0 / (double)n : 1.0;
        p.scale2 = 1.0;
        p.nvalid = (int64_t)n;
        const int cls = tile_class(cb, *std::max_element(rad.begin(), rad.end()));
        const int threads = single ? single_pass_threads(R, C, rad, 0) : threads_for(R, C, kMaxThreads);
        const size_t smem = smem_for(cb, R, C, single);
        const unsigned grid = (unsigned)((p.ncols + C - 1) / C);
        cudaError_t e = launch_tagged(cb, cls, p, grid, threads, smem, st);
        if (e != cudaSuccess) return cuda_error(e, "allocation-free pass launch");
        Ns *= (uint64_t)R;
    }
    return FYG_OK;
}
