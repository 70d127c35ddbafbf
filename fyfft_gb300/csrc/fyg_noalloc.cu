// fyg_noalloc.cu -- an entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code running while a stream is being captured into a CUDA
// graph, host applications that own every byte of device memory and hand plugins only their
// input and output buffers, and latency-bound loops that cannot afford the device-wide
// synchronization an allocation can cause.  fyg_execute_noalloc serves them with the
// multi-pass tile-pass kernel (the kernel that needs scratch for its pass intermediates): the
// scratch and the twiddle tables live in one file-scope __device__ array of fixed size that
// every GPU loading this library holds until the process exits.
//
// Limits: plain (13-smooth) lengths only; pass intermediates of at most kNoAllocScratchBytes
// (n * batch * element size, twice that for three or more passes) and twiddle tables of at most
// kNoAllocTableBytes.  The first call on a device looks up the array's device address with
// cudaGetSymbolAddress and uploads this file's codelet constants; make that first call before
// any stream capture.  All calls share the array: two calls that overlap on the GPU (e.g. on
// different streams) race.  The intermediates need no clearing (every pass writes all of its
// output before the next pass reads it); the tables are rewritten by every call.
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

bool device_pointer(const void* ptr) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
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
    if (!device_pointer(in) || !device_pointer(out))
        return set_error(FYG_ERR_INVALID_ARG, "allocation-free path: in and out must be device pointers");
    const cudaStream_t st = (cudaStream_t)stream;

    // ---- schedule (the same rules as a plan) ----
    std::vector<int> prad;
    if (n <= 16384 && tile_fits(cb, (int)n, 1, true)) prad = {(int)n};
    else if (!split_passes(n, cb, false, prad))
        return set_error(FYG_ERR_UNSUPPORTED, "no pass decomposition for length " + std::to_string(n));
    const int P = (int)prad.size();
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

    // ---- twiddle tables into the table region (host images, one copy each) ----
    size_t off = 0;
    auto put = [&](const std::vector<unsigned char>& h, const void** dptr) -> int {
        const size_t aligned = (off + 255) & ~(size_t)255;
        if (aligned + h.size() > kNoAllocTableBytes)
            return set_error(FYG_ERR_INVALID_LENGTH, "allocation-free path: twiddle tables exceed the table region");
        cudaError_t e = cudaMemcpyAsync(tab + aligned, h.data(), h.size(), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_error(e, "table copy");
        *dptr = tab + aligned;
        off = aligned + h.size();
        return FYG_OK;
    };
    std::vector<const void*> local(P, nullptr);
    for (int i = 0; i < P; ++i) {
        int same = -1;
        for (int j = 0; j < i; ++j) if (prad[j] == prad[i]) same = j;
        if (same >= 0) { local[i] = local[same]; continue; }
        rc = put(host_local_table(prad[i], cb), &local[i]);
        if (rc) return rc;
    }
    const void *tw_hi = nullptr, *tw_lo = nullptr;
    int tw_shift = 1;
    if (P > 1) {
        std::vector<unsigned char> th, tl;
        host_two_level(n, cb, th, tl, &tw_shift);
        rc = put(th, &tw_hi);
        if (!rc) rc = put(tl, &tw_lo);
        if (rc) return rc;
    }

    // ---- passes: in -> scratch0 -> scratch1 -> ... -> out ----
    const bool inverse = direction == FYG_INVERSE;
    uint64_t Ns = 1;
    for (int i = 0; i < P; ++i) {
        PassParams p;
        std::memset(&p, 0, sizeof(p));
        const int R = prad[i];
        const bool single = P == 1;
        const int C = single ? std::max(1, std::min((int)std::min<size_t>(batch, 256), (cb == 8 ? 4096 : 2048) / R))
                             : multi_C(cb, R);
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
        const int threads = threads_for(R, C, kMaxThreads);
        const size_t smem = smem_for(cb, R, C, single);
        const unsigned grid = (unsigned)((p.ncols + C - 1) / C);
        cudaError_t e = launch_tagged(cb, cls, p, grid, threads, smem, st);
        if (e != cudaSuccess) return cuda_error(e, "allocation-free pass launch");
        Ns *= (uint64_t)R;
    }
    return FYG_OK;
}
