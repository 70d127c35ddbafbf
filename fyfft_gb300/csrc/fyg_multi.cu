// fyg_multi.cu -- batch sharding across devices: the partition of a batch (uniform or of uneven
// lengths) into contiguous shards of near-equal cost, and a multi-device plan that runs one
// shard per device with no collective.
//
// Transforms are independent (the reference dispatches one transform per call,
// foye_FFT.hpp:128-151), so a batch shards by transform with no data exchange: shard i is the
// contiguous range [bounds[i], bounds[i+1]) of the batch, run by its own plan on its own device
// and stream.  The same partition serves one process driving several devices
// (fyg_multi_create) and one process per device (each rank calls fyg_partition and runs its
// range, as bench.py does under torchrun).
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "fyg_host.h"

using namespace fyg;

namespace {

// Cost of one transform: proportional to its arithmetic, n log2 n (at least n).
double transform_cost(size_t n) { return n < 2 ? 1.0 : (double)n * std::log2((double)n); }

}  // namespace

struct fyg_multi {
    size_t n = 0, batch = 0;
    int dtype = FYG_C32;
    std::vector<int> devices;
    std::vector<size_t> bounds;          // ndev + 1 transform indices
    std::vector<fyg_plan*> plans;        // one per shard (null for an empty shard)
    std::vector<cudaStream_t> streams;   // one per shard, on the shard's device
    ~fyg_multi() {
        int prev = 0;
        cudaGetDevice(&prev);
        for (size_t i = 0; i < plans.size(); ++i) {
            if (streams[i]) {
                cudaSetDevice(devices[i]);
                cudaStreamDestroy(streams[i]);
            }
            fyg_plan_destroy(plans[i]);
        }
        cudaSetDevice(prev);   // the caller's device, as every other entry point leaves it
    }
};

extern "C" {

int fyg_partition(const size_t* lengths, size_t count, int parts, size_t* bounds) {
    clear_error();
    if (!bounds) return set_error(FYG_ERR_NULL_PTR, "bounds is null");
    if (parts < 1) return set_error(FYG_ERR_INVALID_ARG, "parts must be >= 1");
    bounds[0] = 0;
    if (!lengths) {
        for (int i = 1; i <= parts; ++i) bounds[i] = count * (size_t)i / (size_t)parts;
        return FYG_OK;
    }
    // contiguous shards: boundary i at the first transform whose prefix cost reaches i/parts
    // of the total (ties to the earlier index), so every shard is a run of whole transforms
    double total = 0;
    for (size_t k = 0; k < count; ++k) total += transform_cost(lengths[k]);
    double prefix = 0;
    size_t k = 0;
    for (int i = 1; i < parts; ++i) {
        const double target = total * (double)i / (double)parts;
        while (k < count && prefix + 0.5 * transform_cost(lengths[k]) < target) prefix += transform_cost(lengths[k++]);
        bounds[i] = k;
    }
    bounds[parts] = count;
    return FYG_OK;
}

int fyg_multi_create(size_t n, int dtype, size_t batch, int flags, const int* devices, int ndev, fyg_multi** out) {
    clear_error();
    if (!out || !devices) return set_error(FYG_ERR_NULL_PTR, "null argument");
    *out = nullptr;
    if (ndev < 1) return set_error(FYG_ERR_INVALID_ARG, "ndev must be >= 1");
    if (batch < 1) return set_error(FYG_ERR_INVALID_ARG, "batch must be >= 1");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceCount");
    for (int i = 0; i < ndev; ++i)
        if (devices[i] < 0 || devices[i] >= count)
            return set_error(FYG_ERR_INVALID_ARG, "device " + std::to_string(devices[i]) + " does not exist");
    int prev = 0;
    cudaGetDevice(&prev);
    auto* m = new fyg_multi();
    m->n = n;
    m->batch = batch;
    m->dtype = dtype;
    m->devices.assign(devices, devices + ndev);
    m->bounds.resize(ndev + 1);
    m->plans.assign(ndev, nullptr);
    m->streams.assign(ndev, nullptr);
    int rc = fyg_partition(nullptr, batch, ndev, m->bounds.data());
    for (int i = 0; i < ndev && !rc; ++i) {
        const size_t nb = m->bounds[i + 1] - m->bounds[i];
        if (nb == 0) continue;
        e = cudaSetDevice(devices[i]);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->streams[i], cudaStreamNonBlocking);
        if (e != cudaSuccess) { rc = cuda_error(e, "shard device / stream"); break; }
        rc = fyg_plan_create(n, dtype, nb, flags, &m->plans[i]);
    }
    cudaSetDevice(prev);
    if (rc) {
        delete m;
        return rc;
    }
    *out = m;
    return FYG_OK;
}

int fyg_multi_shards(const fyg_multi* m, int* ndev, size_t* bounds) {
    if (!m) return set_error(FYG_ERR_NULL_PTR, "null multi-device plan");
    if (ndev) *ndev = (int)m->devices.size();
    if (bounds) std::memcpy(bounds, m->bounds.data(), m->bounds.size() * sizeof(size_t));
    return FYG_OK;
}

// Host (or managed) buffers holding the whole batch: each shard is staged to its device, run
// and copied back by its own host thread; returns when every shard's output is in `out`.
int fyg_multi_execute(fyg_multi* m, const void* in, void* out, int direction) {
    clear_error();
    if (!m) return set_error(FYG_ERR_NULL_PTR, "null multi-device plan");
    if (!in || !out) return set_error(FYG_ERR_NULL_PTR, "null buffer");
    const size_t eb = m->dtype == FYG_C32 ? 8 : 16;
    const size_t nd = m->devices.size();
    std::vector<int> rcs(nd, FYG_OK);
    std::vector<std::string> errs(nd);
    std::vector<std::thread> th;
    for (size_t i = 0; i < nd; ++i) {
        if (!m->plans[i]) continue;
        th.emplace_back([&, i] {
            const size_t off = m->bounds[i] * m->n * eb;
            cudaSetDevice(m->devices[i]);
            rcs[i] = fyg_execute(m->plans[i], static_cast<const char*>(in) + off, static_cast<char*>(out) + off,
                                 direction, m->streams[i]);
            if (rcs[i] == FYG_OK) {
                const cudaError_t e = cudaStreamSynchronize(m->streams[i]);
                if (e != cudaSuccess) rcs[i] = cuda_error(e, "shard synchronize");
            }
            if (rcs[i]) errs[i] = last_error();
        });
    }
    for (auto& t : th) t.join();
    for (size_t i = 0; i < nd; ++i)
        if (rcs[i]) return set_error(rcs[i], "shard " + std::to_string(i) + ": " + errs[i]);
    return FYG_OK;
}

// Per-shard device buffers (ins[i], outs[i] on devices[i], holding shard i's transforms back
// to back): every shard is launched on its stream; returns after the launches (asynchronous,
// fyg_multi_synchronize waits).
int fyg_multi_execute_device(fyg_multi* m, const void* const* ins, void* const* outs, int direction) {
    clear_error();
    if (!m || !ins || !outs) return set_error(FYG_ERR_NULL_PTR, "null argument");
    int prev = 0;
    cudaGetDevice(&prev);
    int rc = FYG_OK;
    for (size_t i = 0; i < m->devices.size() && !rc; ++i) {
        if (!m->plans[i]) continue;
        cudaSetDevice(m->devices[i]);
        rc = fyg_execute(m->plans[i], ins[i], outs[i], direction, m->streams[i]);
        if (rc) rc = set_error(rc, "shard " + std::to_string(i) + ": " + last_error());
    }
    cudaSetDevice(prev);
    return rc;
}

int fyg_multi_synchronize(fyg_multi* m) {
    if (!m) return set_error(FYG_ERR_NULL_PTR, "null multi-device plan");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaError_t err = cudaSuccess;
    for (size_t i = 0; i < m->devices.size(); ++i) {
        if (!m->streams[i]) continue;
        cudaSetDevice(m->devices[i]);
        const cudaError_t e = cudaStreamSynchronize(m->streams[i]);
        if (e != cudaSuccess && err == cudaSuccess) err = e;
    }
    cudaSetDevice(prev);
    return err == cudaSuccess ? FYG_OK : cuda_error(err, "shard synchronize");
}

int fyg_multi_destroy(fyg_multi* m) {
    delete m;
    return FYG_OK;
}

}  // extern "C"
