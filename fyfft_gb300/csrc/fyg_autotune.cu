// fyg_autotune.cu -- measured choice of a length's schedule, cached in a JSON file.
//
// For one length the candidates are the knobs the planner otherwise sets by rule:
//   single-pass lengths   transforms per CTA (C) and the thread policy (about 16 points per
//                         thread, or one thread per butterfly of the widest stage), i.e. the
//                         threads per transform
//   multi-pass lengths    a cap on the pass radix (more, smaller passes or fewer, larger ones),
//                         the pass order and the register-resident tile width (wide tiles)
//   Rader / Bluestein     the convolution length (7-smooth lengths up to 8% above the minimum,
//                         and for Bluestein the power of two), a cap on its pass radix, the
//                         pass order (which radix the fused mid pass takes) and the tile width
// FYG_AUTOTUNE_VERBOSE=1 lists every candidate's time on stderr.
// Every candidate plan runs a forward batch on the current device (CUDA events, best of three
// after a warm-up); the fastest is written to the cache under "c32:<n>" / "c64:<n>" together
// with the device signature (name, SM count, compute capability, driver).  A cache written
// for another device signature is ignored.
#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "fyg_host.h"

namespace fyg {
namespace {

std::mutex g_mu;
struct Cache {
    std::string path, device;
    std::map<std::string, TuneChoice> entries;
    bool loaded = false;
};
Cache g_cache;

std::string device_signature() {
    int dev = 0, drv = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) { cudaGetLastError(); return "unknown"; }
    cudaDriverGetVersion(&drv);
    std::ostringstream o;
    o << prop.name << "|" << prop.multiProcessorCount << "|" << prop.major << "." << prop.minor << "|" << drv;
    return o.str();
}

std::string default_path() {
    if (const char* e = std::getenv("FYG_AUTOTUNE_CACHE")) return e;
    const char* home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/fyfft_gb300/autotune.json";
}

std::string key_of(size_t n, int dtype) { return std::string(dtype == FYG_C32 ? "c32:" : "c64:") + std::to_string(n); }

// The cache is written by save() below, one entry per line; load() reads exactly that format.
void load(const std::string& path) {
    g_cache.path = path;
    g_cache.entries.clear();
    g_cache.device.clear();
    g_cache.loaded = true;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        const size_t d = line.find("\"device\": \"");
        if (d != std::string::npos) {
            const size_t a = d + 11, b = line.find('"', a);
            if (b != std::string::npos) g_cache.device = line.substr(a, b - a);
            continue;
        }
        char key[64];
        unsigned long long r = 0, m = 0;
        int c = 0, o = 0, th = 0, w = 0;
        double ms = 0;
        const int got = std::sscanf(line.c_str(),
                                    " \"%63[^\"]\": {\"max_pass_radix\": %llu, \"conv_length\": %llu, \"cols\": %d, "
                                    "\"order\": %d, \"threads\": %d, \"wide\": %d, \"ms\": %lf",
                                    key, &r, &m, &c, &o, &th, &w, &ms);
        if (got == 8) {
            TuneChoice t;
            t.max_pass_radix = r;
            t.conv_length = m;
            t.cols = c;
            t.order = o;
            t.threads = th;
            t.wide = w;
            t.ms = ms;
            g_cache.entries[key] = t;
        }
    }
}

int save() {
    const std::string& path = g_cache.path;
    for (size_t i = 1; i < path.size(); ++i)
        if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
    std::ofstream f(path, std::ios::trunc);
    if (!f) return set_error(FYG_ERR_INVALID_ARG, "cannot write autotune cache " + path);
    f << "{\n  \"device\": \"" << g_cache.device << "\",\n  \"entries\": {\n";
    size_t i = 0;
    for (auto& kv : g_cache.entries) {
        char buf[320];
        std::snprintf(buf, sizeof(buf),
                      "    \"%s\": {\"max_pass_radix\": %llu, \"conv_length\": %llu, \"cols\": %d, \"order\": %d, "
                      "\"threads\": %d, \"wide\": %d, \"ms\": %.6f}%s\n",
                      kv.first.c_str(), (unsigned long long)kv.second.max_pass_radix,
                      (unsigned long long)kv.second.conv_length, kv.second.cols, kv.second.order, kv.second.threads,
                      kv.second.wide, kv.second.ms, ++i < g_cache.entries.size() ? "," : "");
        f << buf;
    }
    f << "  }\n}\n";
    return FYG_OK;
}

bool smooth(uint64_t n, uint64_t b) {
    for (uint64_t p = 2; p <= b; ++p)
        while (n % p == 0) n /= p;
    return n == 1;
}

bool prime(uint64_t n) {
    if (n < 2) return false;
    for (uint64_t q = 2; q * q <= n; ++q)
        if (n % q == 0) return false;
    return true;
}

std::vector<uint64_t> smooth7_from(uint64_t lo, int count, double max_rel) {
    std::vector<uint64_t> out;
    for (uint64_t m = lo; out.size() < (size_t)count && (double)m <= max_rel * (double)lo; ++m)
        if (smooth(m, 7)) out.push_back(m);
    return out;
}

std::vector<TuneChoice> candidates(size_t n, int dtype, size_t batch) {
    const int cb = dtype == FYG_C32 ? 8 : 16;
    std::vector<TuneChoice> out;
    out.push_back(TuneChoice());
    auto add = [&](uint64_t r, uint64_t m, int c, int o = 0, int th = 0, int w = 0) {
        TuneChoice t;
        t.max_pass_radix = r;
        t.conv_length = m;
        t.cols = c;
        t.order = o;
        t.threads = th;
        t.wide = w;
        out.push_back(t);
    };
    const int nwide = dtype == FYG_C32 ? 2 : 1;   // wide register-resident tiles: FP32 only
    // single-pass lengths: transforms per CTA x thread policy (threads per transform)
    auto add_single = [&](uint64_t m, uint64_t L) {
        for (int c : {1, 2, 4, 8, 16, 32, 64})
            if ((size_t)c <= batch && (uint64_t)c * L <= 16384)
                for (int th : {0, 1}) add(0, m, c, 0, th);
    };
    if (smooth(n, 13)) {
        if (single_pass_fits(cb, n, (size_t)-1)) {
            add_single(0, n);
        } else {
            for (int w = 0; w < nwide; ++w) {
                if (w) add(0, 0, 0, 0, 0, 1);
                for (uint64_t r : {2048ull, 1024ull, 512ull, 256ull, 128ull}) add(r, 0, 0, 0, 0, w);
                add(0, 0, 0, 1, 0, w);
            }
        }
        return out;
    }
    std::vector<uint64_t> ms;
    if (prime(n) && smooth(n - 1, 13)) ms.push_back(n - 1);
    else if (prime(n) && 2 * n - 3 <= 78125) ms = smooth7_from(2 * n - 3, 6, 1.08);
    else {
        ms = smooth7_from(2 * n - 1, 8, 1.08);
        uint64_t m2 = 1;
        while (m2 < 2 * n - 1) m2 <<= 1;
        if (std::find(ms.begin(), ms.end(), m2) == ms.end()) ms.push_back(m2);
    }
    for (uint64_t m : ms) {
        if (single_pass_fits(cb, m, (size_t)-1)) {
            add_single(m, m);
            continue;
        }
        for (int o : {0, 1}) {
            for (int w = 0; w < nwide; ++w) add(0, m, 0, o, 0, w);
            add(256, m, 0, o);
        }
    }
    return out;
}

}  // namespace

bool tune_lookup_key(const std::string& key, TuneChoice* out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_cache.loaded) load(default_path());
    if (g_cache.device != device_signature()) return false;
    auto it = g_cache.entries.find(key);
    if (it == g_cache.entries.end()) return false;
    *out = it->second;
    return true;
}

bool tune_lookup(size_t n, int dtype, TuneChoice* out) { return tune_lookup_key(key_of(n, dtype), out); }

int tune_store_key(const std::string& key, const TuneChoice& choice, const char* cache_path) {
    const std::string path = cache_path ? cache_path : default_path();
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_cache.loaded || g_cache.path != path) load(path);
    const std::string dev = device_signature();
    if (g_cache.device != dev) {
        g_cache.entries.clear();
        g_cache.device = dev;
    }
    g_cache.entries[key] = choice;
    return save();
}

}  // namespace fyg

using namespace fyg;

extern "C" int fyg_device_signature(char* buf, size_t len) {
    if (!buf || len == 0) return set_error(FYG_ERR_NULL_PTR, "null buffer");
    const std::string sig = device_signature();
    if (sig.size() + 1 > len) return set_error(FYG_ERR_INVALID_ARG, "buffer too small");
    std::memcpy(buf, sig.c_str(), sig.size() + 1);
    return FYG_OK;
}

extern "C" int fyg_autotune(size_t n, int dtype, size_t batch, const char* cache_path, double* best_ms) {
    clear_error();
    if (n < 2 || batch < 1) return set_error(FYG_ERR_INVALID_ARG, "autotune: n >= 2 and batch >= 1");
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "bad dtype");
    const std::string path = cache_path ? cache_path : default_path();
    const size_t cb = dtype == FYG_C32 ? 8 : 16;
    DevBuf in, out;
    int rc = in.alloc(n * batch * cb);
    if (!rc) rc = out.alloc(n * batch * cb);
    if (rc) return rc;
    rc = fyg_fill_random_device(7, 1, dtype, n * batch, in.ptr, nullptr);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    TuneChoice best;
    bool have = false;
    const bool verbose = std::getenv("FYG_AUTOTUNE_VERBOSE") != nullptr;
    for (const TuneChoice& c : candidates(n, dtype, batch)) {
        fyg_plan* pl = nullptr;
        if (plan_create_opts(n, dtype, batch, c.wide ? FYG_FLAG_WIDE_TILES : 0, c.max_pass_radix, c.conv_length, c.cols,
                             c.order, c.threads, &pl) != FYG_OK)
            continue;
        double t = 1e30;
        bool ok = fyg_execute(pl, in.ptr, out.ptr, FYG_FORWARD, nullptr) == FYG_OK;
        // short plans: several back-to-back executions behind a delay kernel, so the events
        // bracket device time rather than host launch latency
        const int inner = (uint64_t)n * batch < (1u << 22) ? 10 : 1;
        for (int rep = 0; rep < 3 && ok; ++rep) {
            if (inner > 1) launch_delay(200000, nullptr);
            cudaEventRecord(e0, nullptr);
            for (int q = 0; q < inner && ok; ++q) ok = fyg_execute(pl, in.ptr, out.ptr, FYG_FORWARD, nullptr) == FYG_OK;
            cudaEventRecord(e1, nullptr);
            if (cudaEventSynchronize(e1) != cudaSuccess) ok = false;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            t = std::min(t, (double)ms / inner);
        }
        fyg_plan_destroy(pl);
        if (verbose)
            std::fprintf(stderr,
                         "fyg_autotune n=%zu max_pass_radix=%llu conv_length=%llu cols=%d order=%d threads=%d wide=%d: "
                         "%s %.4f ms\n",
                         n, (unsigned long long)c.max_pass_radix, (unsigned long long)c.conv_length, c.cols, c.order,
                         c.threads, c.wide, ok ? "ok" : "failed", ok ? t : 0.0);
        if (ok && (!have || t < best.ms)) {
            best = c;
            best.ms = t;
            have = true;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    clear_error();
    if (!have) return set_error(FYG_ERR_UNSUPPORTED, "autotune: no candidate plan ran");
    if (best_ms) *best_ms = best.ms;
    return tune_store_key(key_of(n, dtype), best, path.c_str());
}
