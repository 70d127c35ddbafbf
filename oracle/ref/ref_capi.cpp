// C entry points over the reference's own fy::fft::FFT1D_C2C_invoker (foye_FFT.hpp:89-185),
// compiled from the unmodified reference headers by oracle/ref/build_ref.sh (natively with
// AVX2 on x86-64, or against oracle/ref/portable_intrin.h on other hosts).
// Test infrastructure only: used to pin the oracle and as the timed CPU baseline; the
// product never links it.
#include "foye_FFT.hpp"
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {
using invoker = fy::fft::FFT1D_C2C_invoker;
using strat = invoker::FFT_execution_strategy;
// The reference's O(N^2) fallback (src/foye_FFT_dft.hpp:63-88) allocates 16*N^2 bytes of tables;
// refuse it above this length instead of exhausting host memory.
constexpr std::size_t kMaxDftLength = 4096;
bool runnable(std::size_t n) {
    if (n < fy::fft::min_input_length) return false;
    strat s = invoker::acquired_execution_strategy(n);
    return !(s == strat::DFT && n > kMaxDftLength);
}

// A fixed set of worker threads, each owning one plan (mixed-radix, Rader and Bluestein plans
// hold mutable workspace, src/foye_FFT_mix_radix.hpp:538, so plans are never shared).  run()
// splits a contiguous batch into one contiguous range per worker and returns when all are done.
struct Pool {
    std::size_t n = 0;
    std::vector<invoker*> plans;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_go, cv_done;
    std::uint64_t generation = 0;
    int pending = 0;
    bool stop = false;
    // the current job
    std::size_t batch = 0;
    int inverse = 0;
    const float* in = nullptr;
    float* out = nullptr;

    void work(int t) {
        std::uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_go.wait(lk, [&] { return stop || generation != seen; });
                if (stop) return;
                seen = generation;
            }
            const int T = (int)plans.size();
            const std::size_t lo = batch * t / T, hi = batch * (t + 1) / T;
            for (std::size_t b = lo; b < hi; ++b) {
                const float* x = in + 2 * n * b;
                float* y = out + 2 * n * b;
                if (inverse) plans[t]->dispatch<true>(x, y); else plans[t]->dispatch<false>(x, y);
            }
            std::lock_guard<std::mutex> lk(mu);
            if (--pending == 0) cv_done.notify_one();
        }
    }
    void run(std::size_t b, int inv, const float* x, float* y) {
        {
            std::lock_guard<std::mutex> lk(mu);
            batch = b; inverse = inv; in = x; out = y;
            pending = (int)plans.size();
            ++generation;
        }
        cv_go.notify_all();
        std::unique_lock<std::mutex> lk(mu);
        cv_done.wait(lk, [&] { return pending == 0; });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_go.notify_all();
        for (auto& w : workers) w.join();
        for (auto* p : plans) delete p;
    }
};
}  // namespace

extern "C" {

// "native" (x86-64 AVX2) or "emulated" (portable intrinsics), and the host architecture
const char* fyref_build_info(void) {
#if defined(FYREF_EMULATED)
#if defined(__aarch64__)
    return "emulated aarch64";
#else
    return "emulated x86_64";
#endif
#else
    return "native x86_64";
#endif
}

// foye_FFT.hpp:162-184
int fyref_strategy(std::size_t n) { return static_cast<int>(invoker::acquired_execution_strategy(n)); }

int fyref_runnable(std::size_t n) { return runnable(n) ? 1 : 0; }

void* fyref_plan_create(std::size_t n) {
    if (!runnable(n)) return nullptr;
    return new invoker(n);
}

void fyref_plan_destroy(void* p) { delete static_cast<invoker*>(p); }

// foye_FFT.hpp:128-151; inverse != 0 -> dispatch<true> (scaled by 1/N)
int fyref_plan_execute(void* p, int inverse, const float* in, float* out) {
    if (!p) return -1;
    auto* inv = static_cast<invoker*>(p);
    if (inverse) inv->dispatch<true>(in, out); else inv->dispatch<false>(in, out);
    return 0;
}

int fyref_fft(std::size_t n, int inverse, const float* in, float* out) {
    void* p = fyref_plan_create(n);
    if (!p) return -1;
    fyref_plan_execute(p, inverse, in, out);
    fyref_plan_destroy(p);
    return 0;
}

// A pool of `threads` workers with one plan of length n each; *plan_seconds receives the plan
// construction time.  Null if the reference cannot run length n.
void* fyref_pool_create(std::size_t n, int threads, double* plan_seconds) {
    if (!runnable(n)) return nullptr;
    if (threads < 1) threads = 1;
    auto t0 = std::chrono::steady_clock::now();
    auto* pool = new Pool();
    pool->n = n;
    // the first plan on this thread (runs every lazily initialized static table once), the
    // others concurrently, one per worker (plan construction of long mixed-radix lengths takes
    // about a second each)
    pool->plans.assign(threads, nullptr);
    pool->plans[0] = new invoker(n);
    {
        std::vector<std::thread> build;
        for (int t = 1; t < threads; ++t) build.emplace_back([pool, t, n] { pool->plans[t] = new invoker(n); });
        for (auto& b : build) b.join();
    }
    auto t1 = std::chrono::steady_clock::now();
    for (int t = 0; t < threads; ++t) pool->workers.emplace_back([pool, t] { pool->work(t); });
    if (plan_seconds) *plan_seconds = std::chrono::duration<double>(t1 - t0).count();
    return pool;
}

// `batch` contiguous transforms of the pool's length split over its workers; *seconds receives
// the wall time of the execution.
int fyref_pool_run(void* pool, std::size_t batch, int inverse, const float* in, float* out, double* seconds) {
    if (!pool) return -1;
    auto t0 = std::chrono::steady_clock::now();
    static_cast<Pool*>(pool)->run(batch, inverse, in, out);
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

void fyref_pool_destroy(void* pool) { delete static_cast<Pool*>(pool); }

// One-shot form of the pool: plans built, batch run once, plans destroyed.
int fyref_batch(std::size_t n, std::size_t batch, int inverse, const float* in, float* out,
                int threads, double* seconds, double* plan_seconds) {
    if (!runnable(n)) return -1;
    if (threads < 1) threads = 1;
    if ((std::size_t)threads > batch) threads = (int)(batch ? batch : 1);
    void* pool = fyref_pool_create(n, threads, plan_seconds);
    if (!pool) return -1;
    fyref_pool_run(pool, batch, inverse, in, out, seconds);
    fyref_pool_destroy(pool);
    return 0;
}

}  // extern "C"
