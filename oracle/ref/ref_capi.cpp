// C entry points over the reference's own fy::fft::FFT1D_C2C_invoker (foye_FFT.hpp:89-185),
// compiled from the unmodified reference headers by oracle/ref/build_ref.sh.
// Test infrastructure only: used to pin the oracle and as the timed CPU baseline; the
// product never links it.
#include "foye_FFT.hpp"
#include <chrono>
#include <thread>
#include <vector>
#include <cstdio>

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
}

extern "C" {

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

// `batch` contiguous transforms of length n split across `threads` std::threads, one plan per
// thread (mixed-radix, Rader and Bluestein plans hold mutable workspace, so they are not
// shared). Plan construction is outside the timed region; *seconds receives the wall time of
// the execution only and *plan_seconds the plan construction time.
int fyref_batch(std::size_t n, std::size_t batch, int inverse, const float* in, float* out,
                int threads, double* seconds, double* plan_seconds) {
    if (!runnable(n)) return -1;
    if (threads < 1) threads = 1;
    if ((std::size_t)threads > batch) threads = (int)(batch ? batch : 1);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<invoker*> plans(threads);
    for (int t = 0; t < threads; ++t) plans[t] = new invoker(n);
    auto t1 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&, t] {
            std::size_t lo = batch * t / threads, hi = batch * (t + 1) / threads;
            for (std::size_t b = lo; b < hi; ++b) {
                const float* x = in + 2 * n * b;
                float* y = out + 2 * n * b;
                if (inverse) plans[t]->dispatch<true>(x, y); else plans[t]->dispatch<false>(x, y);
            }
        });
    }
    for (auto& th : pool) th.join();
    auto t2 = std::chrono::steady_clock::now();
    for (auto* p : plans) delete p;
    if (seconds) *seconds = std::chrono::duration<double>(t2 - t1).count();
    if (plan_seconds) *plan_seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

}  // extern "C"
