// foye_FFT_gpu.hpp -- drop-in GPU replacement for fyFFT's foye_FFT.hpp (kjear/fyFFT).
//
// Same class, constructor, dispatch<bool invert> and static strategy query as
// fy::fft::FFT1D_C2C_invoker (foye_FFT.hpp:89-185), implemented over the C ABI of libfygpu.so
// (fygpu.h).  A caller swaps `#include "foye_FFT.hpp"` for this header and links libfygpu.so.
//
// Differences a caller can observe:
//   * buffers may be host pointers (staged to the GPU and synchronized before dispatch returns,
//     as the reference's dispatch is synchronous) or device pointers (asynchronous on the
//     invoker's stream);
//   * complex<double> overloads, a batch count, an adjoint entry point;
//   * any length >= 1 works (the reference declares 2..80000 and is undefined outside it); the
//     GPU never uses an O(N^2) DFT;
//   * failures throw std::runtime_error instead of being undefined behaviour.
#pragma once

#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>

#include "fygpu.h"

namespace fy::fft {

inline constexpr std::size_t min_input_length = 2;
inline constexpr std::size_t max_input_length = 80'000;

struct FFT1D_C2C_invoker {
    enum class FFT_execution_strategy { kernel_direct, mix_radix, rader, bluestein, DFT };

    // foye_FFT.hpp:101: plan for `batch` contiguous transforms of `length` on `stream`
    // (a cudaStream_t; nullptr = legacy default stream).
    explicit FFT1D_C2C_invoker(std::size_t length, std::size_t batch = 1, void* stream = nullptr)
        : N(length), B(batch), stream_(stream) {
        if (length < 1) throw std::invalid_argument("FFT1D_C2C_invoker: length must be >= 1");
    }

    FFT1D_C2C_invoker(const FFT1D_C2C_invoker&) = delete;
    FFT1D_C2C_invoker& operator=(const FFT1D_C2C_invoker&) = delete;
    FFT1D_C2C_invoker(FFT1D_C2C_invoker&& o) noexcept { *this = std::move(o); }
    FFT1D_C2C_invoker& operator=(FFT1D_C2C_invoker&& o) noexcept {
        if (this != &o) {
            release();
            N = o.N; B = o.B; stream_ = o.stream_;
            p32_ = std::exchange(o.p32_, nullptr);
            p64_ = std::exchange(o.p64_, nullptr);
        }
        return *this;
    }
    ~FFT1D_C2C_invoker() { release(); }

    // foye_FFT.hpp:128-151: interleaved complex<float> (re, im) buffers of N * batch elements
    template <bool invert>
    void dispatch(const float* input, float* output) {
        check(fyg_execute(plan(FYG_C32), input, output, invert ? FYG_INVERSE : FYG_FORWARD, stream_));
    }
    template <bool invert>
    void dispatch(const double* input, double* output) {
        check(fyg_execute(plan(FYG_C64), input, output, invert ? FYG_INVERSE : FYG_FORWARD, stream_));
    }
    template <bool invert>
    void dispatch(const std::complex<float>* input, std::complex<float>* output) {
        dispatch<invert>(reinterpret_cast<const float*>(input), reinterpret_cast<float*>(output));
    }
    template <bool invert>
    void dispatch(const std::complex<double>* input, std::complex<double>* output) {
        dispatch<invert>(reinterpret_cast<const double*>(input), reinterpret_cast<double*>(output));
    }

    // output = scale * F^H g (conjugate transpose of the forward transform)
    void adjoint(const float* g, float* output, double scale = 1.0) {
        check(fyg_execute_adjoint(plan(FYG_C32), g, output, scale, stream_));
    }
    void adjoint(const double* g, double* output, double scale = 1.0) {
        check(fyg_execute_adjoint(plan(FYG_C64), g, output, scale, stream_));
    }

    // foye_FFT.hpp:162-184 (the reference's choice for `length`)
    static FFT_execution_strategy acquired_execution_strategy(std::size_t length) {
        const int s = fyg_strategy(length);
        if (s < 0) throw std::invalid_argument("acquired_execution_strategy: length must be >= 2");
        return static_cast<FFT_execution_strategy>(s);
    }

    std::size_t length() const { return N; }

private:
    std::size_t N = 0, B = 1;
    void* stream_ = nullptr;
    fyg_plan* p32_ = nullptr;
    fyg_plan* p64_ = nullptr;

    static void check(int rc) {
        if (rc != FYG_OK) throw std::runtime_error(std::string("fyFFT GPU: ") + fyg_last_error_string());
    }
    fyg_plan* plan(int dtype) {
        fyg_plan*& p = dtype == FYG_C32 ? p32_ : p64_;
        if (!p) check(fyg_plan_create(N, dtype, B, 0, &p));
        return p;
    }
    void release() {
        if (p32_) fyg_plan_destroy(p32_);
        if (p64_) fyg_plan_destroy(p64_);
        p32_ = p64_ = nullptr;
    }
};

}  // namespace fy::fft
