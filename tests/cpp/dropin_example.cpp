// The reference's example (example.cpp: aligned host buffers, uniform[-1,1] input, an invoker
// per length, dispatch<false>) written against the drop-in GPU header, plus the inverse that
// example meant to call and a complex<double> run.  Exits non-zero on a parity failure.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "foye_FFT_gpu.hpp"

template <typename T>
static double naive_err(const std::vector<std::complex<T>>& x, const std::vector<std::complex<T>>& y) {
    const std::size_t n = x.size();
    long double num = 0, den = 0;
    const long double tp = 6.283185307179586476925286766559005768L;
    for (std::size_t k = 0; k < n; ++k) {
        long double re = 0, im = 0;
        for (std::size_t j = 0; j < n; ++j) {
            const long double a = -tp * (long double)((j * k) % n) / (long double)n;
            re += (long double)x[j].real() * cosl(a) - (long double)x[j].imag() * sinl(a);
            im += (long double)x[j].real() * sinl(a) + (long double)x[j].imag() * cosl(a);
        }
        num += (re - y[k].real()) * (re - y[k].real()) + (im - y[k].imag()) * (im - y[k].imag());
        den += re * re + im * im;
    }
    return (double)sqrtl(num / den);
}

int main() {
    int fails = 0;
    for (std::size_t length : {1024u, 1009u, 999u, 2520u}) {
        std::vector<std::complex<float>> in(length), fwd(length), inv(length);
        unsigned s = 12345u + (unsigned)length;
        for (auto& v : in) {
            s = s * 1664525u + 1013904223u; const float a = (float)(s >> 8) / 16777216.0f * 2.f - 1.f;
            s = s * 1664525u + 1013904223u; const float b = (float)(s >> 8) / 16777216.0f * 2.f - 1.f;
            v = {a, b};
        }
        fy::fft::FFT1D_C2C_invoker invoker{length};
        invoker.dispatch<false>(reinterpret_cast<float*>(in.data()), reinterpret_cast<float*>(fwd.data()));
        invoker.dispatch<true>(reinterpret_cast<float*>(fwd.data()), reinterpret_cast<float*>(inv.data()));
        const double e = naive_err(in, fwd);
        double rt = 0, nr = 0;
        for (std::size_t i = 0; i < length; ++i) { rt += std::norm(inv[i] - in[i]); nr += std::norm(in[i]); }
        rt = std::sqrt(rt / nr);
        const double tol = 4.0 * std::log2((double)length) * 1.1920929e-7;
        const int strat = (int)fy::fft::FFT1D_C2C_invoker::acquired_execution_strategy(length);
        std::printf("n=%zu strategy=%d fwd rel-L2 %.2e round trip %.2e\n", length, strat, e, rt);
        if (!(e <= tol && rt <= tol)) ++fails;
        // complex<double>
        std::vector<std::complex<double>> ind(in.begin(), in.end()), outd(length);
        invoker.dispatch<false>(ind.data(), outd.data());
        const double ed = naive_err(ind, outd);
        std::printf("   complex<double> fwd rel-L2 %.2e\n", ed);
        if (!(ed <= 4.0 * std::log2((double)length) * 2.220446e-16)) ++fails;
    }
    return fails ? 1 : 0;
}
