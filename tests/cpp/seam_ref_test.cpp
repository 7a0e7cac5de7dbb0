// seam_ref_test.cpp -- the reference library's own classes (<genFFT/fft.h>,
// unmodified) with the GB300 backend plugged into their factory seam
// (fft.h:56, 117, 173, FFTReal.h:188).  Built against the reference's
// headers where a genFFT checkout is available; it checks that reference
// code spelling genfft::FFT<T, genfft::gb300::GetImpl> compiles and links.
// When run (on a GB300), it compares each transform with the reference's
// own default backend on the same input, within the reference's FFT_Eps.
#include <genFFT/fft.h>
#include <genfft/gb300_backend.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

static int failures = 0;

template <typename T>
double fft_eps(int n) { return sizeof(T) == 8 ? 1e-8 + n * 1e-12 : 1e-5 + n * 1e-8; }

template <typename T>
void fill(std::vector<std::complex<T>> &v, unsigned seed)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> d(-1, 1);
    for (auto &c : v) c = {(T)d(rng), (T)d(rng)};
}

template <typename T>
void compare(const char *what, int n, const std::complex<T> *a, const std::complex<T> *b, int count)
{
    const double eps = fft_eps<T>(n);
    for (int i = 0; i < count; i++)
        if (std::abs(a[i].real() - b[i].real()) > eps || std::abs(a[i].imag() - b[i].imag()) > eps) {
            std::printf("FAIL %s n=%d i=%d\n", what, n, i);
            failures++;
            return;
        }
}

template <typename T>
void run(int n)
{
    std::vector<std::complex<T>> x(n), ref(n), gpu(n);
    fill(x, 11u + n);
    genfft::FFT<T> cpu(n);
    genfft::FFT<T, genfft::gb300::GetImpl> gb(n);
    cpu.template transform<false>(ref.data(), x.data());
    gb.template transform<false>(gpu.data(), x.data());
    compare("FFT forward", n, gpu.data(), ref.data(), n);
    cpu.template transform<true>(ref.data(), x.data());
    gb.template transform<true>(gpu.data(), x.data());
    compare("FFT inverse", n, gpu.data(), ref.data(), n);

    const int cols = 5;
    std::vector<std::complex<T>> vx((size_t)n * cols), vref(vx.size()), vgpu(vx.size());
    fill(vx, 17u + n);
    genfft::FFTVert<T> vcpu(n);
    genfft::FFTVert<T, genfft::gb300::GetVertImpl> vgb(n);
    vcpu.template transform<false>(vref.data(), vx.data(), cols);
    vgb.template transform<false>(vgpu.data(), vx.data(), cols);
    compare("FFTVert forward", n, vgpu.data(), vref.data(), n * cols);

    if (n >= 2) {
        std::vector<T> r(n);
        for (int i = 0; i < n; i++) r[i] = x[i].real();
        std::vector<std::complex<T>> rref(n, {43, 21}), rgpu(n, {43, 21});
        genfft::RealFFT<T> rcpu(n);
        genfft::RealFFT<T, genfft::gb300::GetImpl, genfft::gb300::GetDITImpl> rgb(n);
        rcpu.forward(rref.data(), r.data(), true);
        rgb.forward(rgpu.data(), r.data(), true);
        compare("RealFFT half", n, rgpu.data(), rref.data(), n);  // the canary past n/2+1 too
        genfft::DIT<T> dcpu(n);
        genfft::DIT<T, genfft::gb300::GetDITImpl> dgb(n);
        std::vector<std::complex<T>> dref(n), dgpu(n);
        dcpu.apply(dref.data(), x.data(), false);
        dgb.apply(dgpu.data(), x.data(), false);
        compare("DIT full", n, dgpu.data(), dref.data(), n);
    }
}

int main()
{
    for (int l = 0; l <= 12; l++) {
        run<float>(1 << l);
        run<double>(1 << l);
    }
    std::printf("OK: %d failures\n", failures);
    return failures ? 1 : 0;
}
