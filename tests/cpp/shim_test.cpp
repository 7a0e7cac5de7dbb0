// shim_test.cpp -- the reference's own test cases (test/fft_test_impl.h),
// written against the drop-in header genfft/fft.h and run on the GPU.
// Each case compares with an FP64 DFT using the reference's tolerance
// FFT_Eps (test/test_util.h:62-72), on host buffers (the reference's calling
// convention) and, for one case, on device buffers.
#include <genfft/fft.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

static int failures = 0;
#define CHECK(cond, ...)                        \
    do {                                        \
        if (!(cond)) {                          \
            std::printf("FAIL: " __VA_ARGS__);  \
            std::printf("\n");                  \
            failures++;                         \
        }                                       \
    } while (0)

template <typename T>
double fft_eps(int n) { return sizeof(T) == 8 ? 1e-8 + n * 1e-12 : 1e-5 + n * 1e-8; }

template <typename T>
void dummy(std::vector<std::complex<T>> &v, bool real, unsigned seed = 0)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> d(-1, 1);
    for (auto &c : v) c = {(T)d(rng), real ? (T)0 : (T)d(rng)};
}

// FP64 DFT with exact phase
template <typename T>
std::vector<std::complex<double>> dft(const std::complex<T> *x, int n, bool inv, long stride = 1)
{
    std::vector<std::complex<double>> out(n);
    for (int k = 0; k < n; k++) {
        std::complex<double> s = 0;
        for (int j = 0; j < n; j++) {
            const double a = (inv ? 2 : -2) * M_PI * (double)(((long long)j * k) % n) / n;
            s += std::complex<double>(x[j * stride]) * std::complex<double>(std::cos(a), std::sin(a));
        }
        out[k] = s;
    }
    return out;
}

template <typename T>
void TestFFT_Pow2(int n)
{
    genfft::FFT<T> fft(n);
    std::vector<std::complex<T>> in(n), out(n), invout(n);
    dummy(in, false);
    fft.template transform<false>(out.data(), in.data());
    fft.template transform<true>(invout.data(), out.data());
    const auto ref = dft(in.data(), n, false);
    const double eps = fft_eps<T>(n);
    for (int i = 0; i < n; i++) {
        CHECK(std::abs(out[i].real() - ref[i].real()) <= eps && std::abs(out[i].imag() - ref[i].imag()) <= eps,
              "FFT n=%d i=%d", n, i);
        CHECK(std::abs(invout[i].real() / n - in[i].real()) <= eps, "FFT inverse n=%d i=%d", n, i);
    }
    // README spelling
    std::vector<std::complex<T>> out2(n);
    fft.forward(out2.data(), in.data());
    for (int i = 0; i < n; i++) CHECK(out2[i] == out[i], "forward alias n=%d", n);
}

template <typename T>
void TestRealFFT_Pow2(int n, bool half)
{
    genfft::RealFFT<T> fft(n);
    const std::complex<T> fill = {43, 21};
    std::vector<std::complex<T>> out(n, fill), cin(n);
    std::vector<T> in(n);
    dummy(cin, true, 7);
    for (int i = 0; i < n; i++) in[i] = cin[i].real();
    fft.forward(out.data(), in.data(), half);
    const auto ref = dft(cin.data(), n, false);
    const double eps = fft_eps<T>(n);
    const int limit = half ? n / 2 + 1 : n;
    int i = 0;
    for (; i < limit; i++)
        CHECK(std::abs(out[i].real() - ref[i].real()) <= eps && std::abs(out[i].imag() - ref[i].imag()) <= eps,
              "RealFFT n=%d half=%d i=%d", n, half, i);
    for (; i < n; i++) CHECK(out[i] == fill, "RealFFT corruption n=%d @ %d", n, i);
}

template <typename T>
void TestDIT_Pow2(int n)
{
    std::vector<std::complex<T>> cin(n), half_in(n / 2 > 0 ? n / 2 : 1), out(n), zin(n);
    dummy(cin, true, 3);
    std::vector<T> real(n);
    for (int i = 0; i < n; i++) real[i] = cin[i].real();
    genfft::FFT<T> h(n == 1 ? 1 : n / 2);
    h.template transform<false>(zin.data(), (const std::complex<T> *)real.data());
    genfft::DIT<T> dit(n);
    dit.apply(out.data(), zin.data(), false);
    const auto ref = dft(cin.data(), n, false);
    const double eps = fft_eps<T>(n);
    for (int i = 0; i < n; i++)
        CHECK(std::abs(out[i].real() - ref[i].real()) <= eps && std::abs(out[i].imag() - ref[i].imag()) <= eps,
              "DIT n=%d i=%d", n, i);
}

template <typename T>
void TestFFTVert_Pow2(int n, int cols)
{
    genfft::FFTVert<T> fft(n);
    std::vector<std::complex<T>> in(n * cols), out(n * cols), invout(n * cols);
    dummy(in, false, 5);
    fft.template transform<false>(out.data(), cols, in.data(), cols, cols);
    fft.template transform<true>(invout.data(), cols, out.data(), cols, cols);
    const double eps = fft_eps<T>(n);
    for (int c = 0; c < cols; c += (cols > 8 ? cols / 7 : 1)) {
        const auto ref = dft(in.data() + c, n, false, cols);
        for (int i = 0; i < n; i++) {
            const auto g = out[i * cols + c];
            CHECK(std::abs(g.real() - ref[i].real()) <= eps && std::abs(g.imag() - ref[i].imag()) <= eps,
                  "FFTVert n=%d cols=%d c=%d i=%d", n, cols, c, i);
            CHECK(std::abs(invout[i * cols + c].real() / n - in[i * cols + c].real()) <= eps, "FFTVert inverse");
        }
    }
}

template <typename T>
void Test2D(int w, int h)
{
    genfft::FFT2D<T> fft(w, h);
    std::vector<std::complex<T>> in(w * h), out(w * h);
    dummy(in, false, 9);
    fft.template transform<false>(out.data(), w, in.data(), w);
    // separable FP64 reference
    std::vector<std::complex<double>> rows(w * h), ref(w * h);
    for (int r = 0; r < h; r++) {
        auto d = dft(in.data() + r * w, w, false);
        for (int c = 0; c < w; c++) rows[r * w + c] = d[c];
    }
    for (int c = 0; c < w; c++) {
        auto d = dft(rows.data() + c, h, false, w);
        for (int r = 0; r < h; r++) ref[r * w + c] = d[r];
    }
    const double eps = fft_eps<T>(w * h) * 4;
    for (int i = 0; i < w * h; i++)
        CHECK(std::abs(out[i] - std::complex<T>(ref[i])) <= eps, "FFT2D %dx%d i=%d", w, h, i);

    // real 2D, full-width Hermitian output
    genfft::RealFFT2D<T> rfft(w, h);
    std::vector<T> rin(w * h);
    for (int i = 0; i < w * h; i++) rin[i] = in[i].real();
    std::vector<std::complex<T>> cin(w * h), rout(w * h);
    for (int i = 0; i < w * h; i++) cin[i] = {rin[i], 0};
    rfft.forward(rout.data(), w, rin.data(), w);
    genfft::FFT2D<T> c2d(w, h);
    c2d.template transform<false>(out.data(), w, cin.data(), w);
    for (int i = 0; i < w * h; i++) CHECK(std::abs(rout[i] - out[i]) <= eps, "RealFFT2D %dx%d i=%d", w, h, i);
}

template <typename T>
void TestDevicePointers(int n)
{
    std::vector<std::complex<T>> in(n), out(n);
    dummy(in, false, 11);
    std::complex<T> *d_in, *d_out;
    cudaMalloc(&d_in, sizeof(std::complex<T>) * n);
    cudaMalloc(&d_out, sizeof(std::complex<T>) * n);
    cudaMemcpy(d_in, in.data(), sizeof(std::complex<T>) * n, cudaMemcpyHostToDevice);
    genfft::FFT<T> fft(n);
    fft.template transform<false>(d_out, d_in);
    cudaMemcpy(out.data(), d_out, sizeof(std::complex<T>) * n, cudaMemcpyDeviceToHost);
    const auto ref = dft(in.data(), n, false);
    for (int i = 0; i < n; i++) CHECK(std::abs(out[i] - std::complex<T>(ref[i])) <= fft_eps<T>(n) * 2, "device n=%d", n);
    cudaFree(d_in);
    cudaFree(d_out);
}

int main()
{
    try {
        for (int n = 1; n <= 4096; n *= 2) {
            TestFFT_Pow2<float>(n);
            TestFFT_Pow2<double>(n);
            TestRealFFT_Pow2<float>(n, true);
            TestRealFFT_Pow2<float>(n, false);
            TestRealFFT_Pow2<double>(n, true);
            TestDIT_Pow2<float>(n);
        }
        TestFFT_Pow2<float>(1 << 15);  // four-step path
        const int vert[][2] = {{1, 1}, {2, 7}, {4, 33}, {8, 47}, {16, 999}, {64, 1023}, {256, 3}};
        for (auto &v : vert) {
            TestFFTVert_Pow2<float>(v[0], v[1]);
            TestFFTVert_Pow2<double>(v[0], v[1]);
        }
        Test2D<float>(64, 32);
        Test2D<float>(16, 1);
        Test2D<double>(32, 64);
        TestDevicePointers<float>(1024);
        // errors throw instead of asserting
        bool threw = false;
        try {
            genfft::FFT<float> bad(3);
        } catch (const genfft::gb300_error &e) {
            threw = e.status == GFFT_ERR_INVALID_SIZE;
        }
        CHECK(threw, "invalid size must throw");
    } catch (const std::exception &e) {
        std::printf("FAIL: exception %s\n", e.what());
        return 2;
    }
    std::printf("%s: %d failures\n", failures ? "FAILED" : "OK", failures);
    return failures ? 1 : 0;
}
