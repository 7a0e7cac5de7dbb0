// seam_test.cpp -- drives the GB300 backend objects of the reference's
// factory seam (genfft/gb300_backend.h) through the backend interface
// declared with the reference's signatures (genfft/backend_iface.h:
// impl::FFTBase, FFTVertBase, FFTDITBase; FFTLevel.h:43-118, FFTDIT.h:43-49),
// and the drop-in classes with a factory given explicitly.
//
//   seam_test <op> <f|d> <n> <cols> <in.bin> <out.bin>
//     fft_fwd / fft_inv   GetImpl(n)->forward/inverse in place (bit-reversed in)
//     vert_fwd / vert_inv GetVertImpl(n)->forward/inverse: n rows x cols,
//                         rows bit-reversed on input, stride 2*cols scalars
//     dit_half / dit_full GetDITImpl(n)->apply(out, in, half), in = n/2 complex
//     cls_fwd             genfft::FFT<T, genfft::gb300::GetImpl>::transform<false>
//     cls_custom          genfft::FFT<T, cpu_dft>::transform<false> with a
//                         naive CPU backend: the reference's host algorithm
//                         (scramble + the factory's object)
// Input and output are raw interleaved complex arrays of T.
#include <genfft/fft.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

// a naive O(n^2) CPU backend in the reference's contract (bit-reversed in,
// natural out, in place), to exercise the drop-in classes' generic path
template <class T>
struct CpuDft : genfft::impl::FFTBase<T> {
    explicit CpuDft(int n) : n(n) {}
    void run(T *d, bool inv)
    {
        int bits = 0;
        while ((1 << bits) < n) bits++;
        std::vector<std::complex<double>> x(n), y(n);
        for (int i = 0; i < n; i++) {
            int r = 0;
            for (int b = 0; b < bits; b++) r |= ((i >> b) & 1) << (bits - 1 - b);
            x[r] = {d[2 * i], d[2 * i + 1]};  // undo the bit reversal
        }
        for (int k = 0; k < n; k++) {
            std::complex<double> s = 0;
            for (int j = 0; j < n; j++) {
                const double a = (inv ? 2 : -2) * M_PI * (double)(((long long)j * k) % n) / n;
                s += x[j] * std::complex<double>(std::cos(a), std::sin(a));
            }
            y[k] = s;
        }
        for (int k = 0; k < n; k++) d[2 * k] = (T)y[k].real(), d[2 * k + 1] = (T)y[k].imag();
    }
    void forward(T *d) override { run(d, false); }
    void inverse(T *d) override { run(d, true); }
    int n;
};
template <class T>
std::shared_ptr<genfft::impl::FFTBase<T>> cpu_dft(int n, T)
{
    return std::make_shared<CpuDft<T>>(n);
}

template <class T>
int run(const std::string &op, int n, int cols, const char *fin, const char *fout)
{
    using C = std::complex<T>;
    FILE *f = std::fopen(fin, "rb");
    if (!f) return 2;
    std::vector<C> in;
    C c;
    while (std::fread(&c, sizeof(C), 1, f) == 1) in.push_back(c);
    std::fclose(f);
    std::vector<C> out;
    if (op == "fft_fwd" || op == "fft_inv") {
        out = in;
        auto impl = genfft::gb300::GetImpl<T>(n, T());
        // the per-size singleton: a second lookup returns the same object
        if (genfft::gb300::GetImpl<T>(n, T()) != impl) return 3;
        if (op == "fft_fwd") impl->forward((T *)out.data());
        else impl->template transform<true>((T *)out.data());
    } else if (op == "vert_fwd" || op == "vert_inv") {
        out = in;
        auto impl = genfft::gb300::GetVertImpl<T>(n, T());
        if (op == "vert_fwd") impl->forward((T *)out.data(), 2 * cols, cols);
        else impl->inverse((T *)out.data(), 2 * cols, cols);
    } else if (op == "dit_half" || op == "dit_full") {
        const bool half = op == "dit_half";
        out.assign(half ? n / 2 + 1 : n, C(0, 0));
        auto impl = genfft::gb300::GetDITImpl<T>(n, T());
        impl->apply((T *)out.data(), (const T *)in.data(), half);
    } else if (op == "cls_fwd") {
        out.assign(in.size(), C(0, 0));
        genfft::FFT<T, genfft::gb300::GetImpl> fft(n);
        fft.template transform<false>(out.data(), in.data());
    } else if (op == "cls_custom") {
        out.assign(in.size(), C(0, 0));
        genfft::FFT<T, cpu_dft<T>> fft(n);
        static_assert(!genfft::FFT<T, cpu_dft<T>>::native, "a custom factory takes the generic path");
        fft.template transform<false>(out.data(), in.data());
    } else {
        return 4;
    }
    f = std::fopen(fout, "wb");
    if (!f) return 2;
    std::fwrite(out.data(), sizeof(C), out.size(), f);
    std::fclose(f);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc != 7) {
        std::fprintf(stderr, "usage: seam_test <op> <f|d> <n> <cols> <in.bin> <out.bin>\n");
        return 1;
    }
    const std::string op = argv[1];
    const int n = std::atoi(argv[3]), cols = std::atoi(argv[4]);
    try {
        return argv[2][0] == 'd' ? run<double>(op, n, cols, argv[5], argv[6]) : run<float>(op, n, cols, argv[5], argv[6]);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 5;
    }
}
