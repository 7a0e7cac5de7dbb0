// genfft/fft.h -- drop-in replacement for the reference's <genFFT/fft.h>,
// backed by libgenfft_gb300.so (GB300 kernels behind the C ABI in
// genfft_gb300.h).
//
// Same namespace, class templates and method names as mzient/genFFT:
//   genfft::FFT<T>        transform<inv>, transform_no_scramble<inv>,
//                         transform_real, transform_interleave   (fft.h:56-113)
//   genfft::FFTVert<T>    transform<inv>, transform_no_scramble<inv> (fft.h:115-171)
//   genfft::DIT<T>        apply                                  (fft.h:173-196)
//   genfft::FFT2D<T>      transform<inv>                          (fft.h:198-245)
//   genfft::RealFFT<T>    forward(out, in, half)                  (FFTReal.h:186-221)
//   genfft::RealFFT2D<T>  forward, forward_2x                     (FFTReal.h:69-184)
//   genfft::separate_2x_real_FFT                                  (FFTReal.h:34-66)
// plus the README's forward/inverse spelling (README.txt:28-31) and batched
// overloads.  T is float or double.
//
// Semantics follow the reference: calls are synchronous and the inverse is
// unscaled.  Buffers may be host memory (as with the reference: they are
// staged through device memory owned by the object) or device memory (the
// transform runs in place on the GPU, no copies).  Errors throw
// genfft::gb300_error (the reference asserts instead).
//
// The classes keep the reference's factory template parameters (fft.h:56,
// 117, 173, FFTReal.h:188), defaulting to genfft::backend::{GetImpl,
// GetVertImpl, GetDITImpl}, which here name the GB300 backend
// (gb300_backend.h).  With those factories the classes call the C ABI
// directly (no host bit reversal: the kernels are Stockham auto-sort).  With
// any other factory they run the reference's own algorithm on host
// buffers: bit-reversal copy (FFTUtil.h:51-98), then the factory's backend
// object, as fft.h:80-171 and FFTReal.h:204-213 do.
#ifndef GENFFT_GB300_FFT_H
#define GENFFT_GB300_FFT_H

#include <cuda_runtime.h>

#include <complex>
#include <cstddef>
#include <memory>
#include <string>

#include "gb300_backend.h"

namespace genfft {

/// the backend alias set of the reference (FFTBackend.h:40-70), here the GPU
namespace backend {
using gb300::GetDITImpl;
using gb300::GetImpl;
using gb300::GetVertImpl;
}  // namespace backend

namespace gb300 {
namespace detail {
inline int rev_bits(int i, int bits)
{
    int r = 0;
    for (int b = 0; b < bits; b++) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}
inline int log2i(int n)
{
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}
// out[rev(i)] = f(i) for i < n: the reference's scramble (FFTUtil.h:51-83)
template <class F>
void scramble_by(int n, F &&f)
{
    const int bits = log2i(n);
    for (int i = 0; i < n; i++) f(rev_bits(i, bits), i);
}
}  // namespace detail
}  // namespace gb300

/// 1D FFT of densely packed data (reference fft.h:56-113)
template <class T, FFTImplFactory<T> *factory = backend::GetImpl>
struct FFT {
    /// true when the factory is the GB300 backend: the direct C-ABI path
    static constexpr bool native = factory == static_cast<FFTImplFactory<T> *>(&gb300::GetImpl<T>);

    FFT() = default;
    explicit FFT(int n) : n(n)
    {
        gb300::check(n > 0 && (n & (n - 1)) == 0 ? GFFT_OK : GFFT_ERR_INVALID_SIZE);
        if (!native) impl = factory(n, T());
    }

    /// in place, bit-reversed input, natural-order output (fft.h:69-73)
    template <bool inv>
    void transform_no_scramble(std::complex<T> *inout, long long batch = 1)
    {
        if (!native) {
            for (long long b = 0; b < batch; b++) impl->template transform<inv>((T *)(inout + b * n));
            return;
        }
        const size_t bytes = sizeof(std::complex<T>) * (size_t)n * batch;
        gb300::staged(inout, bytes, inout, bytes, out_, in_, [&](void *o, const void *) {
            gb300::check(gfft_fft_transform_no_scramble(gb300::dtype<T>(), n, batch, inv, o, nullptr));
        });
    }

    /// out-of-place natural-order transform (fft.h:80-85); batch dense rows
    template <bool inv>
    void transform(std::complex<T> *out, const std::complex<T> *in, long long batch = 1)
    {
        if (!native) {
            for (long long b = 0; b < batch; b++) {
                std::complex<T> *o = out + b * n;
                const std::complex<T> *i = in + b * n;
                gb300::detail::scramble_by(n, [&](int r, int k) { o[r] = i[k]; });
                impl->template transform<inv>((T *)o);
            }
            return;
        }
        const size_t bytes = sizeof(std::complex<T>) * (size_t)n * batch;
        gb300::staged(out, bytes, in, bytes, out_, in_, [&](void *o, const void *i) {
            gb300::check(gfft_fft_transform(gb300::dtype<T>(), n, batch, inv, o, i, nullptr));
        });
    }

    /// README spelling (README.txt:28-31): forward, unscaled inverse
    void forward(std::complex<T> *out, const std::complex<T> *in, long long batch = 1) { transform<false>(out, in, batch); }
    void inverse(std::complex<T> *out, const std::complex<T> *in, long long batch = 1) { transform<true>(out, in, batch); }
    void forward(T *out, const T *in) { transform<false>((std::complex<T> *)out, (const std::complex<T> *)in); }
    void inverse(T *out, const T *in) { transform<true>((std::complex<T> *)out, (const std::complex<T> *)in); }

    /// full complex spectrum of n reals (fft.h:90-94)
    void transform_real(std::complex<T> *out, const T *in, long long batch = 1)
    {
        if (!native) {
            for (long long b = 0; b < batch; b++) {
                std::complex<T> *o = out + b * n;
                const T *i = in + b * n;
                gb300::detail::scramble_by(n, [&](int r, int k) { o[r] = std::complex<T>(i[k], T(0)); });
                impl->template transform<false>((T *)o);
            }
            return;
        }
        gb300::staged(out, sizeof(std::complex<T>) * (size_t)n * batch, in, sizeof(T) * (size_t)n * batch, out_, in_,
                      [&](void *o, const void *i) {
                          gb300::check(gfft_fft_transform_real(gb300::dtype<T>(), n, batch, o, i, nullptr));
                      });
    }

    /// FFT of in1 + i*in2; separate with separate_2x_real_FFT (fft.h:100-105)
    void transform_interleave(std::complex<T> *out, const T *in1, const T *in2)
    {
        if (!native) {
            gb300::detail::scramble_by(n, [&](int r, int k) { out[r] = std::complex<T>(in1[k], in2[k]); });
            impl->template transform<false>((T *)out);
            return;
        }
        const bool dev = gb300::on_device(in1) && gb300::on_device(in2);
        const T *a = in1, *b = in2;
        if (!dev) {
            T *s = (T *)in2_.get(2 * sizeof(T) * n);
            gb300::check_cuda(cudaMemcpy(s, in1, sizeof(T) * n, cudaMemcpyHostToDevice));
            gb300::check_cuda(cudaMemcpy(s + n, in2, sizeof(T) * n, cudaMemcpyHostToDevice));
            a = s;
            b = s + n;
        }
        gb300::staged(out, sizeof(std::complex<T>) * n, a, sizeof(T) * n, out_, in_, [&](void *o, const void *) {
            gb300::check(gfft_fft_transform_interleave(gb300::dtype<T>(), n, o, a, b, nullptr));
        });
    }

    int size() const noexcept { return n; }
    explicit operator bool() const noexcept { return n > 0; }

private:
    int n = 0;
    FFTImplPtr<T> impl;  // the factory's backend object (non-GB300 factories)
    gb300::Buffer in_, out_, in2_;
};

/// Column-wise FFT of `cols` columns of n rows (fft.h:115-171)
template <class T, FFTVertImplFactory<T> *factory = backend::GetVertImpl>
struct FFTVert {
    static constexpr bool native = factory == static_cast<FFTVertImplFactory<T> *>(&gb300::GetVertImpl<T>);

    FFTVert() = default;
    explicit FFTVert(int n) : n(n)
    {
        gb300::check(n > 0 && (n & (n - 1)) == 0 ? GFFT_OK : GFFT_ERR_INVALID_SIZE);
        if (!native) impl = factory(n, T());
    }

    template <bool inv>
    void transform_no_scramble(std::complex<T> *data, stride_t stride, index_t cols)
    {
        if (!native) {
            impl->template transform<inv>((T *)data, (int)(2 * stride), cols);
            return;
        }
        const size_t bytes = sizeof(std::complex<T>) * (size_t)n * stride;
        gb300::staged(data, bytes, data, bytes, out_, in_, [&](void *o, const void *) {
            gb300::check(gfft_vert_transform_no_scramble(gb300::dtype<T>(), n, inv, o, stride, cols, nullptr));
        });
    }

    template <bool inv>
    void transform(std::complex<T> *out, stride_t out_stride, const std::complex<T> *in, stride_t in_stride,
                   index_t cols)
    {
        if (!native) {
            // rows in bit-reversed order (scramble_rows, FFTUtil.h:85-98)
            gb300::detail::scramble_by(n, [&](int r, int k) {
                for (index_t c = 0; c < cols; c++) out[r * out_stride + c] = in[k * in_stride + c];
            });
            impl->template transform<inv>((T *)out, (int)(2 * out_stride), cols);
            return;
        }
        gb300::staged(out, sizeof(std::complex<T>) * (size_t)n * out_stride, in,
                      sizeof(std::complex<T>) * (size_t)n * in_stride, out_, in_,
                      [&](void *o, const void *i) {
                          gb300::check(gfft_vert_transform(gb300::dtype<T>(), n, inv, o, out_stride, i, in_stride,
                                                           cols, nullptr));
                      }, /*out_preload=*/out_stride > cols);
    }

    template <bool inv>
    void transform(std::complex<T> *out, const std::complex<T> *in, index_t cols)
    {
        transform<inv>(out, cols, in, cols, cols);
    }

    int size() const noexcept { return n; }
    explicit operator bool() const noexcept { return n > 0; }

private:
    int n = 0;
    FFTVertImplPtr<T> impl;
    gb300::Buffer in_, out_;
};

/// Real-FFT adjustment of an n/2-point spectrum (fft.h:173-196)
template <class T, FFTDITImplFactory<T> *factory = backend::GetDITImpl>
class DIT {
public:
    static constexpr bool native = factory == static_cast<FFTDITImplFactory<T> *>(&gb300::GetDITImpl<T>);

    DIT() = default;
    explicit DIT(int n) : n(n)
    {
        if (!native) impl = factory(n, T());
    }

    void apply(std::complex<T> *out, const std::complex<T> *in, bool half)
    {
        if (!native) {
            impl->apply((T *)out, (const T *)in, half);
            return;
        }
        const size_t in_bytes = sizeof(std::complex<T>) * (size_t)(n > 1 ? n / 2 : 1);
        const size_t out_bytes = sizeof(std::complex<T>) * (size_t)(half ? n / 2 + 1 : n);
        gb300::staged(out, out_bytes, in, in_bytes, out_, in_, [&](void *o, const void *i) {
            gb300::check(gfft_dit_apply(gb300::dtype<T>(), n, o, i, half, nullptr));
        });
    }
    void apply(T *out, const T *in, bool half) { apply((std::complex<T> *)out, (const std::complex<T> *)in, half); }

    int size() const noexcept { return n; }
    explicit operator bool() const noexcept { return n > 0; }

private:
    int n = 0;
    FFTDITImplPtr<T> impl;
    gb300::Buffer in_, out_;
};

/// 2D FFT, row-major [height][width] (fft.h:198-245)
template <class T>
class FFT2D {
public:
    FFT2D() = default;
    FFT2D(int width, int height) : w(width), h(height) {}

    template <bool inv>
    void transform(std::complex<T> *out, stride_t out_stride, const std::complex<T> *in, stride_t in_stride)
    {
        gb300::staged(out, sizeof(std::complex<T>) * (size_t)h * out_stride, in,
                      sizeof(std::complex<T>) * (size_t)h * in_stride, out_, in_,
                      [&](void *o, const void *i) {
                          gb300::check(gfft_fft2d_transform(gb300::dtype<T>(), w, h, inv, o, out_stride, i, in_stride,
                                                            nullptr));
                      }, /*out_preload=*/out_stride > w);
    }

    int cols() const noexcept { return w; }
    int rows() const noexcept { return h; }
    explicit operator bool() const noexcept { return w > 0 && h > 0; }

private:
    int w = 0, h = 0;
    gb300::Buffer in_, out_;
};

/// Recovers two real spectra from one interleaved transform (FFTReal.h:34-66)
template <class T>
void separate_2x_real_FFT(std::complex<T> *out1, std::complex<T> *out2, const std::complex<T> *in, int N)
{
    const size_t bytes = sizeof(std::complex<T>) * (size_t)N;
    if (gb300::on_device(out1) && gb300::on_device(out2) && gb300::on_device(in)) {
        gb300::check(gfft_separate_2x_real_fft(gb300::dtype<T>(), N, out1, out2, in, nullptr));
        gb300::check_cuda(cudaDeviceSynchronize());
        return;
    }
    gb300::Buffer b;
    char *d = (char *)b.get(3 * bytes);
    gb300::check_cuda(cudaMemcpy(d, in, bytes, cudaMemcpyHostToDevice));
    gb300::check(gfft_separate_2x_real_fft(gb300::dtype<T>(), N, d + bytes, d + 2 * bytes, d, nullptr));
    gb300::check_cuda(cudaMemcpy(out1, d + bytes, bytes, cudaMemcpyDeviceToHost));
    gb300::check_cuda(cudaMemcpy(out2, d + 2 * bytes, bytes, cudaMemcpyDeviceToHost));
}

/// 1D FFT of real data (FFTReal.h:186-221); the output buffer holds n bins
template <class T, FFTImplFactory<T> *factory = backend::GetImpl, FFTDITImplFactory<T> *dit_factory = backend::GetDITImpl>
struct RealFFT {
    static constexpr bool native = factory == static_cast<FFTImplFactory<T> *>(&gb300::GetImpl<T>) &&
                                   dit_factory == static_cast<FFTDITImplFactory<T> *>(&gb300::GetDITImpl<T>);

    RealFFT() = default;
    RealFFT(int n) : n(n)
    {
        if (!native && n > 1) {
            impl = factory(n / 2, T());
            dit = dit_factory(n, T());
        }
    }

    void forward(std::complex<T> *out, const T *in, bool half, long long batch = 1)
    {
        if (!native) {
            for (long long b = 0; b < batch; b++) {
                std::complex<T> *o = out + b * n;
                const T *i = in + b * n;
                if (n == 1) {
                    o[0] = i[0];
                    continue;
                }
                // n reals as n/2 complex, bit-reversed, transformed, adjusted
                gb300::detail::scramble_by(n / 2, [&](int r, int k) { o[r] = std::complex<T>(i[2 * k], i[2 * k + 1]); });
                impl->forward((T *)o);
                dit->apply((T *)o, (const T *)o, half);
            }
            return;
        }
        // half mode writes n/2+1 bins per transform and leaves the rest of
        // each n-element output slot untouched, like the reference
        gb300::staged(out, sizeof(std::complex<T>) * (size_t)n * batch, in, sizeof(T) * (size_t)n * batch, out_, in_,
                      [&](void *o, const void *i) {
                          gb300::check(gfft_real_fft_forward(gb300::dtype<T>(), n, batch, o, i, half, nullptr));
                      }, /*out_preload=*/half);
    }

    int size() const noexcept { return n; }

private:
    int n = 0;
    FFTImplPtr<T> impl;
    FFTDITImplPtr<T> dit;
    gb300::Buffer in_, out_;
};

/// 2D FFT of real data, full-width Hermitian output (FFTReal.h:69-184)
template <class T>
class RealFFT2D {
public:
    RealFFT2D() = default;
    RealFFT2D(int width, int height) : w(width), h(height) {}

    /// out_stride in complex elements, in_stride in scalars (FFTReal.h:330-335)
    void forward(std::complex<T> *out, int out_stride, const T *in, int in_stride)
    {
        gb300::staged(out, sizeof(std::complex<T>) * (size_t)h * out_stride, in, sizeof(T) * (size_t)h * in_stride,
                      out_, in_, [&](void *o, const void *i) {
                          gb300::check(gfft_real_fft2d_forward(gb300::dtype<T>(), w, h, o, out_stride, i, in_stride,
                                                               nullptr));
                      }, /*out_preload=*/out_stride > w);
    }

    void forward_2x(std::complex<T> *out, int out_stride, const T *in1, int in_stride1, const T *in2, int in_stride2)
    {
        const bool dev = gb300::on_device(in1) && gb300::on_device(in2);
        const T *a = in1, *b = in2;
        if (!dev) {
            T *s = (T *)in2_.get(sizeof(T) * ((size_t)h * in_stride1 + (size_t)h * in_stride2));
            gb300::check_cuda(cudaMemcpy(s, in1, sizeof(T) * (size_t)h * in_stride1, cudaMemcpyHostToDevice));
            gb300::check_cuda(cudaMemcpy(s + (size_t)h * in_stride1, in2, sizeof(T) * (size_t)h * in_stride2,
                                         cudaMemcpyHostToDevice));
            a = s;
            b = s + (size_t)h * in_stride1;
        }
        gb300::staged(out, sizeof(std::complex<T>) * (size_t)h * out_stride, a, 0, out_, in_,
                      [&](void *o, const void *) {
                          gb300::check(gfft_real_fft2d_forward_2x(gb300::dtype<T>(), w, h, o, out_stride, a,
                                                                  in_stride1, b, in_stride2, nullptr));
                      }, /*out_preload=*/out_stride > w);
    }

    int cols() const { return w; }
    int rows() const { return h; }

private:
    int w = 0, h = 0;
    gb300::Buffer in_, out_, in2_;
};

}  // namespace genfft

#endif  // GENFFT_GB300_FFT_H
