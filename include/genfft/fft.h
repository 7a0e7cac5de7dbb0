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
// transform runs in place on the GPU, no copies).  The factory template
// parameter of the reference classes is not needed: the backend is fixed.
// Errors throw genfft::gb300_error (the reference asserts instead).
#ifndef GENFFT_GB300_FFT_H
#define GENFFT_GB300_FFT_H

#include <cuda_runtime.h>

#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>

#include "../genfft_gb300.h"

namespace genfft {

using stride_t = ptrdiff_t;
using index_t = int;

struct gb300_error : std::runtime_error {
    gfft_status status;
    gb300_error(gfft_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

namespace gb300 {

template <class T>
constexpr int dtype()
{
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "genfft::gb300 supports float and double");
    return sizeof(T) == 4 ? GFFT_F32 : GFFT_F64;
}

inline void check(gfft_status s)
{
    if (s != GFFT_OK) throw gb300_error(s, std::string(gfft_status_string(s)) + ": " + gfft_last_error());
}

inline void check_cuda(cudaError_t e)
{
    if (e != cudaSuccess) throw gb300_error(GFFT_ERR_CUDA, cudaGetErrorString(e));
}

inline bool on_device(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device staging buffer owned by a transform object (grown on demand).
class Buffer {
public:
    Buffer() = default;
    Buffer(const Buffer &) = delete;
    Buffer &operator=(const Buffer &) = delete;
    Buffer(Buffer &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
    ~Buffer() { if (p_) cudaFree(p_); }
    void *get(size_t bytes)
    {
        if (bytes > n_) {
            if (p_) cudaFree(p_);
            p_ = nullptr;
            n_ = 0;
            check_cuda(cudaMalloc(&p_, bytes));
            n_ = bytes;
        }
        return p_;
    }

private:
    void *p_ = nullptr;
    size_t n_ = 0;
};

// Runs `op(dev_out, dev_in)` on device pointers, staging host buffers:
// in_bytes are copied in, out_bytes copied back, then synchronised.
template <class Op>
void staged(void *out, size_t out_bytes, const void *in, size_t in_bytes, Buffer &bo, Buffer &bi, Op op,
            bool out_preload = false)
{
    const bool din = on_device(in), dout = on_device(out);
    const void *dev_in = in;
    void *dev_out = out;
    if (!din) {
        void *b = bi.get(in_bytes);
        check_cuda(cudaMemcpy(b, in, in_bytes, cudaMemcpyHostToDevice));
        dev_in = b;
    }
    if (!dout) {
        dev_out = (in == out && !din) ? const_cast<void *>(dev_in) : bo.get(out_bytes);
        if (out_preload && dev_out != dev_in) check_cuda(cudaMemcpy(dev_out, out, out_bytes, cudaMemcpyHostToDevice));
    }
    op(dev_out, dev_in);
    check_cuda(cudaDeviceSynchronize());
    if (!dout) check_cuda(cudaMemcpy(out, dev_out, out_bytes, cudaMemcpyDeviceToHost));
}

}  // namespace gb300

/// 1D FFT of densely packed data (reference fft.h:56-113)
template <class T>
struct FFT {
    FFT() = default;
    explicit FFT(int n) : n(n) { gb300::check(n > 0 && (n & (n - 1)) == 0 ? GFFT_OK : GFFT_ERR_INVALID_SIZE); }

    /// in place, bit-reversed input, natural-order output (fft.h:69-73)
    template <bool inv>
    void transform_no_scramble(std::complex<T> *inout, long long batch = 1)
    {
        const size_t bytes = sizeof(std::complex<T>) * (size_t)n * batch;
        gb300::staged(inout, bytes, inout, bytes, out_, in_, [&](void *o, const void *) {
            gb300::check(gfft_fft_transform_no_scramble(gb300::dtype<T>(), n, batch, inv, o, nullptr));
        });
    }

    /// out-of-place natural-order transform (fft.h:80-85); batch dense rows
    template <bool inv>
    void transform(std::complex<T> *out, const std::complex<T> *in, long long batch = 1)
    {
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
        gb300::staged(out, sizeof(std::complex<T>) * (size_t)n * batch, in, sizeof(T) * (size_t)n * batch, out_, in_,
                      [&](void *o, const void *i) {
                          gb300::check(gfft_fft_transform_real(gb300::dtype<T>(), n, batch, o, i, nullptr));
                      });
    }

    /// FFT of in1 + i*in2; separate with separate_2x_real_FFT (fft.h:100-105)
    void transform_interleave(std::complex<T> *out, const T *in1, const T *in2)
    {
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
    gb300::Buffer in_, out_, in2_;
};

/// Column-wise FFT of `cols` columns of n rows (fft.h:115-171)
template <class T>
struct FFTVert {
    FFTVert() = default;
    explicit FFTVert(int n) : n(n) { gb300::check(n > 0 && (n & (n - 1)) == 0 ? GFFT_OK : GFFT_ERR_INVALID_SIZE); }

    template <bool inv>
    void transform_no_scramble(std::complex<T> *data, stride_t stride, index_t cols)
    {
        const size_t bytes = sizeof(std::complex<T>) * (size_t)n * stride;
        gb300::staged(data, bytes, data, bytes, out_, in_, [&](void *o, const void *) {
            gb300::check(gfft_vert_transform_no_scramble(gb300::dtype<T>(), n, inv, o, stride, cols, nullptr));
        });
    }

    template <bool inv>
    void transform(std::complex<T> *out, stride_t out_stride, const std::complex<T> *in, stride_t in_stride,
                   index_t cols)
    {
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
    gb300::Buffer in_, out_;
};

/// Real-FFT adjustment of an n/2-point spectrum (fft.h:173-196)
template <class T>
class DIT {
public:
    DIT() = default;
    explicit DIT(int n) : n(n) {}

    void apply(std::complex<T> *out, const std::complex<T> *in, bool half)
    {
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
template <class T>
struct RealFFT {
    RealFFT() = default;
    RealFFT(int n) : n(n) {}

    void forward(std::complex<T> *out, const T *in, bool half, long long batch = 1)
    {
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
