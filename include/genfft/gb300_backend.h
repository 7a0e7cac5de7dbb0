// genfft/gb300_backend.h -- a GB300 backend for the reference library's
// own plug-in seam: the factory template parameter of its user classes,
//   template <class T, FFTImplFactory<T> *factory = backend::GetImpl> struct FFT      (fft.h:56)
//   template <class T, FFTVertImplFactory<T> *factory = ...GetVertImpl> struct FFTVert (fft.h:117)
//   template <class T, FFTDITImplFactory<T> *factory = ...GetDITImpl> class DIT       (fft.h:173)
//   template <class T, ..GetImpl, ..GetDITImpl> struct RealFFT                        (FFTReal.h:188)
// and the alias set genfft::backend::{GetImpl, GetVertImpl, GetDITImpl}
// (FFTBackend.h:40-70).  This header supplies a third set,
//   genfft::gb300::GetImpl / GetVertImpl / GetDITImpl,
// so that reference code can keep its classes and swap the backend:
//   #include <genFFT/fft.h>           // the reference
//   #include <genfft/gb300_backend.h> // this header, after it
//   genfft::FFT<float, genfft::gb300::GetImpl> fft(1 << 20);
// The objects these factories return implement the reference's backend
// contract on the GPU (libgenfft_gb300.so, C ABI in genfft_gb300.h):
//   FFTBase<T>::forward/inverse(data)          in place, bit-reversed input,
//       natural-order output, unscaled            (FFTLevel.h:43-59)
//   FFTVertBase<T>::forward/inverse(data, stride, columns): `columns`
//       columns in place, rows in bit-reversed order on input, stride in
//       scalars                                    (FFTLevel.h:102-118)
//   FFTDITBase<T>::apply(out, in, half)         the real-FFT adjustment of an
//       n/2-point spectrum, out may equal in      (FFTDIT.h:43-49)
// Buffers may be host memory (the reference's convention: staged through
// device memory the object owns, synchronously) or device memory (run in
// place on the GPU).  Like the reference's backends the objects are
// per-size singletons (FFTLevel.h:76-88); here creation is mutex-guarded
// and each object serialises its own calls (its staging buffers are shared).
// Errors throw genfft::gb300_error where the reference asserts; DIT's
// apply is noexcept in the reference, so a failure there aborts the process
// with a message, as a failed assert would.
#ifndef GENFFT_GB300_BACKEND_H
#define GENFFT_GB300_BACKEND_H

#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>

#include "backend_iface.h"
#include "gb300_common.h"

namespace genfft {
namespace gb300 {

inline void check_size(int n)
{
    if (n < 1 || (n & (n - 1)) != 0)
        throw gb300_error(GFFT_ERR_INVALID_SIZE, "genfft::gb300: transform length must be a power of two");
}

/// impl::FFTBase<T> on the GPU: one in-place transform of n complex values
template <class T>
class GpuFFT : public impl::FFTBase<T> {
public:
    explicit GpuFFT(int n) : n_(n) { check_size(n); }
    void forward(T *data) override { run(data, 0); }
    void inverse(T *data) override { run(data, 1); }
    int size() const noexcept { return n_; }

private:
    void run(T *data, int inv)
    {
        std::lock_guard<std::mutex> lk(mu_);
        const size_t bytes = 2 * sizeof(T) * (size_t)n_;
        staged(data, bytes, data, bytes, out_, in_, [&](void *o, const void *) {
            check(gfft_fft_transform_no_scramble(dtype<T>(), n_, 1, inv, o, nullptr));
        });
    }
    int n_;
    std::mutex mu_;
    Buffer in_, out_;
};

/// impl::FFTVertBase<T> on the GPU: n-row column FFTs in place
template <class T>
class GpuFFTVert : public impl::FFTVertBase<T> {
public:
    explicit GpuFFTVert(int n) : n_(n) { check_size(n); }
    void forward(T *data, int stride, int columns) override { run(data, stride, columns, 0); }
    void inverse(T *data, int stride, int columns) override { run(data, stride, columns, 1); }
    int size() const noexcept { return n_; }

private:
    void run(T *data, int stride, int columns, int inv)
    {
        if (stride % 2 != 0 || stride < 2 * columns)
            throw gb300_error(GFFT_ERR_INVALID_VALUE, "genfft::gb300: vertical stride must be an even scalar count "
                                                      "covering the columns");
        if (columns <= 0) return;
        std::lock_guard<std::mutex> lk(mu_);
        // the span the rows occupy: the last row ends after its columns
        const size_t bytes = sizeof(T) * ((size_t)(n_ - 1) * (size_t)stride + 2 * (size_t)columns);
        staged(data, bytes, data, bytes, out_, in_, [&](void *o, const void *) {
            check(gfft_vert_transform_no_scramble(dtype<T>(), n_, inv, o, stride / 2, columns, nullptr));
        });
    }
    int n_;
    std::mutex mu_;
    Buffer in_, out_;
};

/// impl::FFTDITBase<T> on the GPU: n/2 complex in, n/2+1 (half) or n out
template <class T>
class GpuDIT : public impl::FFTDITBase<T> {
public:
    explicit GpuDIT(int n) : n_(n) { check_size(n); }
    void apply(T *out, const T *in, bool half) const noexcept override
    {
        try {
            std::lock_guard<std::mutex> lk(mu_);
            const size_t in_bytes = 2 * sizeof(T) * (size_t)(n_ > 1 ? n_ / 2 : 1);
            const size_t out_bytes = 2 * sizeof(T) * (size_t)(half ? n_ / 2 + 1 : n_);
            if (on_device(out) && on_device(in)) {
                check(gfft_dit_apply(dtype<T>(), n_, out, in, half, nullptr));
                check_cuda(cudaDeviceSynchronize());
                return;
            }
            // one device buffer large enough for either side, so that the
            // in-place call (out == in, as RealFFT::forward makes it) works
            char *d = (char *)buf_.get(in_bytes > out_bytes ? in_bytes : out_bytes);
            check_cuda(cudaMemcpy(d, in, in_bytes, cudaMemcpyDefault));
            check(gfft_dit_apply(dtype<T>(), n_, d, d, half, nullptr));
            check_cuda(cudaDeviceSynchronize());
            check_cuda(cudaMemcpy(out, d, out_bytes, cudaMemcpyDefault));
        } catch (const std::exception &e) {
            std::fprintf(stderr, "genfft::gb300::GpuDIT::apply failed: %s\n", e.what());
            std::abort();
        }
    }
    int size() const noexcept { return n_; }

private:
    int n_;
    mutable std::mutex mu_;
    mutable Buffer buf_;
};

namespace detail {
// per-size singleton cache (the reference keeps one weak_ptr per size,
// FFTLevel.h:76-88); guarded, unlike the reference's
template <class Base, class Impl>
std::shared_ptr<Base> singleton(int n)
{
    static std::mutex mu;
    static std::map<int, std::weak_ptr<Base>> cache;
    std::lock_guard<std::mutex> lk(mu);
    std::shared_ptr<Base> p = cache[n].lock();
    if (!p) {
        p = std::make_shared<Impl>(n);
        cache[n] = p;
    }
    return p;
}
}  // namespace detail

/// factories with the reference's signatures (fft.h:47-52)
template <class T>
std::shared_ptr<impl::FFTBase<T>> GetImpl(int n, T)
{
    return detail::singleton<impl::FFTBase<T>, GpuFFT<T>>(n);
}

template <class T>
std::shared_ptr<impl::FFTVertBase<T>> GetVertImpl(int n, T)
{
    return detail::singleton<impl::FFTVertBase<T>, GpuFFTVert<T>>(n);
}

template <class T>
std::shared_ptr<impl::FFTDITBase<T>> GetDITImpl(int n, T)
{
    return detail::singleton<impl::FFTDITBase<T>, GpuDIT<T>>(n);
}

}  // namespace gb300
}  // namespace genfft

#endif  // GENFFT_GB300_BACKEND_H
