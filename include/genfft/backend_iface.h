// genfft/backend_iface.h -- the backend interface of mzient/genFFT, declared
// with the reference's names and signatures so that a backend written
// against it (gb300_backend.h) plugs into either header set:
//   genfft::impl::FFTBase<T>      forward/inverse(T *data)            FFTLevel.h:43-59
//   genfft::impl::FFTVertBase<T>  forward/inverse(T *, int, int)      FFTLevel.h:102-118
//   genfft::impl::FFTDITBase<T>   apply(T *, const T *, bool) const   FFTDIT.h:43-49
//   genfft::FFTImplPtr / FFTImplFactory and the Vert / DIT variants   fft.h:41-52
//   genfft::stride_t, genfft::index_t                                 FFTTypes.h:35-36
// Each block is skipped when the reference's own header that defines it has
// already been included (its include guard is set), so including the
// reference's <genFFT/fft.h> first and this header (or gb300_backend.h)
// after it is fine.  The other order is not supported.
#ifndef GENFFT_GB300_BACKEND_IFACE_H
#define GENFFT_GB300_BACKEND_IFACE_H

#include <cstddef>
#include <memory>

#ifndef GENFFT_FFT_TYPES_H
namespace genfft {
using stride_t = ptrdiff_t;
using index_t = int;
}  // namespace genfft
#endif

#ifndef GEN_FFT_LEVEL_H
namespace genfft {
namespace impl {

// one row, in place: bit-reversed input, natural-order output, unscaled
template <class T>
struct FFTBase {
    virtual ~FFTBase() = default;
    template <bool inv>
    void transform(T *data)
    {
        if (inv)
            inverse(data);
        else
            forward(data);
    }
    virtual void forward(T *data) = 0;
    virtual void inverse(T *data) = 0;
};

// `columns` columns, in place, rows in bit-reversed order on input; stride
// between rows in scalars (twice the complex stride)
template <class T>
struct FFTVertBase {
    virtual ~FFTVertBase() = default;
    template <bool inv>
    void transform(T *data, int stride, int columns)
    {
        if (inv)
            inverse(data, stride, columns);
        else
            forward(data, stride, columns);
    }
    virtual void forward(T *data, int stride, int columns) = 0;
    virtual void inverse(T *data, int stride, int columns) = 0;
};

}  // namespace impl
}  // namespace genfft
#endif

#ifndef FFT_DIT_H
namespace genfft {
namespace impl {

// real-FFT adjustment of an n/2-point complex spectrum into n/2+1 (half) or
// n bins; out may equal in
template <class T>
struct FFTDITBase {
    virtual ~FFTDITBase() = default;
    virtual void apply(T *out, const T *in, bool half) const noexcept = 0;
};

}  // namespace impl
}  // namespace genfft
#endif

#ifndef GENFFT_FFT_H
namespace genfft {
template <typename T>
using FFTImplPtr = std::shared_ptr<impl::FFTBase<T>>;
template <typename T>
using FFTVertImplPtr = std::shared_ptr<impl::FFTVertBase<T>>;
template <typename T>
using FFTDITImplPtr = std::shared_ptr<impl::FFTDITBase<T>>;
template <typename T>
using FFTImplFactory = FFTImplPtr<T>(int n, T);
template <typename T>
using FFTVertImplFactory = FFTVertImplPtr<T>(int n, T);
template <typename T>
using FFTDITImplFactory = FFTDITImplPtr<T>(int n, T);
}  // namespace genfft
#endif

#endif  // GENFFT_GB300_BACKEND_IFACE_H
