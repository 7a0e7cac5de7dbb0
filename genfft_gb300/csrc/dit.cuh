// dit.cuh -- the real-FFT post-twiddle ("DIT adjustment") of one bin pair.
//
// The reference (DIT<T>::apply, fft.h:173-196; adjust_DIT_impl,
// fft_dit_impl_generic.inl:27-61) turns the n/2-point complex FFT Z of the
// n reals read as n/2 complex values into the spectrum F of the reals:
//   F_k = E_k - t_k * O_k,  E_k = (Z_k + conj Z_j) / 2,  O_k = (Z_k - conj Z_j) / 2,
// with j = n/2 - k (mod n/2) and t_k = sin(2 pi k/n) + i cos(2 pi k/n)
// (DITTwiddle, FFTTwiddle.h:116-127), which equals -W_n^k / i: the usual
// E_k + W_n^k (Z_k - conj Z_j) / (2 i).
#pragma once

#include "common.cuh"

namespace gfft {

// F_k from Z_k, Z_j and the DIT twiddle t_k = (sin, cos) = dtw[k]
template <typename T>
__device__ __forceinline__ cpx<T> dit_value(cpx<T> zk, cpx<T> zj, cpx<T> t)
{
    const T h = (T)0.5;
    const cpx<T> e{(zk.x + zj.x) * h, (zk.y - zj.y) * h};
    const cpx<T> o{(zk.x - zj.x) * h, (zk.y + zj.y) * h};
    const cpx<T> to = cmul(t, o);
    return {e.x - to.x, e.y - to.y};
}

}  // namespace gfft
