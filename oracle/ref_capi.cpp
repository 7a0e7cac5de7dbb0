// ref_capi.cpp -- a C entry-point shim over the UNMODIFIED reference genFFT
// headers, compiled by oracle/Makefile straight from the reference tree into
// oracle/_ref/.  TEST INFRASTRUCTURE ONLY: it exists to pin the oracle
// (genfft_oracle.c) against the reference itself and, on an x86 host, to
// time the reference's own CPU build as the baseline.  Nothing in the
// product links it.
//
// Two builds of this file:
//   GFR_FORCE_GENERIC  -- the reference's portable scalar backend, i.e. what
//                          FFTBackend.h:37-45 selects on a non-x86 host.  The
//                          x86 feature macros are dropped after the standard
//                          headers are in, so FFTBackend.h takes that branch.
//   (default)           -- the reference's native x86 backend (AVX/FMA when
//                          compiled with -mavx2 -mfma), FFTBackend.h:15-35.

#include <cassert>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

#ifdef GFR_FORCE_GENERIC
#undef __x86_64__
#undef __amd64__
#undef __i386__
#endif

#include <genFFT/fft.h>

using cf = std::complex<float>;
using cd = std::complex<double>;

namespace {

template <class T>
void run_batch(T *out, const T *in, int n, long batch, int inv, int nthreads)
{
    // plan created once, before the threads start (FFTLevel.h:76-88 is not
    // thread-safe); each thread takes a strided slice of the batch.
    genfft::FFT<T> fft(n);
    auto body = [&](int tid) {
        genfft::FFT<T> local = fft;
        for (long b = tid; b < batch; b += nthreads) {
            auto *o = reinterpret_cast<std::complex<T> *>(out) + (size_t)n * b;
            auto *i = reinterpret_cast<const std::complex<T> *>(in) + (size_t)n * b;
            if (inv)
                local.template transform<true>(o, i);
            else
                local.template transform<false>(o, i);
        }
    };
    if (nthreads <= 1) {
        body(0);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back(body, t);
    for (auto &t : th) t.join();
}

}  // namespace

extern "C" {

int gfr_is_generic(void)
{
#ifdef GFR_FORCE_GENERIC
    return 1;
#else
    return 0;
#endif
}

void gfr_fft_f(float *out, const float *in, int n, int inv)
{
    genfft::FFT<float> fft(n);
    if (inv) fft.transform<true>((cf *)out, (const cf *)in);
    else     fft.transform<false>((cf *)out, (const cf *)in);
}

void gfr_fft_d(double *out, const double *in, int n, int inv)
{
    genfft::FFT<double> fft(n);
    if (inv) fft.transform<true>((cd *)out, (const cd *)in);
    else     fft.transform<false>((cd *)out, (const cd *)in);
}

void gfr_fft_no_scramble_f(float *inout, int n, int inv)
{
    genfft::FFT<float> fft(n);
    if (inv) fft.transform_no_scramble<true>((cf *)inout);
    else     fft.transform_no_scramble<false>((cf *)inout);
}

void gfr_fft_real_input_f(float *out, const float *in, int n)
{
    genfft::FFT<float> fft(n);
    fft.transform_real((cf *)out, in);
}

void gfr_fft_interleave_f(float *out, const float *in1, const float *in2, int n)
{
    genfft::FFT<float> fft(n);
    fft.transform_interleave((cf *)out, in1, in2);
}

int gfr_fft_batch_f(float *out, const float *in, int n, long batch, int inv, int nthreads)
{
    run_batch<float>(out, in, n, batch, inv, nthreads);
    return 0;
}

int gfr_fft_batch_d(double *out, const double *in, int n, long batch, int inv, int nthreads)
{
    run_batch<double>(out, in, n, batch, inv, nthreads);
    return 0;
}

void gfr_fft_vert_f(float *out, long os, const float *in, long is, int n, int cols, int inv)
{
    genfft::FFTVert<float> fft(n);
    if (inv) fft.transform<true>((cf *)out, os, (const cf *)in, is, cols);
    else     fft.transform<false>((cf *)out, os, (const cf *)in, is, cols);
}

void gfr_fft_vert_d(double *out, long os, const double *in, long is, int n, int cols, int inv)
{
    genfft::FFTVert<double> fft(n);
    if (inv) fft.transform<true>((cd *)out, os, (const cd *)in, is, cols);
    else     fft.transform<false>((cd *)out, os, (const cd *)in, is, cols);
}

void gfr_dit_f(float *out, const float *in, int n, int half)
{
    genfft::DIT<float> dit(n);
    dit.apply(out, in, half != 0);
}

void gfr_dit_d(double *out, const double *in, int n, int half)
{
    genfft::DIT<double> dit(n);
    dit.apply(out, in, half != 0);
}

void gfr_real_fft_f(float *out, const float *in, int n, int half)
{
    genfft::RealFFT<float> fft(n);
    fft.forward((cf *)out, in, half != 0);
}

void gfr_real_fft_d(double *out, const double *in, int n, int half)
{
    genfft::RealFFT<double> fft(n);
    fft.forward((cd *)out, in, half != 0);
}

int gfr_real_fft_batch_f(float *out, long odist, const float *in, long idist, int n,
                         long batch, int half, int nthreads)
{
    genfft::RealFFT<float> fft(n);
    auto body = [&](int tid) {
        genfft::RealFFT<float> local = fft;
        for (long b = tid; b < batch; b += nthreads)
            local.forward((cf *)out + (size_t)odist * b, in + (size_t)idist * b, half != 0);
    };
    if (nthreads <= 1) {
        body(0);
        return 0;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back(body, t);
    for (auto &t : th) t.join();
    return 0;
}

void gfr_separate_2x_f(float *out1, float *out2, const float *in, int n)
{
    genfft::separate_2x_real_FFT((cf *)out1, (cf *)out2, (const cf *)in, n);
}

void gfr_fft2d_f(float *out, long os, const float *in, long is, int w, int h, int inv)
{
    genfft::FFT2D<float> fft(w, h);
    if (inv) fft.transform<true>((cf *)out, os, (const cf *)in, is);
    else     fft.transform<false>((cf *)out, os, (const cf *)in, is);
}

void gfr_fft2d_d(double *out, long os, const double *in, long is, int w, int h, int inv)
{
    genfft::FFT2D<double> fft(w, h);
    if (inv) fft.transform<true>((cd *)out, os, (const cd *)in, is);
    else     fft.transform<false>((cd *)out, os, (const cd *)in, is);
}

void gfr_real_fft2d_f(float *out, long os, const float *in, long is, int w, int h)
{
    genfft::RealFFT2D<float> fft(w, h);
    fft.forward((cf *)out, (int)os, in, (int)is);
}

void gfr_real_fft2d_d(double *out, long os, const double *in, long is, int w, int h)
{
    genfft::RealFFT2D<double> fft(w, h);
    fft.forward((cd *)out, (int)os, in, (int)is);
}

void gfr_real_fft2d_2x_f(float *out, long os, const float *in1, long is1, const float *in2,
                         long is2, int w, int h)
{
    genfft::RealFFT2D<float> fft(w, h);
    fft.forward_2x((cf *)out, (int)os, in1, (int)is1, in2, (int)is2);
}

}  // extern "C"
