/*
 * genfft_oracle.h -- CPU restatement of genFFT's generic transform path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker and the
 * CPU baseline: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * legs may load it.  The product library (libgenfft_gb300.so) never links
 * or calls it.
 *
 * Every function restates one piece of the reference's scalar ("generic")
 * backend, operation for operation, so that compiled with
 * -ffp-contract=off it reproduces the reference's generic build bit for bit
 * (pinned by tests/golden/, generated from the reference itself).
 *
 * Layout: complex numbers are interleaved {re, im} pairs of T; sizes are in
 * complex elements unless stated otherwise; strides follow the reference's
 * public API (fft.h) -- row strides in complex elements for complex arrays,
 * in scalars for real arrays.
 *
 * The FP64 DFT (gfo_dft_*) is the independent accuracy oracle: double
 * accumulation with exact integer phase reduction (j*k mod n).
 */
#ifndef GENFFT_ORACLE_H
#define GENFFT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* bit-reversal copy of n complex values (FFTUtil.h:51-58 scramble) */
void gfo_scramble_f(float *out, const float *in, int n);
void gfo_scramble_d(double *out, const double *in, int n);

/* in-place radix-2 DIT on bit-reversed data (fft_impl_generic.h:36-120) */
void gfo_fft_inplace_f(float *data, int n, int inv);
void gfo_fft_inplace_d(double *data, int n, int inv);

/* FFT<T>::transform<inv>(out, in): scramble + in-place (fft.h:80-85) */
void gfo_fft_f(float *out, const float *in, int n, int inv);
void gfo_fft_d(double *out, const double *in, int n, int inv);

/* batched out-of-place C2C on nthreads POSIX threads, each thread taking a
 * strided slice of the batch through one shared plan (CPU baseline) */
int gfo_fft_batch_f(float *out, const float *in, int n, long batch, int inv, int nthreads);
int gfo_fft_batch_d(double *out, const double *in, int n, long batch, int inv, int nthreads);

/* FFT<T>::transform_real (fft.h:90-94): real in -> full complex spectrum */
void gfo_fft_real_input_f(float *out, const float *in, int n);
void gfo_fft_real_input_d(double *out, const double *in, int n);

/* FFT<T>::transform_interleave (fft.h:100-105) */
void gfo_fft_interleave_f(float *out, const float *in1, const float *in2, int n);
void gfo_fft_interleave_d(double *out, const double *in1, const double *in2, int n);

/* FFTVert<T>::transform<inv>(out, out_stride, in, in_stride, cols)
 * (fft.h:145-150, FFTUtil.h:60-73, fft_impl_generic.h:124-243) */
void gfo_fft_vert_f(float *out, long out_stride, const float *in, long in_stride,
                    int n, int cols, int inv);
void gfo_fft_vert_d(double *out, long out_stride, const double *in, long in_stride,
                    int n, int cols, int inv);
/* FFTVert<T>::transform_no_scramble<inv>(data, stride, cols) (fft.h:132-136) */
void gfo_fft_vert_inplace_f(float *data, long stride, int n, int cols, int inv);
void gfo_fft_vert_inplace_d(double *data, long stride, int n, int cols, int inv);

/* DIT<T>::apply(out, in, half) -> adjust_DIT_impl (fft_dit_impl_generic.inl:27-61) */
void gfo_dit_f(float *out, const float *in, int n, int half);
void gfo_dit_d(double *out, const double *in, int n, int half);

/* RealFFT<T>::forward(out, in, half) (FFTReal.h:186-221) */
void gfo_real_fft_f(float *out, const float *in, int n, int half);
void gfo_real_fft_d(double *out, const double *in, int n, int half);
int gfo_real_fft_batch_f(float *out, long odist, const float *in, long idist,
                         int n, long batch, int half, int nthreads);

/* separate_2x_real_FFT (FFTReal.h:34-66); out1/out2/in may alias */
void gfo_separate_2x_f(float *out1, float *out2, const float *in, int n);
void gfo_separate_2x_d(double *out1, double *out2, const double *in, int n);

/* FFT2D<T>::transform<inv>(out, out_stride, in, in_stride) (fft.h:198-245) */
void gfo_fft2d_f(float *out, long out_stride, const float *in, long in_stride,
                 int width, int height, int inv);
void gfo_fft2d_d(double *out, long out_stride, const double *in, long in_stride,
                 int width, int height, int inv);

/* RealFFT2D<T>::forward(out, out_stride, in, in_stride) (FFTReal.h:83-104) */
void gfo_real_fft2d_f(float *out, long out_stride, const float *in, long in_stride,
                      int width, int height);
void gfo_real_fft2d_d(double *out, long out_stride, const double *in, long in_stride,
                      int width, int height);

/* RealFFT2D<T>::forward_2x (FFTReal.h:114-118, scramble_row_x2 :167-180) */
void gfo_real_fft2d_2x_f(float *out, long out_stride, const float *in1, long in_stride1,
                         const float *in2, long in_stride2, int width, int height);

/* FP64 DFT oracle: out[k] = sum_j in[j] * exp(-+2 pi i jk/n), double
 * accumulation, exact phase.  Computes bins [k0, k0+nbins) only. */
void gfo_dft_d(double *out, const double *in, int n, int inv, int k0, int nbins);
/* same, float input promoted to double */
void gfo_dft_fin(double *out, const float *in, int n, int inv, int k0, int nbins);

/* exact-rounding FP64 FFT (iterative radix-2 with long-double-free exact
 * twiddles) used to check large sizes where the O(n^2) DFT is too slow;
 * validated against gfo_dft_d in the tests. */
void gfo_fft64(double *out, const double *in, int n, int inv);

#ifdef __cplusplus
}
#endif

#endif
