/*
 * genfft_oracle.c -- CPU restatement of genFFT's generic (scalar) backend.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the CPU baseline.  The
 * product library never links or calls this file.
 *
 * Build with -O3 -ffp-contract=off (oracle/Makefile): every arithmetic
 * operation below follows the reference's generic backend in the same order,
 * so the results are bit-identical to the reference compiled without FMA
 * contraction.  Reference citations are file:line within mzient/genFFT.
 */
#define _GNU_SOURCE
#include "genfft_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static int ilog2(int n)
{
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

/* ------------------------------------------------------------------------ */
/* Twiddle tables: Twiddle<N,T> (FFTTwiddle.h:37-52) holds, for one
 * butterfly level of N complex points, t[i] = cos(pi*i/N), t[i+1] =
 * -sin(pi*i/N) for even i < N, computed in double and rounded to T.
 * One table per level; level L (N = 2^L complex points) has N scalars.   */
#define DEFINE_TWIDDLES(T, SUF)                                                 \
    static T **tw_build_##SUF(int logn)                                         \
    {                                                                           \
        T **lv = (T **)calloc((size_t)logn + 1, sizeof(T *));                  \
        for (int L = 3; L <= logn; L++) {                                       \
            int N = 1 << L;                                                     \
            T *t = (T *)malloc(sizeof(T) * (size_t)N);                          \
            for (int i = 0; i < N; i += 2) {                                    \
                t[i] = (T)cos(M_PI * i / N);                                    \
                t[i + 1] = (T)(-sin(M_PI * i / N));                             \
            }                                                                   \
            lv[L] = t;                                                          \
        }                                                                       \
        return lv;                                                              \
    }                                                                           \
    static void tw_free_##SUF(T **lv, int logn)                                 \
    {                                                                           \
        for (int L = 0; L <= logn; L++) free(lv[L]);                            \
        free(lv);                                                               \
    }

DEFINE_TWIDDLES(float, f)
DEFINE_TWIDDLES(double, d)

/* ------------------------------------------------------------------------ */
/* scramble (FFTUtil.h:51-83): recursive bit-reversal copy; out is written
 * with a stride (in elements of the destination type).                      */
#define DEFINE_SCRAMBLE(T, SUF)                                                 \
    static void scr_##SUF(T *out, const T *in, int N, long stride)             \
    {                                                                           \
        /* complex elements: out/in point at {re,im} pairs */                   \
        if (N == 1) {                                                           \
            out[0] = in[0];                                                     \
            out[1] = in[1];                                                     \
            return;                                                             \
        }                                                                       \
        scr_##SUF(out, in, N >> 1, stride << 1);                                \
        scr_##SUF(out + 2 * stride, in + 2 * (N >> 1), N >> 1, stride << 1);    \
    }                                                                           \
    /* scalar version: used by transform_interleave / RealFFT2D leaves,     */ \
    /* which scramble T values into every other scalar slot of the output.  */ \
    static void scr_scalar_##SUF(T *out, const T *in, int N, long stride)      \
    {                                                                           \
        if (N == 1) {                                                           \
            out[0] = in[0];                                                     \
            return;                                                             \
        }                                                                       \
        scr_scalar_##SUF(out, in, N >> 1, stride << 1);                         \
        scr_scalar_##SUF(out + stride, in + (N >> 1), N >> 1, stride << 1);     \
    }                                                                           \
    /* real -> complex promotion: *out = *in with out complex, in real     */  \
    static void scr_r2c_##SUF(T *out, const T *in, int N, long stride)         \
    {                                                                           \
        if (N == 1) {                                                           \
            out[0] = in[0];                                                     \
            out[1] = (T)0;                                                      \
            return;                                                             \
        }                                                                       \
        scr_r2c_##SUF(out, in, N >> 1, stride << 1);                            \
        scr_r2c_##SUF(out + 2 * stride, in + (N >> 1), N >> 1, stride << 1);    \
    }                                                                           \
    void gfo_scramble_##SUF(T *out, const T *in, int n)                         \
    {                                                                           \
        if (n > 0) scr_##SUF(out, in, n, 1);                                    \
    }

DEFINE_SCRAMBLE(float, f)
DEFINE_SCRAMBLE(double, d)

/* ------------------------------------------------------------------------ */
/* In-place radix-2 DIT, FFTGeneric<N,T>::transform_impl
 * (fft_impl_generic.h:36-63), with the N=4 (:66-98), N=2 (:100-113) and
 * N=1 (:115-120) leaves.  Here N is the number of complex points of the
 * level, `data` points at N complex values in bit-reversed order.          */
#define DEFINE_FFT(T, SUF)                                                      \
    static void fft_rec_##SUF(T *d, int L, int inv, T *const *tw)               \
    {                                                                           \
        if (L == 0) return;                                                     \
        if (L == 1) {                                                           \
            T tr = d[2], ti = d[3];                                             \
            d[2] = d[0] - tr;                                                   \
            d[3] = d[1] - ti;                                                   \
            d[0] += tr;                                                         \
            d[1] += ti;                                                         \
            return;                                                             \
        }                                                                       \
        if (L == 2) {                                                           \
            T tr = d[2], ti = d[3];                                             \
            d[2] = d[0] - tr;                                                   \
            d[3] = d[1] - ti;                                                   \
            d[0] += tr;                                                         \
            d[1] += ti;                                                         \
            tr = d[6];                                                          \
            ti = d[7];                                                          \
            d[6] = inv ? ti - d[5] : d[5] - ti;                                 \
            d[7] = inv ? d[4] - tr : tr - d[4];                                 \
            d[4] += tr;                                                         \
            d[5] += ti;                                                         \
            tr = d[4];                                                          \
            ti = d[5];                                                          \
            d[4] = d[0] - tr;                                                   \
            d[5] = d[1] - ti;                                                   \
            d[0] += tr;                                                         \
            d[1] += ti;                                                         \
            tr = d[6];                                                          \
            ti = d[7];                                                          \
            d[6] = d[2] - tr;                                                   \
            d[7] = d[3] - ti;                                                   \
            d[2] += tr;                                                         \
            d[3] += ti;                                                         \
            return;                                                             \
        }                                                                       \
        const int N = 1 << L; /* complex points; N scalars per half */          \
        fft_rec_##SUF(d, L - 1, inv, tw);                                       \
        fft_rec_##SUF(d + N, L - 1, inv, tw);                                   \
        const T *t = tw[L];                                                     \
        for (int i = 0; i < N; i += 2) {                                        \
            T wr = t[i], wi = t[i + 1];                                         \
            T tempr = inv ? d[i + N] * wr + d[i + N + 1] * wi                   \
                          : d[i + N] * wr - d[i + N + 1] * wi;                  \
            T tempi = inv ? d[i + N + 1] * wr - d[i + N] * wi                   \
                          : d[i + N] * wi + d[i + N + 1] * wr;                  \
            d[i + N] = d[i] - tempr;                                            \
            d[i + N + 1] = d[i + 1] - tempi;                                    \
            d[i] += tempr;                                                      \
            d[i + 1] += tempi;                                                  \
        }                                                                       \
    }                                                                           \
    void gfo_fft_inplace_##SUF(T *data, int n, int inv)                         \
    {                                                                           \
        int L = ilog2(n);                                                       \
        T **tw = tw_build_##SUF(L);                                             \
        fft_rec_##SUF(data, L, inv, tw);                                        \
        tw_free_##SUF(tw, L);                                                   \
    }                                                                           \
    void gfo_fft_##SUF(T *out, const T *in, int n, int inv)                     \
    {                                                                           \
        int L = ilog2(n);                                                       \
        T **tw = tw_build_##SUF(L);                                             \
        gfo_scramble_##SUF(out, in, n);                                         \
        fft_rec_##SUF(out, L, inv, tw);                                         \
        tw_free_##SUF(tw, L);                                                   \
    }                                                                           \
    void gfo_fft_real_input_##SUF(T *out, const T *in, int n)                   \
    {                                                                           \
        int L = ilog2(n);                                                       \
        T **tw = tw_build_##SUF(L);                                             \
        if (n > 0) scr_r2c_##SUF(out, in, n, 1);                                \
        fft_rec_##SUF(out, L, 0, tw);                                           \
        tw_free_##SUF(tw, L);                                                   \
    }                                                                           \
    void gfo_fft_interleave_##SUF(T *out, const T *in1, const T *in2, int n)    \
    {                                                                           \
        int L = ilog2(n);                                                       \
        T **tw = tw_build_##SUF(L);                                             \
        scr_scalar_##SUF(out, in1, n, 2);                                       \
        scr_scalar_##SUF(out + 1, in2, n, 2);                                   \
        fft_rec_##SUF(out, L, 0, tw);                                           \
        tw_free_##SUF(tw, L);                                                   \
    }

DEFINE_FFT(float, f)
DEFINE_FFT(double, d)

/* ------------------------------------------------------------------------ */
/* Batched CPU runner: each of nthreads threads takes batch items
 * t, t+nthreads, ... through one shared twiddle set (built before the
 * threads start, as the reference's singleton creation is not thread-safe,
 * FFTLevel.h:76-88).                                                        */
typedef struct {
    void *out;
    const void *in;
    int n, inv, L, tid, nthreads, kind, half;
    long batch, idist, odist;
    void *tw;
} batch_job;

static void *batch_worker(void *arg)
{
    batch_job *j = (batch_job *)arg;
    for (long b = j->tid; b < j->batch; b += j->nthreads) {
        if (j->kind == 0) {
            float *o = (float *)j->out + 2 * (size_t)j->n * b;
            const float *i = (const float *)j->in + 2 * (size_t)j->n * b;
            gfo_scramble_f(o, i, j->n);
            fft_rec_f(o, j->L, j->inv, (float *const *)j->tw);
        } else if (j->kind == 1) {
            double *o = (double *)j->out + 2 * (size_t)j->n * b;
            const double *i = (const double *)j->in + 2 * (size_t)j->n * b;
            gfo_scramble_d(o, i, j->n);
            fft_rec_d(o, j->L, j->inv, (double *const *)j->tw);
        } else {
            float *o = (float *)j->out + 2 * (size_t)j->odist * b;
            const float *i = (const float *)j->in + (size_t)j->idist * b;
            gfo_real_fft_f(o, i, j->n, j->half);
        }
    }
    return NULL;
}

static int run_batch(batch_job proto, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    batch_job *jobs = (batch_job *)malloc(sizeof(batch_job) * (size_t)nthreads);
    int rc = 0, started = 0;
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = proto;
        jobs[t].tid = t;
        jobs[t].nthreads = nthreads;
        if (nthreads == 1) {
            batch_worker(&jobs[t]);
        } else if (pthread_create(&th[t], NULL, batch_worker, &jobs[t]) != 0) {
            rc = -1;
            break;
        } else {
            started++;
        }
    }
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
    return rc;
}

int gfo_fft_batch_f(float *out, const float *in, int n, long batch, int inv, int nthreads)
{
    batch_job p;
    memset(&p, 0, sizeof p);
    p.out = out; p.in = in; p.n = n; p.inv = inv; p.batch = batch; p.kind = 0;
    p.L = ilog2(n);
    float **tw = tw_build_f(p.L);
    p.tw = tw;
    int rc = run_batch(p, nthreads);
    tw_free_f(tw, p.L);
    return rc;
}

int gfo_fft_batch_d(double *out, const double *in, int n, long batch, int inv, int nthreads)
{
    batch_job p;
    memset(&p, 0, sizeof p);
    p.out = out; p.in = in; p.n = n; p.inv = inv; p.batch = batch; p.kind = 1;
    p.L = ilog2(n);
    double **tw = tw_build_d(p.L);
    p.tw = tw;
    int rc = run_batch(p, nthreads);
    tw_free_d(tw, p.L);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Column FFT.  FFTVertGeneric<N,T> (fft_impl_generic.h:124-243) performs,
 * per column, exactly the operations of FFTGeneric<N,T> (the column-span
 * loop only changes the visiting order), so each column is transformed by
 * the 1D recursion on a gathered copy.  scramble_rows (FFTUtil.h:60-73)
 * moves input row r to output row bitrev(r).                                */
#define DEFINE_VERT(T, SUF)                                                     \
    static void vert_cols_##SUF(T *data, long stride, int n, int cols, int inv, \
                                T *const *tw, int L)                            \
    {                                                                           \
        T *col = (T *)malloc(sizeof(T) * 2 * (size_t)(n ? n : 1));             \
        for (int c = 0; c < cols; c++) {                                        \
            for (int r = 0; r < n; r++) {                                       \
                col[2 * r] = data[2 * (r * stride + c)];                        \
                col[2 * r + 1] = data[2 * (r * stride + c) + 1];                \
            }                                                                   \
            fft_rec_##SUF(col, L, inv, tw);                                     \
            for (int r = 0; r < n; r++) {                                       \
                data[2 * (r * stride + c)] = col[2 * r];                        \
                data[2 * (r * stride + c) + 1] = col[2 * r + 1];                \
            }                                                                   \
        }                                                                       \
        free(col);                                                              \
    }                                                                           \
    void gfo_fft_vert_inplace_##SUF(T *data, long stride, int n, int cols, int inv) \
    {                                                                           \
        int L = ilog2(n);                                                       \
        T **tw = tw_build_##SUF(L);                                             \
        vert_cols_##SUF(data, stride, n, cols, inv, tw, L);                     \
        tw_free_##SUF(tw, L);                                                   \
    }                                                                           \
    static void scr_rows_##SUF(T *out, long os, const T *in, long is, int rows, \
                               int cols)                                        \
    {                                                                           \
        if (rows == 1) {                                                        \
            memcpy(out, in, sizeof(T) * 2 * (size_t)cols);                      \
            return;                                                             \
        }                                                                       \
        scr_rows_##SUF(out, 2 * os, in, is, rows / 2, cols);                    \
        scr_rows_##SUF(out + 2 * os, 2 * os, in + 2 * (rows / 2) * is, is,      \
                       rows / 2, cols);                                         \
    }                                                                           \
    void gfo_fft_vert_##SUF(T *out, long out_stride, const T *in, long in_stride, \
                            int n, int cols, int inv)                           \
    {                                                                           \
        scr_rows_##SUF(out, out_stride, in, in_stride, n, cols);                \
        gfo_fft_vert_inplace_##SUF(out, out_stride, n, cols, inv);              \
    }

DEFINE_VERT(float, f)
DEFINE_VERT(double, d)

/* ------------------------------------------------------------------------ */
/* Real-FFT post-pass adjust_DIT_impl (fft_dit_impl_generic.inl:27-61) with
 * DITTwiddle<N,T> (FFTTwiddle.h:96-128): t[i] = sin(pi*i/N),
 * t[i+1] = cos(pi*i/N) for even i <= N/2, in double rounded to T.
 * Complex products follow std::complex: (a*c - b*d, a*d + b*c).            */
#define DEFINE_DIT(T, SUF)                                                      \
    void gfo_dit_##SUF(T *F, const T *Z, int N, int half)                       \
    {                                                                           \
        T zeroval = Z[0] + Z[1];                                                \
        if (N == 1) {                                                           \
            F[0] = zeroval;                                                     \
            F[1] = (T)0;                                                        \
            return;                                                             \
        }                                                                       \
        T centerval = Z[0] - Z[1];                                              \
        if (N == 2) {                                                           \
            F[0] = zeroval;                                                     \
            F[1] = (T)0;                                                        \
            F[2] = centerval;                                                   \
            F[3] = (T)0;                                                        \
            return;                                                             \
        }                                                                       \
        int halfN = N >> 1;                                                     \
        T *tw = (T *)malloc(sizeof(T) * (size_t)(halfN + 4));                   \
        for (int i = 0; i <= halfN; i += 2) {                                   \
            tw[i] = (T)sin(M_PI * i / N);                                       \
            tw[i + 1] = (T)cos(M_PI * i / N);                                   \
        }                                                                       \
        F[2 * halfN] = Z[0];                                                    \
        F[2 * halfN + 1] = Z[1];                                                \
        T qre = Z[2 * (halfN / 2)], qim = -Z[2 * (halfN / 2) + 1];              \
        for (int i = 1, j = halfN - 1; i < halfN / 2; i++, j--) {               \
            T zir = Z[2 * i], zii = Z[2 * i + 1];                               \
            T zjr = Z[2 * j], zji = Z[2 * j + 1];                               \
            T er = (zir + zjr) * (T)0.5, ei = (zii + -zji) * (T)0.5;            \
            T orr = (zir - zjr) * (T)0.5, oi = (zii - -zji) * (T)0.5;           \
            T tr = tw[2 * i], ti = tw[2 * i + 1];                               \
            T pr = tr * orr - ti * oi, pi = tr * oi + ti * orr;                 \
            F[2 * i] = er - pr;                                                 \
            F[2 * i + 1] = ei - pi;                                             \
            F[2 * j] = er + pr;                                                 \
            F[2 * j + 1] = -(ei + pi);                                          \
        }                                                                       \
        F[0] = zeroval;                                                         \
        F[1] = (T)0;                                                            \
        F[2 * (halfN / 2)] = qre;                                               \
        F[2 * (halfN / 2) + 1] = qim;                                           \
        F[2 * halfN] = centerval;                                               \
        F[2 * halfN + 1] = (T)0;                                                \
        if (!half)                                                              \
            for (int i = halfN + 1; i < N; i++) {                               \
                F[2 * i] = F[2 * (N - i)];                                      \
                F[2 * i + 1] = -F[2 * (N - i) + 1];                             \
            }                                                                   \
        free(tw);                                                               \
    }                                                                           \
    void gfo_real_fft_##SUF(T *out, const T *in, int n, int half)               \
    {                                                                           \
        if (n == 1) {                                                           \
            out[0] = in[0];                                                     \
            out[1] = (T)0;                                                      \
            return;                                                             \
        }                                                                       \
        gfo_fft_##SUF(out, in, n / 2, 0);                                       \
        gfo_dit_##SUF(out, out, n, half);                                       \
    }

DEFINE_DIT(float, f)
DEFINE_DIT(double, d)

int gfo_real_fft_batch_f(float *out, long odist, const float *in, long idist,
                         int n, long batch, int half, int nthreads)
{
    batch_job p;
    memset(&p, 0, sizeof p);
    p.out = out; p.in = in; p.n = n; p.batch = batch; p.kind = 2;
    p.half = half; p.idist = idist; p.odist = odist;
    return run_batch(p, nthreads);
}

/* ------------------------------------------------------------------------ */
/* separate_2x_real_FFT (FFTReal.h:34-66).  Write order matters for the
 * i == N/2 element (its imaginary part ends as -0.0), so it is kept.       */
#define DEFINE_SEP(T, SUF)                                                      \
    void gfo_separate_2x_##SUF(T *Fx, T *Fy, const T *Fz, int N)                \
    {                                                                           \
        T xr, xi, yr, yi;                                                       \
        xr = Fz[0];                                                             \
        yr = Fz[1];                                                             \
        Fx[0] = xr;                                                             \
        Fx[1] = 0;                                                              \
        Fy[0] = yr;                                                             \
        Fy[1] = 0;                                                              \
        for (int i = 1; i <= N / 2; i++) {                                      \
            int k = N - i;                                                      \
            xr = (Fz[2 * i] + Fz[2 * k]) * 0.5f;                                \
            xi = (Fz[2 * i + 1] - Fz[2 * k + 1]) * 0.5f;                        \
            yr = (Fz[2 * k + 1] + Fz[2 * i + 1]) * 0.5f;                        \
            yi = (Fz[2 * k] - Fz[2 * i]) * 0.5f;                                \
            Fx[2 * i + 0] = xr;                                                 \
            Fx[2 * i + 1] = xi;                                                 \
            Fy[2 * i + 0] = yr;                                                 \
            Fy[2 * i + 1] = yi;                                                 \
            Fx[2 * k + 0] = xr;                                                 \
            Fx[2 * k + 1] = -xi;                                                \
            Fy[2 * k + 0] = yr;                                                 \
            Fy[2 * k + 1] = -yi;                                                \
        }                                                                       \
    }

DEFINE_SEP(float, f)
DEFINE_SEP(double, d)

/* ------------------------------------------------------------------------ */
/* FFT2D<T>::transform (fft.h:213-241): row FFTs written to bit-reversed row
 * positions (scramble_row_fft), then in-place column FFTs over all columns.
 * RealFFT2D<T>::forward (FFTReal.h:83-104, scramble_row_fwd :144-165).     */
#define DEFINE_2D(T, SUF)                                                       \
    static void row_fft_##SUF(T *out, long os, const T *in, long is, int rows,  \
                              int W, int inv, T *const *tw, int LW)             \
    {                                                                           \
        if (rows == 1) {                                                        \
            gfo_scramble_##SUF(out, in, W);                                     \
            fft_rec_##SUF(out, LW, inv, tw);                                    \
            return;                                                             \
        }                                                                       \
        row_fft_##SUF(out, 2 * os, in, is, rows / 2, W, inv, tw, LW);           \
        row_fft_##SUF(out + 2 * os, 2 * os, in + 2 * (rows / 2) * is, is,       \
                      rows / 2, W, inv, tw, LW);                                \
    }                                                                           \
    void gfo_fft2d_##SUF(T *out, long os, const T *in, long is, int W, int H,   \
                         int inv)                                               \
    {                                                                           \
        int LW = ilog2(W);                                                      \
        T **tw = tw_build_##SUF(LW);                                            \
        row_fft_##SUF(out, os, in, is, H, W, inv, tw, LW);                      \
        tw_free_##SUF(tw, LW);                                                  \
        gfo_fft_vert_inplace_##SUF(out, os, H, W, inv);                         \
    }                                                                           \
    static void row_fwd_##SUF(T *out, long os, const T *in, long is, int rows,  \
                              int W, T *const *tw, int LW)                      \
    {                                                                           \
        if (rows == 1) {                                                        \
            scr_r2c_##SUF(out, in, W, 1);                                       \
            fft_rec_##SUF(out, LW, 0, tw);                                      \
        } else if (rows == 2) {                                                 \
            scr_scalar_##SUF(out, in, W, 2);                                    \
            scr_scalar_##SUF(out + 1, in + is, W, 2);                           \
            fft_rec_##SUF(out, LW, 0, tw);                                      \
            gfo_separate_2x_##SUF(out, out + 2 * os, out, W);                   \
        } else {                                                                \
            row_fwd_##SUF(out, 2 * os, in, is, rows / 2, W, tw, LW);            \
            row_fwd_##SUF(out + 2 * os, 2 * os, in + (rows / 2) * is, is,       \
                          rows / 2, W, tw, LW);                                 \
        }                                                                       \
    }                                                                           \
    void gfo_real_fft2d_##SUF(T *out, long os, const T *in, long is, int W,     \
                              int H)                                            \
    {                                                                           \
        int LW = ilog2(W);                                                      \
        T **tw = tw_build_##SUF(LW);                                            \
        row_fwd_##SUF(out, os, in, is, H, W, tw, LW);                           \
        tw_free_##SUF(tw, LW);                                                  \
        int vcols = W / 2 + 1;                                                  \
        gfo_fft_vert_inplace_##SUF(out, os, H, vcols, 0);                       \
        if (vcols != W) {                                                       \
            for (int i = 0; i < H; i++) {                                       \
                int k = i ? H - i : 0;                                          \
                T *irow = out + 2 * (long)i * os;                               \
                T *orow = out + 2 * (long)k * os;                               \
                for (int j = W - 1; j >= vcols; j--) {                          \
                    orow[2 * j] = irow[2 * (W - j)];                            \
                    orow[2 * j + 1] = -irow[2 * (W - j) + 1];                   \
                }                                                               \
            }                                                                   \
        }                                                                       \
    }

DEFINE_2D(float, f)
DEFINE_2D(double, d)

/* forward_2x: two real images packed as re/im of one complex image
 * (FFTReal.h:114-118, scramble_row_x2 :167-180), then column FFTs over all
 * columns.  The reference's second-image offset uses in_stride1 (:178);
 * this restatement uses in_stride2, which agrees when the strides match. */
static void row_x2_f(float *out, long os, const float *in1, long is1,
                     const float *in2, long is2, int rows, int W,
                     float *const *tw, int LW)
{
    if (rows == 1) {
        scr_scalar_f(out, in1, W, 2);
        scr_scalar_f(out + 1, in2, W, 2);
        fft_rec_f(out, LW, 0, tw);
        return;
    }
    row_x2_f(out, 2 * os, in1, is1, in2, is2, rows / 2, W, tw, LW);
    row_x2_f(out + 2 * os, 2 * os, in1 + (rows / 2) * is1, is1,
             in2 + (rows / 2) * is2, is2, rows / 2, W, tw, LW);
}

void gfo_real_fft2d_2x_f(float *out, long os, const float *in1, long is1,
                         const float *in2, long is2, int W, int H)
{
    int LW = ilog2(W);
    float **tw = tw_build_f(LW);
    row_x2_f(out, os, in1, is1, in2, is2, H, W, tw, LW);
    tw_free_f(tw, LW);
    gfo_fft_vert_inplace_f(out, os, H, W, 0);
}

/* ------------------------------------------------------------------------ */
/* FP64 DFT (the accuracy oracle; same math as test/fft_ref_impl.h:120-135
 * but with exact phase reduction (j*k mod n) and compensated summation).  */
static void dft_core(double *out, const double *xin, const float *xin_f, int n,
                     int inv, int k0, int nbins)
{
    double *c = (double *)malloc(sizeof(double) * (size_t)n);
    double *s = (double *)malloc(sizeof(double) * (size_t)n);
    const double sg = inv ? 1.0 : -1.0;
    for (int m = 0; m < n; m++) {
        c[m] = cos(2.0 * M_PI * (double)m / (double)n);
        s[m] = sg * sin(2.0 * M_PI * (double)m / (double)n);
    }
    for (int b = 0; b < nbins; b++) {
        long k = k0 + b;
        double sr = 0, si = 0, cr = 0, ci = 0; /* Neumaier sums */
        long ph = 0;
        for (int j = 0; j < n; j++) {
            double xr = xin ? xin[2 * j] : (double)xin_f[2 * j];
            double xi = xin ? xin[2 * j + 1] : (double)xin_f[2 * j + 1];
            double tr = xr * c[ph] - xi * s[ph];
            double ti = xr * s[ph] + xi * c[ph];
            double t = sr + tr;
            cr += fabs(sr) >= fabs(tr) ? (sr - t) + tr : (tr - t) + sr;
            sr = t;
            t = si + ti;
            ci += fabs(si) >= fabs(ti) ? (si - t) + ti : (ti - t) + si;
            si = t;
            ph += k;
            if (ph >= n) ph %= n;
        }
        out[2 * b] = sr + cr;
        out[2 * b + 1] = si + ci;
    }
    free(c);
    free(s);
}

void gfo_dft_d(double *out, const double *in, int n, int inv, int k0, int nbins)
{
    dft_core(out, in, NULL, n, inv, k0, nbins);
}

void gfo_dft_fin(double *out, const float *in, int n, int inv, int k0, int nbins)
{
    dft_core(out, NULL, in, n, inv, k0, nbins);
}

/* Extended-precision FFT for large-n FP64 checks: iterative radix-2 in long
 * double with exactly reduced twiddles.  Error ~ log2(n) * eps(long double),
 * far below double rounding.                                               */
void gfo_fft64(double *out, const double *in, int n, int inv)
{
    long double *a = (long double *)malloc(sizeof(long double) * 2 * (size_t)n);
    long double *w = (long double *)malloc(sizeof(long double) * (size_t)n);
    const long double PI_L = 3.141592653589793238462643383279502884L;
    int L = ilog2(n);
    for (int i = 0; i < n; i++) {
        unsigned r = 0;
        for (int b = 0; b < L; b++) r |= (unsigned)((i >> b) & 1) << (L - 1 - b);
        a[2 * r] = in[2 * i];
        a[2 * r + 1] = in[2 * i + 1];
    }
    for (int k = 0; k < n / 2; k++) {
        long double ang = 2.0L * PI_L * (long double)k / (long double)n;
        w[2 * k] = cosl(ang);
        w[2 * k + 1] = (inv ? 1.0L : -1.0L) * sinl(ang);
    }
    for (int len = 2; len <= n; len <<= 1) {
        int step = n / len;
        for (int s0 = 0; s0 < n; s0 += len) {
            for (int k = 0; k < len / 2; k++) {
                long double wr = w[2 * k * step], wi = w[2 * k * step + 1];
                long double *e = a + 2 * (s0 + k), *o = a + 2 * (s0 + k + len / 2);
                long double tr = o[0] * wr - o[1] * wi;
                long double ti = o[0] * wi + o[1] * wr;
                o[0] = e[0] - tr;
                o[1] = e[1] - ti;
                e[0] += tr;
                e[1] += ti;
            }
        }
    }
    for (int i = 0; i < 2 * n; i++) out[i] = (double)a[i];
    free(a);
    free(w);
}
