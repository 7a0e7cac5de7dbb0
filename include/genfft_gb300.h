/*
 * genfft_gb300.h -- C ABI of libgenfft_gb300.so, the GB300 (sm_103a)
 * implementation of genFFT's transform hot path.
 *
 * Plain C: pointers, sizes and status codes only.  Data pointers passed to
 * the gfft_* transform entry points are DEVICE pointers (cudaMalloc'd or
 * managed) unless the function name ends in _host; `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  Calls are
 * stream-ordered and return as soon as the work is enqueued.
 *
 * Conventions follow the reference library (mzient/genFFT):
 *   - power-of-two sizes only (README.txt:10-11);
 *   - forward transform uses exp(-2*pi*i*j*k/n) (FFTTwiddle.h:44-51);
 *   - the inverse is UNSCALED: inverse(forward(x)) == n * x (README.txt:28-31);
 *   - complex data is interleaved {re, im} pairs of float or double
 *     (FFTComplex.h:33-37);
 *   - row strides are in complex elements for complex arrays and in scalar
 *     elements for real arrays (fft.h:140-146, FFTReal.h:330-335).
 * Where the reference asserts or has undefined behaviour (unsupported sizes,
 * fft_impl_generic.h:276-278), these functions return an error status and
 * record a message readable with gfft_last_error().
 */
#ifndef GENFFT_GB300_H
#define GENFFT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFFT_VERSION 1

typedef enum gfft_status {
    GFFT_OK = 0,
    GFFT_ERR_INVALID_SIZE = 1,   /* not a power of two, zero/negative, or above the limit */
    GFFT_ERR_INVALID_VALUE = 2,  /* bad enum, NULL pointer, bad stride */
    GFFT_ERR_ALIAS = 3,          /* out == in where the reference forbids it */
    GFFT_ERR_ALIGN = 4,          /* pointer not aligned to its element type */
    GFFT_ERR_ARCH = 5,           /* no sm_103 device current */
    GFFT_ERR_CUDA = 6,           /* a CUDA runtime call failed */
    GFFT_ERR_TIMEOUT = 7,        /* a bounded device-side wait gave up */
    GFFT_ERR_UNSUPPORTED = 8,    /* valid request this build does not implement */
    GFFT_ERR_ALLOC = 9,          /* device or host allocation failed */
    GFFT_ERR_INVALID_PLAN = 10   /* NULL or destroyed plan handle */
} gfft_status;

typedef enum gfft_dtype { GFFT_F32 = 0, GFFT_F64 = 1 } gfft_dtype;

typedef enum gfft_kind {
    GFFT_KIND_C2C = 0,     /* batched 1D complex, FFT<T> (fft.h:56-113) */
    GFFT_KIND_R2C = 1,     /* batched 1D real input, RealFFT<T> (FFTReal.h:186-221) */
    /* column lengths (2D heights, FFTVert rows) up to 2^24: up to 2^12 in
     * one launch of column tiles, above that as two launches of shorter
     * column FFTs per band of columns through a plan-owned scratch */
    GFFT_KIND_C2C_2D = 2,  /* 2D complex, FFT2D<T> (fft.h:198-245) */
    GFFT_KIND_R2C_2D = 3,  /* 2D real input, RealFFT2D<T> (FFTReal.h:69-184) */
    GFFT_KIND_VERT = 4     /* column FFT, FFTVert<T> (fft.h:115-171) */
} gfft_kind;

typedef enum gfft_mode {
    GFFT_MODE_PLAIN = 0,   /* FP32/FP64 CUDA-core arithmetic */
    /* Split-precision tensor-core C2C (fp32 data, GFFT_KIND_C2C, n = 256,
     * 4096 or 65536, unit strides).  No counterpart in the reference.
     * Radix-16 DFT blocks run as dense 16-bit products on the tcgen05 tensor
     * cores with FP32 accumulation; twiddles are compensated fp32 products. */
    GFFT_MODE_TC_FP16 = 1, /* FP16 hi + lo terms, per-vector power-of-two scaling, 3 products */
    GFFT_MODE_TC_BF16 = 2  /* BF16 hi + mid + lo terms, 6 products */
} gfft_mode;

/* gfft_desc.flags */
#define GFFT_FLAG_HALF_SPECTRUM 0x1u /* R2C: store n/2+1 bins (RealFFT::forward half=true) */
#define GFFT_FLAG_BITREV_INPUT 0x2u  /* C2C/VERT: input in bit-reversed order
                                        (transform_no_scramble, fft.h:69-73, 132-136) */

typedef struct gfft_desc {
    int kind;             /* gfft_kind */
    int dtype;            /* gfft_dtype */
    int mode;             /* gfft_mode */
    unsigned flags;       /* GFFT_FLAG_* */
    long long n0;         /* 1D/VERT: transform length; 2D: width (columns) */
    long long n1;         /* 2D: height (rows); VERT: number of columns; else 0 */
    long long batch;      /* number of transforms (>= 1) */
    long long istride;    /* input element stride (0 = contiguous = 1); VERT: row stride */
    long long idist;      /* input distance between transforms (0 = dense) */
    long long ostride;    /* output element stride (0 = 1); VERT: row stride */
    long long odist;      /* output distance between transforms (0 = dense) */
} gfft_desc;

typedef struct gfft_plan_s *gfft_plan;

/* ---- plan API -------------------------------------------------------- */
/* Plans are immutable after creation.  Sizes that run in one kernel (see
 * gfft_max_fused_size) read nothing but the plan's tables, so their execs may
 * run concurrently on different streams.  Multi-pass sizes own a workspace
 * (gfft_plan_workspace_size) that one exec uses at a time: execs of such a
 * plan must be ordered (one stream, or events); use one plan per stream to
 * run them concurrently.  Creation is thread-safe. */
gfft_status gfft_plan_create(gfft_plan *plan, const gfft_desc *desc);
gfft_status gfft_plan_destroy(gfft_plan plan);
/* forward (inverse = 0) or unscaled inverse (inverse = 1) on device memory.
 * For GFFT_KIND_R2C plans the inverse is the half-spectrum inverse (C2R):
 * bins in the plan's output layout -> reals in its input layout, unscaled,
 * imaginary parts of the DC and Nyquist bins ignored (no counterpart in the
 * reference, whose RealFFT has no inverse, FFTReal.h:127-130). */
gfft_status gfft_exec(gfft_plan plan, int inverse, void *out, const void *in, void *stream);
/* gfft_exec with every output multiplied by `scale` inside the kernel that
 * writes it (no extra pass): the norm= factors of torch.fft-style APIs
 * (1/n, 1/sqrt(n)).  No counterpart in the reference, whose inverse is
 * always unscaled (README.txt:28-31). */
gfft_status gfft_exec_scaled(gfft_plan plan, int inverse, double scale, void *out, const void *in,
                             void *stream);
/* Adjoint (reverse-mode gradient) of the plan's transform in direction
 * `inverse`: grad_in = A^H grad_out with PyTorch's complex convention.
 * C2C / 2D / VERT: the conjugate-direction transform.  R2C forward: a C2R of
 * the gradient with the Hermitian weighting (interior bins halved, or the
 * full spectrum folded); C2R: an R2C with interior bins doubled.  `in` has
 * the layout of the transform's output, `out` that of its input. */
gfft_status gfft_exec_adjoint(gfft_plan plan, int inverse, void *out, const void *in, void *stream);
/* Same transform on HOST buffers (the reference's calling convention):
 * copies in, transforms and copies out in pipelined chunks, synchronously.
 * Pinned host memory gives full link bandwidth; pageable memory works.
 * Single-kernel C2C sizes (see gfft_max_fused_size) on pinned buffers, on a
 * device that reads host memory through the host's page tables (GB300 with
 * Grace), skip the staging: the kernel reads the input and writes the
 * output over the host link itself (GFFT_HOST_DIRECT=0 turns this off).
 * Whole transforms are staged, so each must lie inside its own idist /
 * odist block (GFFT_ERR_UNSUPPORTED for batch-interleaved layouts, which
 * run on device buffers). */
gfft_status gfft_exec_host(gfft_plan plan, int inverse, void *out, const void *in);
/* number of kernel launches one forward gfft_exec makes (for launch
 * accounting) */
gfft_status gfft_plan_launches(gfft_plan plan, int *launches);
/* the same for either direction (inverse != 0: the inverse, which for an
 * R2C plan is the half-spectrum inverse) */
gfft_status gfft_plan_launches_dir(gfft_plan plan, int inverse, int *launches);
/* device workspace the plan owns (bytes; 0 for single-kernel sizes) */
gfft_status gfft_plan_workspace_size(gfft_plan plan, size_t *bytes);

/* ---- reference-shaped entry points (device pointers) ------------------ */
/* Each mirrors one call of the reference C++ API; plans are cached per
 * (kind, type, size) like the reference's per-size singletons
 * (FFTLevel.h:76-88), but creation here is mutex-guarded.  Like the
 * reference's transforms, these calls may be made from any thread on any
 * stream at once: where the cached plan has a workspace (multi-pass
 * sizes), its transforms run one after another on the GPU, in issue order,
 * whatever their streams. */

/* FFT<T>(n).transform<inverse>(out, in) over `batch` dense transforms
 * (fft.h:80-85).  out != in is not required here (in-place is allowed). */
gfft_status gfft_fft_transform(int dtype, int n, long long batch, int inverse, void *out,
                               const void *in, void *stream);
/* FFT<T>(n).transform_no_scramble<inverse>(inout): in place, bit-reversed
 * input, natural-order output (fft.h:69-73). */
gfft_status gfft_fft_transform_no_scramble(int dtype, int n, long long batch, int inverse,
                                           void *inout, void *stream);
/* FFT<T>(n).transform_real(out, in): n reals -> n complex bins (fft.h:90-94) */
gfft_status gfft_fft_transform_real(int dtype, int n, long long batch, void *out, const void *in,
                                    void *stream);
/* FFT<T>(n).transform_interleave(out, in1, in2): FFT of in1 + i*in2,
 * separate with gfft_separate_2x_real_fft (fft.h:100-105) */
gfft_status gfft_fft_transform_interleave(int dtype, int n, void *out, const void *in1,
                                          const void *in2, void *stream);
/* FFTVert<T>(n).transform<inverse>(out, out_stride, in, in_stride, cols):
 * length-n FFT down each of `cols` columns; strides in complex elements;
 * out must not be in (fft.h:145-150). */
gfft_status gfft_vert_transform(int dtype, int n, int inverse, void *out, long long out_stride,
                                const void *in, long long in_stride, int cols, void *stream);
/* FFTVert<T>(n).transform_no_scramble<inverse>(data, stride, cols): in
 * place, rows in bit-reversed order (fft.h:132-136). */
gfft_status gfft_vert_transform_no_scramble(int dtype, int n, int inverse, void *data,
                                            long long stride, int cols, void *stream);
/* DIT<T>(n).apply(out, in, half): real-FFT adjustment of the n/2-point
 * complex FFT `in` into the spectrum `out` (n/2+1 bins if half, else n);
 * out may equal in (fft.h:180-188, fft_dit_impl_generic.inl:27-61). */
gfft_status gfft_dit_apply(int dtype, int n, void *out, const void *in, int half, void *stream);
/* FFT2D<T>(width, height).transform<inverse>(out, out_stride, in, in_stride):
 * row-major [height][width], strides in complex elements (fft.h:213-218). */
gfft_status gfft_fft2d_transform(int dtype, int width, int height, int inverse, void *out,
                                 long long out_stride, const void *in, long long in_stride,
                                 void *stream);
/* RealFFT<T>(n).forward(out, in, half) over `batch` transforms: n reals in,
 * n/2+1 (half) or n bins out; transforms are n reals / n complex apart like
 * the reference's buffers (FFTReal.h:204-213). */
gfft_status gfft_real_fft_forward(int dtype, int n, long long batch, void *out, const void *in,
                                  int half, void *stream);
/* RealFFT2D<T>(width, height).forward(out, out_stride, in, in_stride):
 * full-width Hermitian output; in_stride in reals, out_stride in complex
 * elements (FFTReal.h:83-104). */
gfft_status gfft_real_fft2d_forward(int dtype, int width, int height, void *out, long long out_stride,
                                    const void *in, long long in_stride, void *stream);
/* RealFFT2D<T>(width, height).forward_2x: 2D FFT of in1 + i*in2
 * (FFTReal.h:114-118) */
gfft_status gfft_real_fft2d_forward_2x(int dtype, int width, int height, void *out,
                                       long long out_stride, const void *in1, long long in_stride1,
                                       const void *in2, long long in_stride2, void *stream);
/* separate_2x_real_FFT(out1, out2, in, n); out1 or out2 may be in
 * (FFTReal.h:34-66) */
gfft_status gfft_separate_2x_real_fft(int dtype, int n, void *out1, void *out2, const void *in,
                                      void *stream);

/* Allocation-free fp32 C2C for n = 2^15 .. 2^22 (the multi-pass sizes).
 * No counterpart in the reference: the reference computes on the host and
 * allocates its plans' tables itself.  This variant is for callers that
 * cannot allocate device memory when they transform (memory owned by a
 * caching allocator or a fixed pool, or a loop where cudaMalloc would
 * stall the device).  Its scratch and twiddle tables are fixed __device__
 * arrays (32 MiB + ~0.3 MiB) that every GPU loading the library keeps until
 * exit.  The first call on each device sets them up (cudaGetSymbolAddress,
 * a synchronous table upload): make it before any stream capture.  All calls
 * share the scratch, so calls that can overlap on the GPU race and must be
 * serialised by the caller.  Sizes outside 2^15 .. 2^22 and fp64 are
 * rejected.  Same results as gfft_fft_transform. */
gfft_status gfft_fft_transform_noalloc(int dtype, int n, long long batch, int inverse, void *out,
                                       const void *in, void *stream);

/* ---- ragged batches (no counterpart in the reference, which plans one
 * size per FFT<T> object, fft.h:56-113) ----------------------------------
 * `count` fp32 C2C transforms of power-of-two sizes 1 .. 2^18 packed back to
 * back (transform i starts at the sum of the earlier sizes).  One exec is
 * one CUDA-graph replay of a single persistent kernel; the graph is
 * captured on the first exec with a given (in, out, direction).  The plan
 * owns scratch for its transforms above 2^12 points and a work counter:
 * execs of one plan must be ordered by the caller (one stream, or events);
 * use one plan per stream to run ragged batches concurrently. */
typedef struct gfft_ragged_s *gfft_ragged;
gfft_status gfft_ragged_create(gfft_ragged *plan, int dtype, const long long *sizes, long long count);
gfft_status gfft_ragged_destroy(gfft_ragged plan);
gfft_status gfft_ragged_exec(gfft_ragged plan, int inverse, void *out, const void *in, void *stream);
/* adjoint of direction `inverse` (the conjugate-direction transform) */
gfft_status gfft_ragged_exec_adjoint(gfft_ragged plan, int inverse, void *out, const void *in, void *stream);
/* Times the candidate schedules on these buffers and keeps the fastest;
 * params = {row-tile lag (in multiples of the work items in flight), CTAs
 * per SM (0 = occupancy), large transforms first}; *ms = its time.  With
 * GFFT_AUTOTUNE_CACHE set the choice is cached in that file per size
 * histogram. */
gfft_status gfft_ragged_autotune(gfft_ragged plan, void *out, const void *in, void *stream, int *params,
                                 double *ms);
/* total complex elements of the packed batch */
gfft_status gfft_ragged_elements(gfft_ragged plan, long long *elements);

/* Device-side error status of this device's kernels since the last call
 * (synchronous): *code = 0 and GFFT_OK if none; otherwise the recorded
 * bits (1 = a bounded TMA or dependency wait gave up, 2 = a bounded wait
 * for tensor-core MMAs gave up) and GFFT_ERR_TIMEOUT.  Reading resets it. */
gfft_status gfft_device_error(int *code);

/* Arithmetic-rate probe of the current device (no counterpart in the
 * reference): times independent fused multiply-add chains with CUDA events
 * on a private stream.  which = 0 fp32 fma, 1 packed fp32x2 fma
 * (fma.rn.f32x2), 2 fp64 fma; *tflops counts two flops per FMA lane, *ms is
 * the best of five timed launches.  Allocates a 4-byte device buffer; it is
 * the denominator of the fp64 kernels' roofline. */
gfft_status gfft_diag_fma_rate(int which, double *tflops, double *ms);
/* Read (mode 0) or copy (mode 1) bandwidth over a device buffer of `bytes`
 * bytes (1 MiB .. 8 GiB): below the L2 capacity the L2's rate, above it
 * HBM's.  *gbs counts bytes read plus bytes written.  A probe, not a
 * transform. */
gfft_status gfft_diag_mem_rate(long long bytes, int mode, double *gbs, double *ms);

const char *gfft_status_string(gfft_status status);
/* message of the last failed call on this thread ("" if none) */
const char *gfft_last_error(void);
int gfft_version(void);
/* largest n handled by a single fused kernel for dtype (informational) */
int gfft_max_fused_size(int dtype);

#ifdef __cplusplus
}
#endif

#endif /* GENFFT_GB300_H */
