// peaks.cu -- arithmetic-throughput probe: the FP32, packed FP32x2 and FP64
// fused multiply-add rates of the current device, measured with CUDA events
// over independent FMA chains.  It is the denominator of the fp64 path's
// roofline (GB300 keeps a small FP64 pipe) and shows whether packed
// fma.rn.f32x2 doubles the FP32 rate or only halves the issue slots.
// No counterpart in the reference (a CPU library).
#include <cuda_runtime.h>

#include "internal.h"

namespace gfft {
namespace {

constexpr int CHAINS = 8;     // independent accumulators per thread
constexpr int ITERS = 4096;   // FMAs per chain per launch
constexpr int THREADS = 256;

// which: 0 fp32 fma.rn.f32, 1 packed fma.rn.f32x2, 2 fp64 fma.rn.f64
template <int WHICH>
__global__ void __launch_bounds__(THREADS) k_fma_chains(float seed, float *sink)
{
    if constexpr (WHICH == 2) {
        double a[CHAINS];
        const double b = 1.0 - 1e-9 * seed, c = 1e-12 * seed;
#pragma unroll
        for (int i = 0; i < CHAINS; i++) a[i] = (double)(threadIdx.x + i) * 1e-3;
#pragma unroll 4
        for (int k = 0; k < ITERS; k++) {
#pragma unroll
            for (int i = 0; i < CHAINS; i++) a[i] = fma(a[i], b, c);
        }
        double s = 0;
#pragma unroll
        for (int i = 0; i < CHAINS; i++) s += a[i];
        if (s == 12345.678) sink[0] = (float)s;  // keeps the chains alive
    } else if constexpr (WHICH == 1) {
        float2 a[CHAINS];
        const float2 b = make_float2(1.0f - 1e-7f * seed, 1.0f - 2e-7f * seed);
        const float2 c = make_float2(1e-9f * seed, 2e-9f * seed);
#pragma unroll
        for (int i = 0; i < CHAINS; i++) a[i] = make_float2((float)(threadIdx.x + i), (float)i);
#pragma unroll 4
        for (int k = 0; k < ITERS; k++) {
#pragma unroll
            for (int i = 0; i < CHAINS; i++) a[i] = __ffma2_rn(a[i], b, c);
        }
        float s = 0;
#pragma unroll
        for (int i = 0; i < CHAINS; i++) s += a[i].x + a[i].y;
        if (s == 12345.678f) sink[0] = s;
    } else {
        float a[CHAINS];
        const float b = 1.0f - 1e-7f * seed, c = 1e-9f * seed;
#pragma unroll
        for (int i = 0; i < CHAINS; i++) a[i] = (float)(threadIdx.x + i);
#pragma unroll 4
        for (int k = 0; k < ITERS; k++) {
#pragma unroll
            for (int i = 0; i < CHAINS; i++) a[i] = fmaf(a[i], b, c);
        }
        float s = 0;
#pragma unroll
        for (int i = 0; i < CHAINS; i++) s += a[i];
        if (s == 12345.678f) sink[0] = s;
    }
}

}  // namespace
}  // namespace gfft

// Measures one rate: which = 0 (fp32), 1 (packed fp32x2), 2 (fp64).
// *tflops = 2 * FMAs / time (an FMA counts two flops; a packed FMA four),
// *ms = the timed launch.  Allocates a 4-byte sink.  A measurement probe,
// not a transform.
extern "C" gfft_status gfft_diag_fma_rate(int which, double *tflops, double *ms)
{
    using namespace gfft;
    if (!tflops || !ms || which < 0 || which > 2) return GFFT_ERR_INVALID_VALUE;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return GFFT_ERR_CUDA;
    const void *fn = which == 0 ? (const void *)&k_fma_chains<0>
                   : which == 1 ? (const void *)&k_fma_chains<1>
                                : (const void *)&k_fma_chains<2>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, THREADS, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int grid = sms * per_sm * 4;  // four full waves
    float *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) return GFFT_ERR_ALLOC;
    cudaStream_t st = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    gfft_status rc = GFFT_OK;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&a) != cudaSuccess ||
        cudaEventCreate(&b) != cudaSuccess) {
        rc = GFFT_ERR_CUDA;
    } else {
        float seed = 1.0f;
        void *args[] = {(void *)&seed, (void *)&sink};
        float best = 1e30f;
        for (int rep = 0; rep < 6 && rc == GFFT_OK; rep++) {  // the first is a warm-up
            if (cudaEventRecord(a, st) != cudaSuccess ||
                cudaLaunchKernel(fn, dim3(grid), dim3(THREADS), args, 0, st) != cudaSuccess ||
                cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) {
                rc = GFFT_ERR_CUDA;
                break;
            }
            float t = 0;
            cudaEventElapsedTime(&t, a, b);
            if (rep > 0 && t < best) best = t;
        }
        if (rc == GFFT_OK) {
            const double fmas = (double)grid * THREADS * CHAINS * ITERS * (which == 1 ? 2 : 1);
            *ms = best;
            *tflops = 2.0 * fmas / (best * 1e-3) / 1e12;
        }
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    return rc;
}
