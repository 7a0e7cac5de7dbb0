// peaks.cu -- throughput probes of the current device, measured with CUDA
// events:
//   gfft_diag_fma_rate  the FP32, packed FP32x2 and FP64 fused multiply-add
//                       rates over independent FMA chains: the denominator
//                       of the fp64 path's roofline (GB300 keeps a small
//                       FP64 pipe), and whether packed fma.rn.f32x2 doubles
//                       the FP32 rate or only halves the issue slots;
//   gfft_diag_mem_rate  read and copy bandwidth over a buffer of a given
//                       size: below the L2 capacity it is the L2's rate,
//                       the ceiling of any pass whose intermediate stays in
//                       L2, above it the HBM rate.
// No counterpart in the reference (a CPU library).
#include <cuda_runtime.h>

#include <algorithm>

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

// grid-stride 16-byte loads (reps passes over n vectors), summed into a
// value that is stored only if it hits a constant, so the loads stay
__global__ void __launch_bounds__(THREADS) k_mem_read(const float4 *__restrict__ p, long long n, int reps, float *sink)
{
    float acc = 0.f;
    const long long stride = (long long)gridDim.x * THREADS;
    for (int r = 0; r < reps; r++)
        for (long long i = (long long)blockIdx.x * THREADS + threadIdx.x; i < n; i += stride) {
            const float4 v = __ldcg(p + i);
            acc += v.x + v.w;
        }
    if (acc == 12345.678f) sink[0] = acc;
}

// grid-stride 16-byte copy of n vectors, reps times
__global__ void __launch_bounds__(THREADS) k_mem_copy(const float4 *__restrict__ a, float4 *__restrict__ b, long long n,
                                                      int reps)
{
    const long long stride = (long long)gridDim.x * THREADS;
    for (int r = 0; r < reps; r++)
        for (long long i = (long long)blockIdx.x * THREADS + threadIdx.x; i < n; i += stride) __stcg(b + i, __ldcg(a + i));
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

// Read (mode 0) or copy (mode 1: the first half of the buffer into the
// second) bandwidth over a device buffer of `bytes` bytes (1 MiB .. 8 GiB).
// Each timed launch repeats the pass until it has moved at least 2 GiB;
// *gbs = bytes moved (read + written) / time, best of 5 after a warm-up,
// *ms = that launch.  Allocates the buffer.  A measurement probe, not a
// transform.
extern "C" gfft_status gfft_diag_mem_rate(long long bytes, int mode, double *gbs, double *ms)
{
    using namespace gfft;
    if (!gbs || !ms || mode < 0 || mode > 1 || bytes < (1LL << 20) || bytes > (8LL << 30))
        return GFFT_ERR_INVALID_VALUE;
    bytes &= ~255LL;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return GFFT_ERR_CUDA;
    char *buf = nullptr;
    float *sink = nullptr;
    if (cudaMalloc(&buf, (size_t)bytes) != cudaSuccess) return GFFT_ERR_ALLOC;
    if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) {
        cudaFree(buf);
        return GFFT_ERR_ALLOC;
    }
    cudaStream_t st = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    gfft_status rc = GFFT_OK;
    const int grid = sms * 8;  // eight 256-thread CTAs an SM
    const int reps = (int)std::max<long long>(1, (2LL << 30) / bytes);
    if (cudaMemsetAsync(buf, 0, (size_t)bytes) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&a) != cudaSuccess ||
        cudaEventCreate(&b) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        rc = GFFT_ERR_CUDA;
    } else {
        const float4 *src = reinterpret_cast<const float4 *>(buf);
        float4 *dst = reinterpret_cast<float4 *>(buf + bytes / 2);
        long long n = mode == 0 ? bytes / 16 : bytes / 32;
        int r = reps;
        void *rargs[] = {(void *)&src, (void *)&n, (void *)&r, (void *)&sink};
        void *cargs[] = {(void *)&src, (void *)&dst, (void *)&n, (void *)&r};
        const void *fn = mode == 0 ? (const void *)&k_mem_read : (const void *)&k_mem_copy;
        float best = 1e30f;
        for (int rep = 0; rep < 6 && rc == GFFT_OK; rep++) {
            if (cudaEventRecord(a, st) != cudaSuccess ||
                cudaLaunchKernel(fn, dim3(grid), dim3(THREADS), mode == 0 ? rargs : cargs, 0, st) != cudaSuccess ||
                cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) {
                rc = GFFT_ERR_CUDA;
                break;
            }
            float t = 0;
            cudaEventElapsedTime(&t, a, b);
            if (rep > 0 && t < best) best = t;
        }
        if (rc == GFFT_OK) {
            *ms = best;
            *gbs = (double)bytes * reps / (best * 1e-3) / 1e9;  // read bytes, or half read + half written
        }
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    cudaFree(buf);
    return rc;
}
