// c2c_fused.cu -- single-kernel batched C2C transforms for sizes whose whole
// transform fits one CTA's shared memory (fp32 up to 2^14, fp64 up to 2^13).
//
// Replaces the reference's FFT<T>::transform<inv> (fft.h:80-85): there a
// bit-reversal copy (FFTUtil.h:51-83) is followed by recursive radix-2
// butterflies (fft_impl_generic.h:36-63).  Here each transform makes one
// HBM read and one HBM write: the first Stockham pass reads its operands
// straight from global memory (coalesced), radix-16 (fp32) or radix-8
// (fp64) passes exchange through padded shared memory, and the last pass
// stores straight to global memory.  Roofline: HBM-bound, 2 * N * 2 *
// sizeof(T) algorithmic bytes per transform.
#include <mutex>

#include "internal.h"
#include "stockham.cuh"
#include "twiddle.h"

namespace gfft {

// points per thread: radix-16 registers for fp32, radix-8 for fp64;
// radix-32 for fp32 2^13 and 2^14 (three passes instead of four)
template <typename T, int LOGN>
struct FusedE {
    static constexpr int value = sizeof(T) == 4 ? ((LOGN == 13 || LOGN == 14) ? 32 : 16) : 8;
};

template <typename T>
struct FusedMax {
    static constexpr int value = sizeof(T) == 4 ? 14 : 13;
};

// threads per CTA: one transform per CTA when its group already has >= 256
// threads, else several transforms share the CTA
template <typename T, int LOGN>
struct FusedCfg {
    using SP = StockhamPlan<T, LOGN, FusedE<T, LOGN>::value>;
    static constexpr int TPC = SP::G >= 256 ? 1 : 256 / SP::G;
    static constexpr int THREADS = SP::G * TPC;
    static constexpr size_t SMEM = (size_t)SP::SMEM * TPC * sizeof(cpx<T>);
    // four resident CTAs (64 registers a thread) where that costs no spill
    // (fp32 n = 2^12 and n <= 2^8, ptxas -v), else three for CTAs of up to
    // 256 threads (the residency the compiler picked unconstrained) and two
    // for 512-thread CTAs
    static constexpr int MIN_BLOCKS = (sizeof(T) == 4 && (LOGN == 12 || (LOGN >= 5 && LOGN <= 8))) ? 4
                                    : (sizeof(T) == 4 && LOGN == 13) ? 2
                                    : (sizeof(T) == 4 && LOGN == 14) ? 1
                                    : THREADS <= 256 ? 3 : THREADS <= 512 ? 2 : 1;
};

template <typename T, int LOGN, bool INV>
__global__ void __launch_bounds__(FusedCfg<T, LOGN>::THREADS, FusedCfg<T, LOGN>::MIN_BLOCKS)
    k_c2c_fused(const cpx<T> *__restrict__ in, cpx<T> *__restrict__ out, long long batch,
                long long idist, long long odist, long long istride, long long ostride,
                const cpx<T> *__restrict__ tw, T scale)
{
    using Cfg = FusedCfg<T, LOGN>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G;
    extern __shared__ unsigned char smem_raw[];
    cpx<T> *sm = reinterpret_cast<cpx<T> *>(smem_raw);

    const int g = threadIdx.x / G;
    const int t = threadIdx.x - g * G;
    const long long b = (long long)blockIdx.x * Cfg::TPC + g;
    const bool active = b < batch;

    // programmatic dependent launch: the next kernel's CTAs may fill the
    // slots this grid's last wave frees; this grid waits for the previous one
    pdl_enter();
    cpx<T> v[E];
    if (active) {
        const cpx<T> *src = in + b * idist + (long long)t * istride;
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = ldcs_c(src + (long long)q * G * istride);
    } else {
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = cpx<T>{(T)0, (T)0};
    }
    cpx<T> *my = sm + g * SP::SMEM;
    stockham_run<T, LOGN, FusedE<T, LOGN>::value, INV>(
        v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
    if (active) {
        cpx<T> *dst = out + b * odist + (long long)t * ostride;
#pragma unroll
        for (int q = 0; q < E; q++) stcs_c(dst + (long long)q * G * ostride, scl(v[q], scale));
    }
}

// ---------------------------------------------------------------------------
// host side

namespace {

template <typename T, int LOGN>
void fill_tw(void *buf)
{
    stockham_fill_twiddles<T, LOGN, FusedE<T, LOGN>::value>(
        static_cast<cpx<T> *>(buf), [](long long k, long long M, cpx<T> *w) { forward_root<T>(k, M, &w->x, &w->y); });
}

struct Entry {
    const void *fwd, *inv;
    int threads, tpc;
    size_t smem;
    size_t twcount;
    void (*fill)(void *);
};

template <typename T, int LOGN>
Entry make_entry()
{
    using Cfg = FusedCfg<T, LOGN>;
    return Entry{(const void *)&k_c2c_fused<T, LOGN, false>, (const void *)&k_c2c_fused<T, LOGN, true>,
                 Cfg::THREADS, Cfg::TPC, Cfg::SMEM, (size_t)Cfg::SP::TW, &fill_tw<T, LOGN>};
}

template <typename T, int... L>
const Entry *table_impl(std::integer_sequence<int, L...>)
{
    static const Entry tab[] = {make_entry<T, L>()...};
    return tab;
}

template <typename T>
const Entry &entry(int logn)
{
    return table_impl<T>(std::make_integer_sequence<int, FusedMax<T>::value + 1>{})[logn];
}

const Entry &entry_for(int dtype, int logn)
{
    return dtype == GFFT_F32 ? entry<float>(logn) : entry<double>(logn);
}

}  // namespace

int fused_max_logn(int dtype) { return dtype == GFFT_F32 ? FusedMax<float>::value : FusedMax<double>::value; }

size_t fused_twiddle_count(int dtype, int logn) { return entry_for(dtype, logn).twcount; }

void fused_twiddle_fill(int dtype, int logn, void *host_buf) { entry_for(dtype, logn).fill(host_buf); }

cudaError_t launch_fused_c2c(int dtype, int logn, int inverse, const FusedC2CArgs &a, cudaStream_t st)
{
    const Entry &e = entry_for(dtype, logn);
    const void *fn = inverse ? e.inv : e.fwd;
    if (e.smem > 48 * 1024) {
        // opt in to large dynamic shared memory once per (device, kernel)
        static std::mutex mu;
        static bool done[64][2][2][16] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        std::lock_guard<std::mutex> lk(mu);
        bool &d = done[dev & 63][dtype][inverse ? 1 : 0][logn];
        if (!d) {
            cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)e.smem);
            if (err != cudaSuccess) return err;
            d = true;
        }
    }
    const long long grid = (a.batch + e.tpc - 1) / e.tpc;
    if (grid <= 0) return cudaSuccess;
    const void *in = a.in;
    void *out = a.out;
    long long batch = a.batch, idist = a.idist, odist = a.odist, istride = a.istride,
              ostride = a.ostride;
    const void *tw = a.tw;
    float scale_f = (float)a.scale;
    double scale_d = a.scale;
    void *args[] = {(void *)&in,      (void *)&out,     (void *)&batch, (void *)&idist, (void *)&odist,
                    (void *)&istride, (void *)&ostride, (void *)&tw,
                    dtype == GFFT_F32 ? (void *)&scale_f : (void *)&scale_d};
    return launch_pdl(fn, dim3((unsigned)grid), dim3(e.threads), args, e.smem, st);
}

}  // namespace gfft
