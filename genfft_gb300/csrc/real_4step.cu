// real_4step.cu -- the row pass of a four-step real-input transform with the
// real-FFT post-twiddle (DIT adjustment) fused in, for n above the fused
// single-kernel limit (RealFFT<T>::forward half = true, FFTReal.h:186-221).
//
// The n reals are read as H = n/2 complex values and transformed by the
// four-step split H = A * B (tiles.cuh): the column pass leaves
// Y[B k1 + b] in the workspace; the row pass FFTs each row k1 and produces
// Z[k1 + A k2].  The DIT pass (dit.cuh) needs Z_k and Z_{H-k} together,
// and for k = k1 + A k2 the partner is
//     H - k = (A - k1) + A (B - 1 - k2)        (k1 >= 1),
//     H - k = 0 + A (B - k2)                   (k1 = 0),
// i.e. row A - k1 mirrored, or row 0 itself.  So a CTA transforms CH rows
// k1 = 1 + CH p + s (s < CH) together with their mirrors A - k1, applies the
// adjustment to every pair straight from shared memory and stores both
// bins of the half spectrum (runs of CH bins); one more CTA does row 0
// (and the Nyquist bin).  The separate DIT pass over the whole output --
// a full extra read and write of the spectrum -- is gone.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <set>

#include "dit.cuh"
#include "internal.h"
#include "plan.h"
#include "stockham.cuh"
#include "twiddle.h"

namespace gfft {

template <typename T, int LOGB, int CH, int E_>
struct RowDitCfg {
    using SP = StockhamPlan<T, LOGB, E_>;
    static constexpr int B = SP::N;
    static constexpr int ROWS = 2 * CH;                 // CH rows and their mirrors
    static constexpr int THREADS = SP::G * ROWS;
    static constexpr int ROWP = SP::P > 1 ? SP::SMEM : 0;  // Stockham exchange pitch
    static constexpr int ZP = B + B / 16 + 1;           // pitch of the Z tile
    static constexpr int SMEM_ELEMS = (ROWP > ZP ? ROWP : ZP) * ROWS;
    static constexpr size_t SMEM = (size_t)SMEM_ELEMS * sizeof(cpx<T>);
};

// in: the column pass's output, rows of B; out: the half spectrum, H + 1
// bins per transform.  grid: (A / (2 CH) + 1) x batch.
template <typename T, int LOGB, int CH, int E_>
__global__ void __launch_bounds__(RowDitCfg<T, LOGB, CH, E_>::THREADS, 1024 / RowDitCfg<T, LOGB, CH, E_>::THREADS)
    k_rowpass_dit(const cpx<T> *__restrict__ in, cpx<T> *__restrict__ out, long long A, long long idist,
                  long long odist, const cpx<T> *__restrict__ tw, const cpx<T> *__restrict__ dtw, T scale)
{
    using Cfg = RowDitCfg<T, LOGB, CH, E_>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G, B = Cfg::B;
    extern __shared__ unsigned char smem_raw[];
    cpx<T> *sm = reinterpret_cast<cpx<T> *>(smem_raw);

    const long long P = A / (2 * CH);
    const long long p = blockIdx.x;
    const bool row0 = p == P;  // the block of row 0 (self-paired)
    const long long b = blockIdx.y;
    const long long H = A * B;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel
    const int s = threadIdx.x / G, t = threadIdx.x - s * G;
    // row of slot s: lo slots 1 + CH p + s, hi slots their mirrors A - k1
    long long k1;
    if (row0) k1 = 0;
    else if (s < CH) k1 = 1 + CH * p + s;
    else k1 = A - 1 - CH * p - (s - CH);
    const bool active = !row0 || s == 0;

    cpx<T> v[E];
    {
        const cpx<T> *src = in + b * idist + k1 * B + t;
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = active ? ld_c(src + q * G) : cpx<T>{(T)0, (T)0};
    }
    cpx<T> *my = sm + s * Cfg::ROWP;
    stockham_run<T, LOGB, E_, false>(
        v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
    __syncthreads();
    // Z tile: slot s, column k2 at s * ZP + k2 + k2 / 16
#pragma unroll
    for (int q = 0; q < E; q++) {
        const int k2 = t + q * G;
        sm[s * Cfg::ZP + k2 + (k2 >> 4)] = v[q];
    }
    __syncthreads();
    auto Z = [sm](int slot, int k2) { return sm[slot * Cfg::ZP + k2 + (k2 >> 4)]; };
    cpx<T> *dst = out + b * odist;
    if (!row0) {
        // pairs (lo slot s2, column k2) <-> (hi slot s2 + CH, column B - 1 - k2);
        // consecutive threads take consecutive rows: runs of CH bins
        for (int idx = threadIdx.x; idx < CH * B; idx += Cfg::THREADS) {
            const int s2 = idx % CH, k2 = idx / CH;
            const long long k = 1 + CH * p + s2 + A * k2;
            const long long j = H - k;
            const cpx<T> zk = Z(s2, k2), zj = Z(s2 + CH, B - 1 - k2);
            st_c(dst + k, scl(dit_value(zk, zj, ldg_c(dtw + k)), scale));
            st_c(dst + j, scl(dit_value(zj, zk, ldg_c(dtw + j)), scale));
        }
    } else {
        // row 0: bins A k2 <-> A (B - k2), k2 in [0, B/2]; k2 = 0 also
        // gives the Nyquist bin H
        for (int k2 = threadIdx.x; k2 <= B / 2; k2 += Cfg::THREADS) {
            const long long k = A * k2, j = H - k;
            const cpx<T> zk = Z(0, k2), zj = Z(0, (B - k2) & (B - 1));
            st_c(dst + k, scl(dit_value(zk, zj, ldg_c(dtw + k)), scale));
            st_c(dst + j, scl(dit_value(zj, zk, ldg_c(dtw + j)), scale));
        }
    }
}

// ---------------------------------------------------------------------------
// host side

namespace {

template <typename T, int LOGB, int E>
void rowdit_fill(void *buf)
{
    stockham_fill_twiddles<T, LOGB, E>(static_cast<cpx<T> *>(buf),
                                       [](long long k, long long M, cpx<T> *w) { forward_root<T>(k, M, &w->x, &w->y); });
}

template <typename T, int LOGB, int CH, int E>
RowDitKernel make_rowdit()
{
    using Cfg = RowDitCfg<T, LOGB, CH, E>;
    RowDitKernel k;
    k.fn = (const void *)&k_rowpass_dit<T, LOGB, CH, E>;
    k.threads = Cfg::THREADS;
    k.smem = Cfg::SMEM;
    k.ch = CH;
    k.logb = LOGB;
    k.twcount = (size_t)StockhamPlan<T, LOGB, E>::TW;
    k.fill = &rowdit_fill<T, LOGB, E>;
    return k;
}

}  // namespace

// fp32 row lengths 2^8 .. 2^12 (half lengths 2^15 .. 2^24)
const RowDitKernel *rowdit_find(int dtype, int logb)
{
    if (dtype != GFFT_F32) return nullptr;
    // rows per half-block measured on GB300 (half-spectrum R2C, 512 MB
    // batches): 8 for 256- and 512-point rows; 1024-thread blocks (8, 4, 2
    // rows) for 1024 .. 4096-point rows, 6-29 % faster there than 512
    static const RowDitKernel tab[] = {make_rowdit<float, 8, 8, 16>(), make_rowdit<float, 9, 8, 16>(),
                                       make_rowdit<float, 10, 8, 16>(), make_rowdit<float, 11, 4, 16>(),
                                       make_rowdit<float, 12, 2, 16>()};
    if (logb < 8 || logb > 12) return nullptr;
    return &tab[logb - 8];
}

cudaError_t launch_rowpass_dit(const RowDitKernel &k, const void *in, void *out, long long A, long long batch,
                               long long idist, long long odist, const void *tw, const void *dtw, cudaStream_t st,
                               double scale)
{
    if (k.smem > 48 * 1024) {
        static std::mutex mu;
        static std::set<std::pair<int, const void *>> done;
        int dev = 0;
        cudaGetDevice(&dev);
        std::lock_guard<std::mutex> lk(mu);
        if (!done.count({dev, k.fn})) {
            cudaError_t e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
            if (e != cudaSuccess) return e;
            done.insert({dev, k.fn});
        }
    }
    float scale_f = (float)scale;
    const long long blocks = A / (2 * k.ch) + 1;
    for (long long b0 = 0; b0 < batch; b0 += 65535) {
        const long long nb = std::min<long long>(65535, batch - b0);
        const void *src = static_cast<const char *>(in) + (size_t)(b0 * idist) * 8;
        void *dst = static_cast<char *>(out) + (size_t)(b0 * odist) * 8;
        void *args[] = {(void *)&src, (void *)&dst, (void *)&A, (void *)&idist, (void *)&odist, (void *)&tw,
                        (void *)&dtw, (void *)&scale_f};
        cudaError_t e = launch_pdl(k.fn, dim3((unsigned)blocks, (unsigned)nb), dim3(k.threads), args, k.smem, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace gfft
