// c2r.cu -- half-spectrum inverse (C2R) and the real-FFT adjoint.
//
// The reference has no half-spectrum inverse (README.txt:51-52,
// FFTReal.h:127-130 asserts TODO); this is the pair of RealFFT::forward.
// Given bins F_0 .. F_{n/2} of a Hermitian spectrum it returns the n reals
//     x_j = sum_{k=0}^{n-1} F_k exp(+2 pi i jk/n)        (unscaled)
// by inverting the decimation-in-time adjustment of the forward transform
// (fft_dit_impl_generic.inl:44-54): with p = n/2 - k and the DIT twiddle
// t_k = sin(2 pi k/n) + i cos(2 pi k/n),
//     Z'_k = (F_k + conj F_p) + conj(t_k) (conj F_p - F_k),   k < n/2
// then x_{2m} + i x_{2m+1} = IFFT_{n/2}(Z')_m.  The imaginary parts of F_0
// and F_{n/2} are ignored (the Hermitian projection).
//
// Input weightings make the same kernel the adjoint of the real-input
// transform for reverse-mode differentiation (the "real-FFT Hermitian
// weighting"): the gradient of x -> Y = rfft(x) is
//     grad_x_j = Re sum_k g_k exp(+2 pi i jk/n)
// over the bins Y exposes, which is C2R of g with interior bins halved
// (half spectrum) or folded as (g_k + conj g_{n-k}) / 2 (full spectrum).
#include <algorithm>

#include "internal.h"
#include "plan.h"
#include "stockham.cuh"
#include "twiddle.h"

namespace gfft {

enum C2RWeight { W_PLAIN = 0, W_HALF_INTERIOR = 1, W_FOLD_FULL = 2 };

// points per thread: the same as the R2C kernels (real.cu), whose twiddle
// table this kernel shares
template <typename T, int LOGH>
struct C2RE {
    static constexpr int value = sizeof(T) == 4 ? ((LOGH == 13 || LOGH == 14) ? 32 : 16) : 8;
};
template <typename T>
struct C2RMax {
    static constexpr int value = sizeof(T) == 4 ? 14 : 13;
};

// bin k of the (weighted, projected) half spectrum; g holds H+1 bins, or
// 2H bins for W_FOLD_FULL
template <int W, typename T, typename Get>
__device__ __forceinline__ cpx<T> c2r_bin(Get g, int k, int H)
{
    cpx<T> b = g(k);
    if (k == 0 || k == H) return cpx<T>{b.x, (T)0};
    const T h = (T)0.5;
    if constexpr (W == W_HALF_INTERIOR) return cpx<T>{b.x * h, b.y * h};
    if constexpr (W == W_FOLD_FULL) {
        const cpx<T> m = g(2 * H - k);
        return cpx<T>{(b.x + m.x) * h, (b.y - m.y) * h};
    }
    return b;
}

// Z'_k from bins k and p = H - k
template <typename T>
__device__ __forceinline__ cpx<T> c2r_pre_value(cpx<T> fk, cpx<T> fp, cpx<T> t)
{
    const cpx<T> s{fk.x + fp.x, fk.y - fp.y};   // F_k + conj F_p
    const cpx<T> d{fp.x - fk.x, -fp.y - fk.y};  // conj F_p - F_k
    const cpx<T> ct{t.x, -t.y};                 // conj t_k
    const cpx<T> m = cmul(ct, d);
    return {s.x + m.x, s.y + m.y};
}

template <typename T, int LOGH, int W>
struct C2RCfg {
    using SP = StockhamPlan<T, LOGH, C2RE<T, LOGH>::value>;
    static constexpr int H = SP::N;
    static constexpr int TPC = SP::G >= 256 ? 1 : 256 / SP::G;
    static constexpr int THREADS = SP::G * TPC;
    static constexpr int SPAD = spad_size<T>(H);
    // shared slots a transform: its input bins (H + 1, or 2H for the folded
    // full spectrum), then the Stockham exchanges
    static constexpr int NIN = W == W_FOLD_FULL ? 2 * H : H + 1;
    static constexpr int SMEM_T = SPAD > NIN ? SPAD : NIN;
    static constexpr size_t SMEM = (size_t)SMEM_T * TPC * sizeof(cpx<T>);
};
// the most dynamic shared memory a CTA can opt in to on GB300 (227 KB)
constexpr size_t C2R_SMEM_MAX = 227 * 1024;

// in: bins (idist complex between transforms), out: reals (odist reals, even)
template <typename T, int LOGH, int W>
__global__ void __launch_bounds__(C2RCfg<T, LOGH, W>::THREADS)
    k_c2r_fused(const cpx<T> *__restrict__ in, T *__restrict__ out, long long batch, long long idist,
                long long odist, const cpx<T> *__restrict__ tw, const cpx<T> *__restrict__ dtw, T scale)
{
    using Cfg = C2RCfg<T, LOGH, W>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G, H = SP::N;
    constexpr int NIN = Cfg::NIN;
    extern __shared__ unsigned char smem_raw[];
    cpx<T> *sm = reinterpret_cast<cpx<T> *>(smem_raw);
    const int g = threadIdx.x / G;
    const int t = threadIdx.x - g * G;
    const long long b = (long long)blockIdx.x * Cfg::TPC + g;
    const bool active = b < batch;
    cpx<T> *my = sm + g * Cfg::SMEM_T;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel

    if (active) {
        // E loads in flight a thread (a loop of one load and one store a
        // step keeps a single load in flight), then their stores
        const cpx<T> *src = in + b * idist;
        constexpr int PER = (NIN + G - 1) / G;
#pragma unroll
        for (int c0 = 0; c0 < PER; c0 += E) {
            cpx<T> tmp[E];
#pragma unroll
            for (int j = 0; j < E; j++) {
                const int i = t + (c0 + j) * G;
                if (c0 + j < PER && i < NIN) tmp[j] = ldcs_c(src + i);
            }
#pragma unroll
            for (int j = 0; j < E; j++) {
                const int i = t + (c0 + j) * G;
                if (c0 + j < PER && i < NIN) my[i] = tmp[j];
            }
        }
    }
    __syncthreads();
    cpx<T> v[E];
    auto get = [my](int i) { return my[i]; };
#pragma unroll
    for (int q = 0; q < E; q++) {
        const int k = t + q * G;
        const int p = H - k;
        v[q] = c2r_pre_value(c2r_bin<W, T>(get, k, H), c2r_bin<W, T>(get, p, H), ldg_c(dtw + k));
    }
    __syncthreads();
    stockham_run<T, LOGH, C2RE<T, LOGH>::value, true>(
        v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
    if (active) {
        cpx<T> *dst = reinterpret_cast<cpx<T> *>(out + b * odist) + t;
#pragma unroll
        for (int q = 0; q < E; q++) stcs_c(dst + q * G, scl(v[q], scale));
    }
}

// pre-pass for sizes above the fused limit: Z' (H complex) into the output
// buffer; pairs (k, H-k) per thread
// (grid: x over the pairs of a transform, y over the batch, both strided)
template <typename T, int W>
__global__ void k_c2r_pre(const cpx<T> *in, cpx<T> *out, long long H, long long batch, long long idist,
                          long long odist, const cpx<T> *__restrict__ dtw)
{
    const int pairs = (int)(H / 2 + 1);
    for (long long b = blockIdx.y; b < batch; b += gridDim.y) {
        const cpx<T> *f = in + b * idist;
        cpx<T> *z = out + b * odist;
        auto get = [f](int i) { return ld_c(f + i); };
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < pairs; k += gridDim.x * blockDim.x) {
            const int p = (int)H - k;
            const cpx<T> fk = c2r_bin<W, T>(get, k, (int)H), fp = c2r_bin<W, T>(get, p, (int)H);
            st_c(z + k, c2r_pre_value(fk, fp, ldg_c(dtw + k)));
            if (k > 0 && p != k) st_c(z + p, c2r_pre_value(fp, fk, ldg_c(dtw + p)));
        }
    }
}

// n == 1: x_0 = Re F_0
template <typename T>
__global__ void k_c2r_one(const cpx<T> *in, T *out, long long batch, long long idist, long long odist, T scale)
{
    for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < batch;
         b += (long long)gridDim.x * blockDim.x)
        out[b * odist] = ld_c(in + b * idist).x * scale;
}

// ---------------------------------------------------------------------------
// host side

namespace {

struct C2REntry {
    const void *fn[3];
    int threads, tpc;
    size_t smem[3];  // per weight mode
};

template <typename T, int LOGH>
C2REntry make_c2r()
{
    using Cfg = C2RCfg<T, LOGH, W_PLAIN>;
    return C2REntry{{(const void *)&k_c2r_fused<T, LOGH, W_PLAIN>, (const void *)&k_c2r_fused<T, LOGH, W_HALF_INTERIOR>,
                     (const void *)&k_c2r_fused<T, LOGH, W_FOLD_FULL>},
                    Cfg::THREADS,
                    Cfg::TPC,
                    {Cfg::SMEM, C2RCfg<T, LOGH, W_HALF_INTERIOR>::SMEM, C2RCfg<T, LOGH, W_FOLD_FULL>::SMEM}};
}

template <typename T, int... L>
const C2REntry *c2r_table(std::integer_sequence<int, L...>)
{
    static const C2REntry tab[] = {make_c2r<T, L>()...};
    return tab;
}

const C2REntry &c2r_entry(int dtype, int logh)
{
    if (dtype == GFFT_F32)
        return c2r_table<float>(std::make_integer_sequence<int, C2RMax<float>::value + 1>{})[logh];
    return c2r_table<double>(std::make_integer_sequence<int, C2RMax<double>::value + 1>{})[logh];
}

// x over the pairs of a transform (256 a CTA), y over the batch; about 16K
// CTAs at most, the kernels stride over the rest
dim3 pair_grid(long long pairs, long long batch)
{
    const long long y = std::min<long long>(std::max<long long>(batch, 1), 65535);
    const long long x = std::max<long long>(1, std::min<long long>((pairs + 255) / 256, std::max<long long>(1, 16384 / y)));
    return dim3((unsigned)x, (unsigned)y);
}

unsigned grid_for2(long long work, int threads)
{
    long long g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 152 * 64) g = 152 * 64;
    return (unsigned)g;
}

template <typename T>
void pre_launch(int w, dim3 g, const void *in, void *out, long long H, long long batch, long long idist,
                long long odist, const void *dtw, cudaStream_t st)
{
    auto i = (const cpx<T> *)in;
    auto o = (cpx<T> *)out;
    auto d = (const cpx<T> *)dtw;
    if (w == W_PLAIN) k_c2r_pre<T, W_PLAIN><<<g, 256, 0, st>>>(i, o, H, batch, idist, odist, d);
    else if (w == W_HALF_INTERIOR) k_c2r_pre<T, W_HALF_INTERIOR><<<g, 256, 0, st>>>(i, o, H, batch, idist, odist, d);
    else k_c2r_pre<T, W_FOLD_FULL><<<g, 256, 0, st>>>(i, o, H, batch, idist, odist, d);
}

}  // namespace

int c2r_fused_max_logh(int dtype) { return dtype == GFFT_F32 ? C2RMax<float>::value : C2RMax<double>::value; }

bool c2r_fused_fits(int dtype, int logh, int wmode)
{
    return logh <= c2r_fused_max_logh(dtype) && c2r_entry(dtype, logh).smem[wmode] <= C2R_SMEM_MAX;
}

cudaError_t launch_c2r_fused(int dtype, int logh, int wmode, const void *in, void *out, long long batch,
                             long long idist, long long odist, const void *tw, const void *dtw, cudaStream_t st,
                             double scale)
{
    const C2REntry &e = c2r_entry(dtype, logh);
    const void *fn = e.fn[wmode];
    const size_t smem = e.smem[wmode];
    if (smem > C2R_SMEM_MAX) return cudaErrorInvalidValue;  // the planner routes these elsewhere
    cudaError_t err = ensure_smem(fn, smem);
    if (err != cudaSuccess) return err;
    const long long grid = (batch + e.tpc - 1) / e.tpc;
    float scale_f = (float)scale;
    void *args[] = {(void *)&in,  (void *)&out, (void *)&batch, (void *)&idist, (void *)&odist, (void *)&tw,
                    (void *)&dtw, dtype == GFFT_F32 ? (void *)&scale_f : (void *)&scale};
    return launch_pdl(fn, dim3((unsigned)grid), dim3(e.threads), args, smem, st);
}

cudaError_t launch_c2r_pre(int dtype, int wmode, const void *in, void *out, long long H, long long batch,
                           long long idist, long long odist, const void *dtw, cudaStream_t st)
{
    const dim3 g = pair_grid(H / 2 + 1, batch);
    if (dtype == GFFT_F32) pre_launch<float>(wmode, g, in, out, H, batch, idist, odist, dtw, st);
    else pre_launch<double>(wmode, g, in, out, H, batch, idist, odist, dtw, st);
    return cudaGetLastError();
}

cudaError_t launch_c2r_one(int dtype, const void *in, void *out, long long batch, long long idist, long long odist,
                           cudaStream_t st, double scale)
{
    const unsigned g = grid_for2(batch, 256);
    if (dtype == GFFT_F32)
        k_c2r_one<float><<<g, 256, 0, st>>>((const cpx<float> *)in, (float *)out, batch, idist, odist, (float)scale);
    else k_c2r_one<double><<<g, 256, 0, st>>>((const cpx<double> *)in, (double *)out, batch, idist, odist, scale);
    return cudaGetLastError();
}

}  // namespace gfft
