// real.cu -- real-input transforms and the two-real helpers.
//
// RealFFT<T>::forward (FFTReal.h:204-213) reads n reals as n/2 complex
// z[k] = x[2k] + i x[2k+1], transforms them (Z = FFT_{n/2} z) and applies
// the decimation-in-time adjustment adjust_DIT_impl
// (fft_dit_impl_generic.inl:27-61).  For every k in [0, n/2], with
// j = (n/2 - k) mod n/2 and t_k = sin(2 pi k/n) + i cos(2 pi k/n)
// (DITTwiddle, FFTTwiddle.h:116-127):
//     E = (Z_k + conj Z_j) / 2,   O = (Z_k - conj Z_j) / 2,   F_k = E - t_k O
// which reproduces the reference's special cases F_0 = Re Z_0 + Im Z_0,
// F_{n/2} = Re Z_0 - Im Z_0 and F_{n/4} = conj Z_{n/4}; the full spectrum
// adds F_{n-k} = conj F_k.
//
// k_r2c_fused does all of it in one kernel (one HBM read of n reals, one
// write of n/2+1 or n complex values) while n/2 fits one CTA; larger sizes
// run the multi-pass C2C into the output buffer and then k_dit in place.
#include <algorithm>

#include "internal.h"
#include "plan.h"
#include "dit.cuh"
#include "stockham.cuh"
#include "twiddle.h"

namespace gfft {

// points per thread of the n/2-point C2C: 16 (fp32) / 8 (fp64); 32 for fp32
// half lengths 2^13 and 2^14 (three radix-32 passes instead of four)
template <typename T, int LOGH>
struct RealE {
    static constexpr int value = sizeof(T) == 4 ? ((LOGH == 13 || LOGH == 14) ? 32 : 16) : 8;
};
template <typename T>
struct RealMax {  // log2 of the largest fused half length
    static constexpr int value = sizeof(T) == 4 ? 14 : 13;
};

template <typename T, int LOGH>
struct R2CCfg {
    using SP = StockhamPlan<T, LOGH, RealE<T, LOGH>::value>;
    static constexpr int TPC = SP::G >= 256 ? 1 : 256 / SP::G;
    static constexpr int THREADS = SP::G * TPC;
    static constexpr int SMEM_T = spad_size<T>(SP::N);
    static constexpr size_t SMEM = (size_t)SMEM_T * TPC * sizeof(cpx<T>);
};

// output modes of the real-input kernels
enum R2CMode { R2C_HALF = 0, R2C_FULL = 1, R2C_HALF_X2 = 2 };
// R2C_HALF_X2 doubles bins 1..n/2-1 (and keeps the real DC / Nyquist bins):
// it is the adjoint of the half-spectrum C2R (c2r.cu), whose output counts
// each interior bin twice through the Hermitian extension.
template <int MODE, typename T>
__device__ __forceinline__ cpx<T> r2c_weight(cpx<T> f, long long k, long long H)
{
    if constexpr (MODE == R2C_HALF_X2) {
        if (k > 0 && k < H) return {f.x + f.x, f.y + f.y};
    }
    return f;
}

// in: reals (idist reals between transforms, even), out: complex (odist)
template <typename T, int LOGH, int MODE>
__global__ void __launch_bounds__(R2CCfg<T, LOGH>::THREADS)
    k_r2c_fused(const T *__restrict__ in, cpx<T> *__restrict__ out, long long batch, long long idist,
                long long odist, const cpx<T> *__restrict__ tw, const cpx<T> *__restrict__ dtw, T scale)
{
    using Cfg = R2CCfg<T, LOGH>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G, H = SP::N;  // H = n/2
    extern __shared__ unsigned char smem_raw[];
    cpx<T> *sm = reinterpret_cast<cpx<T> *>(smem_raw);
    const int g = threadIdx.x / G;
    const int t = threadIdx.x - g * G;
    const long long b = (long long)blockIdx.x * Cfg::TPC + g;
    const bool active = b < batch;
    cpx<T> *my = sm + g * Cfg::SMEM_T;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel

    cpx<T> v[E];
    if (active) {
        const cpx<T> *src = reinterpret_cast<const cpx<T> *>(in + b * idist) + t;
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = ldcs_c(src + q * G);
    } else {
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = cpx<T>{(T)0, (T)0};
    }
    stockham_run<T, LOGH, RealE<T, LOGH>::value, false>(
        v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
    __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) my[spad<T>(t + q * G)] = v[q];
    __syncthreads();
    if (!active) return;
    cpx<T> *dst = out + b * odist;
    // pairs (k, H - k), k in [0, H/2]: both bins from the same two values
    // (k = 0 gives bins 0 and H, k = H/2 is its own partner)
#pragma unroll
    for (int q = 0; q <= E / 2; q++) {
        const int k = t + q * G;  // q == E/2 only reaches k == H/2
        if (k > H / 2) break;
        const int j = (H - k) & (H - 1);
        const cpx<T> zk = my[spad<T>(k)], zj = my[spad<T>(j)];
        const cpx<T> fk = scl(dit_value(zk, zj, ldg_c(dtw + k)), scale);
        stcs_c(dst + k, r2c_weight<MODE>(fk, k, H));
        if constexpr (MODE == R2C_FULL) {
            if (k > 0) stcs_c(dst + 2 * H - k, conj(fk));
        }
        if (H - k != k) {
            const cpx<T> fj = scl(dit_value(zj, zk, ldg_c(dtw + (H - k))), scale);
            stcs_c(dst + (H - k), r2c_weight<MODE>(fj, H - k, H));
            if constexpr (MODE == R2C_FULL) {
                if (k > 0) stcs_c(dst + H + k, conj(fj));
            }
        }
    }
}

// Stand-alone adjustment (DIT<T>::apply, fft.h:180-188), in place or not:
// thread p handles the pair (k, H - k), k = p in [0, H/2], reading both Z
// values before writing, so out == in is safe.
// (grid: x over the pairs of a transform, y over the batch, both strided)
template <typename T, int MODE>
__global__ void k_dit(const cpx<T> *in, cpx<T> *out, long long H, long long batch, long long idist,
                      long long odist, const cpx<T> *__restrict__ dtw, T scale)
{
    const long long pairs = H / 2 + 1;
    for (long long b = blockIdx.y; b < batch; b += gridDim.y) {
        const cpx<T> *z = in + b * idist;
        cpx<T> *f = out + b * odist;
        for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < pairs;
             k += (long long)gridDim.x * blockDim.x) {
            const long long j = (H - k) & (H - 1);
            const cpx<T> zk = ld_c(z + (k & (H - 1))), zj = ld_c(z + j);
            const cpx<T> fk = scl(dit_value(zk, zj, ldg_c(dtw + k)), scale);
            const cpx<T> fj = scl(dit_value(zj, zk, ldg_c(dtw + (H - k))), scale);
            st_c(f + k, r2c_weight<MODE>(fk, k, H));
            if (H - k != k) st_c(f + (H - k), r2c_weight<MODE>(fj, H - k, H));
            if constexpr (MODE == R2C_FULL) {
                if (k > 0) st_c(f + 2 * H - k, conj(fk));
                if (k > 0 && H - k != k) st_c(f + H + k, conj(fj));
            }
        }
    }
}

// n == 1: F_0 = x_0 (RealFFT::forward, FFTReal.h:205-207)
template <typename T>
__global__ void k_r2c_one(const T *in, cpx<T> *out, long long batch, long long idist, long long odist, T scale)
{
    for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < batch;
         b += (long long)gridDim.x * blockDim.x)
        st_c(out + b * odist, cpx<T>{in[b * idist] * scale, (T)0});
}

// separate_2x_real_FFT (FFTReal.h:34-66): X = FFT(x), Y = FFT(y) from
// Z = FFT(x + i y); pairs (k, n-k) per thread, so out1/out2 may alias in.
template <typename T>
__global__ void k_separate2x(const cpx<T> *in, cpx<T> *o1, cpx<T> *o2, long long n)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k <= n / 2;
         k += (long long)gridDim.x * blockDim.x) {
        const long long j = (n - k) & (n - 1);
        const cpx<T> zk = ld_c(in + k), zj = ld_c(in + j);
        if (k == 0) {
            st_c(o1, cpx<T>{zk.x, (T)0});
            st_c(o2, cpx<T>{zk.y, (T)0});
            continue;
        }
        const T h = (T)0.5;
        const T xr = (zk.x + zj.x) * h, xi = (zk.y - zj.y) * h;
        const T yr = (zj.y + zk.y) * h, yi = (zj.x - zk.x) * h;
        st_c(o1 + k, cpx<T>{xr, xi});
        st_c(o2 + k, cpx<T>{yr, yi});
        st_c(o1 + j, cpx<T>{xr, -xi});
        st_c(o2 + j, cpx<T>{yr, -yi});
    }
}

// z[r][k] = a[r][k] + i b[r][k] (transform_interleave, fft.h:100-105;
// RealFFT2D::forward_2x, FFTReal.h:114-118); row strides in elements
template <typename T>
__global__ void k_interleave(const T *a, long long lda, const T *b, long long ldb, cpx<T> *z, long long ldz,
                             long long rows, long long cols)
{
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < rows * cols;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long r = idx / cols, k = idx - r * cols;
        st_c(z + r * ldz + k, cpx<T>{a[r * lda + k], b[r * ldb + k]});
    }
}

// DIT<T>(1).apply: F_0 = Re Z_0 + Im Z_0 (fft_dit_impl_generic.inl:30-35)
template <typename T>
__global__ void k_dit_one(const cpx<T> *in, cpx<T> *out)
{
    const cpx<T> z = ld_c(in);
    st_c(out, cpx<T>{z.x + z.y, (T)0});
}

// in-place bit-reversal permutation (for bit-reversed-input transforms
// above the fused limit): swap x[i] and x[rev(i)] once per pair
template <typename T>
__global__ void k_bitrev_swap(cpx<T> *x, int logn, long long batch, long long dist)
{
    const long long n = 1LL << logn;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n * batch;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long b = idx >> logn;
        const long long i = idx & (n - 1);
        const long long r = (long long)(__brevll((unsigned long long)i) >> (64 - logn));
        if (r > i) {
            cpx<T> *p = x + b * dist;
            const cpx<T> u = ld_c(p + i), w = ld_c(p + r);
            st_c(p + i, w);
            st_c(p + r, u);
        }
    }
}

// ---------------------------------------------------------------------------
// host side

namespace {

struct R2CEntry {
    const void *fn[3];
    int threads, tpc;
    size_t smem, twcount;
    void (*fill)(void *);
};

template <typename T, int LOGH>
void r2c_fill(void *buf)
{
    stockham_fill_twiddles<T, LOGH, RealE<T, LOGH>::value>(
        static_cast<cpx<T> *>(buf), [](long long k, long long M, cpx<T> *w) { forward_root<T>(k, M, &w->x, &w->y); });
}

template <typename T, int LOGH>
R2CEntry make_r2c()
{
    using Cfg = R2CCfg<T, LOGH>;
    return R2CEntry{{(const void *)&k_r2c_fused<T, LOGH, R2C_HALF>, (const void *)&k_r2c_fused<T, LOGH, R2C_FULL>,
                     (const void *)&k_r2c_fused<T, LOGH, R2C_HALF_X2>},
                    Cfg::THREADS, Cfg::TPC, Cfg::SMEM, (size_t)Cfg::SP::TW, &r2c_fill<T, LOGH>};
}

template <typename T, int... L>
const R2CEntry *r2c_table(std::integer_sequence<int, L...>)
{
    static const R2CEntry tab[] = {make_r2c<T, L>()...};
    return tab;
}

const R2CEntry &r2c_entry(int dtype, int logh)
{
    if (dtype == GFFT_F32)
        return r2c_table<float>(std::make_integer_sequence<int, RealMax<float>::value + 1>{})[logh];
    return r2c_table<double>(std::make_integer_sequence<int, RealMax<double>::value + 1>{})[logh];
}

unsigned grid_for(long long work, int threads)
{
    long long g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 152 * 64) g = 152 * 64;
    return (unsigned)g;
}

}  // namespace

int r2c_fused_max_logh(int dtype) { return dtype == GFFT_F32 ? RealMax<float>::value : RealMax<double>::value; }
size_t r2c_twiddle_count(int dtype, int logh) { return r2c_entry(dtype, logh).twcount; }
void r2c_twiddle_fill(int dtype, int logh, void *buf) { r2c_entry(dtype, logh).fill(buf); }

// t_k = sin(2 pi k/n) + i cos(2 pi k/n), k in [0, n/2]
void dit_twiddle_fill(int dtype, int logn, void *buf)
{
    const long long n = 1LL << logn;
    for (long long k = 0; k <= n / 2; k++) {
        double c, s;
        exact_root(k, n, &c, &s);
        if (dtype == GFFT_F32) {
            static_cast<float *>(buf)[2 * k] = (float)s;
            static_cast<float *>(buf)[2 * k + 1] = (float)c;
        } else {
            static_cast<double *>(buf)[2 * k] = s;
            static_cast<double *>(buf)[2 * k + 1] = c;
        }
    }
}

cudaError_t launch_r2c_fused(int dtype, int logh, int mode, const void *in, void *out, long long batch,
                             long long idist, long long odist, const void *tw, const void *dtw, cudaStream_t st,
                             double scale)
{
    const R2CEntry &e = r2c_entry(dtype, logh);
    const void *fn = e.fn[mode];
    cudaError_t err = ensure_smem(fn, e.smem);
    if (err != cudaSuccess) return err;
    const long long grid = (batch + e.tpc - 1) / e.tpc;
    float scale_f = (float)scale;
    void *args[] = {(void *)&in,  (void *)&out, (void *)&batch, (void *)&idist, (void *)&odist, (void *)&tw,
                    (void *)&dtw, dtype == GFFT_F32 ? (void *)&scale_f : (void *)&scale};
    return launch_pdl(fn, dim3((unsigned)grid), dim3(e.threads), args, e.smem, st);
}

template <typename T>
void dit_launch(int mode, dim3 g, const void *in, void *out, long long H, long long batch, long long idist,
                long long odist, const void *dtw, cudaStream_t st, T sc)
{
    auto i = (const cpx<T> *)in;
    auto o = (cpx<T> *)out;
    auto d = (const cpx<T> *)dtw;
    if (mode == R2C_HALF) k_dit<T, R2C_HALF><<<g, 256, 0, st>>>(i, o, H, batch, idist, odist, d, sc);
    else if (mode == R2C_FULL) k_dit<T, R2C_FULL><<<g, 256, 0, st>>>(i, o, H, batch, idist, odist, d, sc);
    else k_dit<T, R2C_HALF_X2><<<g, 256, 0, st>>>(i, o, H, batch, idist, odist, d, sc);
}

cudaError_t launch_dit(int dtype, int mode, const void *in, void *out, long long H, long long batch,
                       long long idist, long long odist, const void *dtw, cudaStream_t st, double scale)
{
    // x over the pairs of a transform (256 a CTA), y over the batch; about
    // 16K CTAs at most, the kernel strides over the rest
    const long long gy = std::min<long long>(std::max<long long>(batch, 1), 65535);
    const long long gx = std::max<long long>(1, std::min<long long>((H / 2 + 1 + 255) / 256, std::max<long long>(1, 16384 / gy)));
    const dim3 g((unsigned)gx, (unsigned)gy);
    if (dtype == GFFT_F32) dit_launch<float>(mode, g, in, out, H, batch, idist, odist, dtw, st, (float)scale);
    else dit_launch<double>(mode, g, in, out, H, batch, idist, odist, dtw, st, scale);
    return cudaGetLastError();
}

cudaError_t launch_r2c_one(int dtype, const void *in, void *out, long long batch, long long idist, long long odist,
                           cudaStream_t st, double scale)
{
    const unsigned g = grid_for(batch, 256);
    if (dtype == GFFT_F32)
        k_r2c_one<float><<<g, 256, 0, st>>>((const float *)in, (cpx<float> *)out, batch, idist, odist, (float)scale);
    else k_r2c_one<double><<<g, 256, 0, st>>>((const double *)in, (cpx<double> *)out, batch, idist, odist, scale);
    return cudaGetLastError();
}

cudaError_t launch_separate2x(int dtype, const void *in, void *o1, void *o2, long long n, cudaStream_t st)
{
    const unsigned g = grid_for(n / 2 + 1, 256);
    if (dtype == GFFT_F32) k_separate2x<float><<<g, 256, 0, st>>>((const cpx<float> *)in, (cpx<float> *)o1, (cpx<float> *)o2, n);
    else k_separate2x<double><<<g, 256, 0, st>>>((const cpx<double> *)in, (cpx<double> *)o1, (cpx<double> *)o2, n);
    return cudaGetLastError();
}

cudaError_t launch_interleave(int dtype, const void *a, long long lda, const void *b, long long ldb, void *z,
                              long long ldz, long long rows, long long cols, cudaStream_t st)
{
    const unsigned g = grid_for(rows * cols, 256);
    if (dtype == GFFT_F32)
        k_interleave<float><<<g, 256, 0, st>>>((const float *)a, lda, (const float *)b, ldb, (cpx<float> *)z, ldz, rows, cols);
    else
        k_interleave<double><<<g, 256, 0, st>>>((const double *)a, lda, (const double *)b, ldb, (cpx<double> *)z, ldz, rows, cols);
    return cudaGetLastError();
}

cudaError_t launch_dit_one(int dtype, const void *in, void *out, cudaStream_t st)
{
    if (dtype == GFFT_F32) k_dit_one<float><<<1, 1, 0, st>>>((const cpx<float> *)in, (cpx<float> *)out);
    else k_dit_one<double><<<1, 1, 0, st>>>((const cpx<double> *)in, (cpx<double> *)out);
    return cudaGetLastError();
}

cudaError_t launch_bitrev_swap(int dtype, void *x, int logn, long long batch, long long dist, cudaStream_t st)
{
    const unsigned g = grid_for((1LL << logn) * batch, 256);
    if (dtype == GFFT_F32) k_bitrev_swap<float><<<g, 256, 0, st>>>((cpx<float> *)x, logn, batch, dist);
    else k_bitrev_swap<double><<<g, 256, 0, st>>>((cpx<double> *)x, logn, batch, dist);
    return cudaGetLastError();
}

}  // namespace gfft
