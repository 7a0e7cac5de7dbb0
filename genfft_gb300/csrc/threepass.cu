// threepass.cu -- C2C of fp32 n = 2^19 .. 2^24 as three passes of short
// tiles, n = A B C (A = 2^a, B = 2^b, C = 2^c, each 2^6 .. 2^8):
//   n = B C n1 + C n2 + n3,  k = k1 + A k2 + A B k3
//   pass 1  for every m = C n2 + n3: the A-point FFT down x[B C n1 + m],
//           times W_n^(m k1)                          -> Y1[k1][m]
//   pass 2  for every (k1, n3): the B-point FFT down Y1[k1][C n2 + n3],
//           times W_(BC)^(n3 k2), in place            -> Y2[k1][k2][n3]
//   pass 3  for every (k1, k2): the C-point FFT along Y2[k1][k2][.],
//           stored at X[k1 + A k2 + A B k3]
// Passes 1 and 2 are the four-step column pass with its inter-pass twiddle
// (tiles.cuh), applied twice; pass 3 is the row pass with its transposed
// store, over rows r = k1 + A k2 read from k1 B C + k2 C.  Every tile is a
// few thousand points (four 256-thread or eight 128-thread CTAs an SM) and
// every global access comes in runs of 128-512 bytes, where the two-pass
// split of these lengths needs tiles of 2^10 .. 2^12-point FFTs with
// 32-64-byte runs at one or two CTAs an SM.  The cost is a third pass
// through the workspace.  Replaces FFT<float>::transform<inv> (fft.h:80-85)
// for these lengths.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "internal.h"
#include "threepass.h"
#include "tiles.cuh"
#include "twiddle.h"

namespace gfft {

using c32 = cpx<float>;

// Column tile: C columns of 2^L points, rows `ld` apart; item y of the grid
// (plus y0) at y * idist in `in` and y * odist in `out`.  Output point k of
// column col is multiplied by W^(col k) from hi[e >> lo_bits] * lo[e & mask],
// e = col k & nmask.  `in` may equal `out`: every CTA loads its whole tile
// before it stores.
template <int L, int C, int MINB, bool INV>
__global__ void __launch_bounds__(StockhamPlan<float, L, 16>::G *C, MINB)
    k3_col(const c32 *in, c32 *out, long long ld, long long idist, long long odist, long long y0,
           const c32 *__restrict__ tw, const c32 *__restrict__ tlo, const c32 *__restrict__ thi, int lo_bits,
           unsigned nmask)
{
    using SP = StockhamPlan<float, L, 16>;
    constexpr int E = SP::E, G = SP::G;
    constexpr int PITCH = tile_pitch<float>(SP::N, C);
    extern __shared__ unsigned char smem_raw[];
    c32 *const sm = reinterpret_cast<c32 *>(smem_raw);
    const int s = threadIdx.x % C, t = threadIdx.x / C;
    const unsigned col = blockIdx.x * C + s;
    const long long y = y0 + blockIdx.y;
    const unsigned lo_mask = (1u << lo_bits) - 1u;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel
    c32 v[E];
    const c32 *src = in + y * idist + col + (long long)t * ld;
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = ldcs_c(src + (long long)q * G * ld);
    c32 *const my = sm + s * PITCH;
    stockham_run<float, L, 16, INV>(
        v, t, [my](int i) -> c32 & { return my[spad<float>(i)]; }, tw, []() { __syncthreads(); });
    c32 *dst = out + y * odist + col + (long long)t * ld;
#pragma unroll
    for (int q = 0; q < E; q++) {
        const unsigned e = (col * (unsigned)(t + q * G)) & nmask;
        const c32 w = cmul(ldg_c(thi + (e >> lo_bits)), ldg_c(tlo + (e & lo_mask)));
        // keep the twiddle loads of later points from being hoisted
        if ((q & 3) == 3) asm volatile("" ::: "memory");
        st_c(dst + (long long)q * G * ld, twmul<INV>(v[q], w));
    }
}

// Row tile of pass 3: R rows r of 2^L points, row r = k1 + 2^la k2 read
// from in[y * idist + k1 * lda + k2 * ldb]; output k of row r stored at
// out[y * odist + r + k * ostride] through a transposed tile (runs of R).
template <int L, int R, int MINB, bool INV>
__global__ void __launch_bounds__(StockhamPlan<float, L, 16>::G *R, MINB)
    k3_row(const c32 *__restrict__ in, c32 *__restrict__ out, int la, long long lda, long long ldb,
           long long ostride, long long idist, long long odist, const c32 *__restrict__ tw, float scale)
{
    using SP = StockhamPlan<float, L, 16>;
    constexpr int E = SP::E, G = SP::G, N = SP::N;
    constexpr int THREADS = G * R;
    constexpr int ROWP = SP::SMEM;   // slots a row while it is transformed
    constexpr int XROW = R + 1;      // transposed tile: one pad slot per output run
    extern __shared__ unsigned char smem_raw[];
    c32 *const sm = reinterpret_cast<c32 *>(smem_raw);
    const int s = threadIdx.x / G, t = threadIdx.x - s * G;
    const long long r0 = (long long)blockIdx.x * R;
    const long long r = r0 + s;
    const long long y = blockIdx.y;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel
    const long long k1 = r & ((1LL << la) - 1), k2 = r >> la;
    const c32 *src = in + y * idist + k1 * lda + k2 * ldb + t;
    c32 v[E];
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = ld_c(src + q * G);
    c32 *const my = sm + s * ROWP;
    stockham_run<float, L, 16, INV>(
        v, t, [my](int i) -> c32 & { return my[spad<float>(i)]; }, tw, []() { __syncthreads(); });
    __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) sm[(t + q * G) * XROW + s] = v[q];
    __syncthreads();
    c32 *dst = out + y * odist + r0;
#pragma unroll
    for (int m = 0; m < E; m++) {
        const int idx = threadIdx.x + m * THREADS;
        const int s2 = idx % R, k = idx / R;
        if (k < N) stcs_c(dst + s2 + (long long)k * ostride, scl(sm[k * XROW + s2], scale));
    }
}

template <int L, int C>
constexpr size_t col_smem()
{
    return (size_t)tile_pitch<float>(1 << L, C) * C * sizeof(c32);
}
template <int L, int R>
constexpr size_t row_smem()
{
    using SP = StockhamPlan<float, L, 16>;
    const size_t a = (size_t)SP::SMEM * R, x = (size_t)(1 << L) * (R + 1);
    return (a > x ? a : x) * sizeof(c32);
}

namespace {

template <int L>
void tp_fill(void *buf)
{
    stockham_fill_twiddles<float, L, 16>(static_cast<c32 *>(buf),
                                         [](long long k, long long M, c32 *w) { forward_root<float>(k, M, &w->x, &w->y); });
}

// resident CTAs an SM at 64 registers a thread (65536 / (64 THREADS))
template <int THREADS>
struct Minb {
    static constexpr int value = 1024 / THREADS > 8 ? 8 : 1024 / THREADS;
};

std::map<int, std::vector<ThreePass>> &tp_registry()
{
    static std::map<int, std::vector<ThreePass>> r;
    return r;
}
std::mutex &tp_mu()
{
    static std::mutex m;
    return m;
}

template <int A, int B, int CC, int C1, int C2, int R3>
struct TpReg {
    TpReg()
    {
        constexpr int T1 = StockhamPlan<float, A, 16>::G * C1, T2 = StockhamPlan<float, B, 16>::G * C2,
                      T3 = StockhamPlan<float, CC, 16>::G * R3;
        ThreePass k;
        k.la = A;
        k.lb = B;
        k.lc = CC;
        k.c1 = C1;
        k.c2 = C2;
        k.r3 = R3;
        k.fwd[0] = (const void *)&k3_col<A, C1, Minb<T1>::value, false>;
        k.inv[0] = (const void *)&k3_col<A, C1, Minb<T1>::value, true>;
        k.fwd[1] = (const void *)&k3_col<B, C2, Minb<T2>::value, false>;
        k.inv[1] = (const void *)&k3_col<B, C2, Minb<T2>::value, true>;
        k.fwd[2] = (const void *)&k3_row<CC, R3, Minb<T3>::value, false>;
        k.inv[2] = (const void *)&k3_row<CC, R3, Minb<T3>::value, true>;
        k.threads[0] = T1;
        k.threads[1] = T2;
        k.threads[2] = T3;
        k.smem[0] = col_smem<A, C1>();
        k.smem[1] = col_smem<B, C2>();
        k.smem[2] = row_smem<CC, R3>();
        k.tw_count[0] = StockhamPlan<float, A, 16>::TW;
        k.tw_count[1] = StockhamPlan<float, B, 16>::TW;
        k.tw_count[2] = StockhamPlan<float, CC, 16>::TW;
        k.tw_fill[0] = &tp_fill<A>;
        k.tw_fill[1] = &tp_fill<B>;
        k.tw_fill[2] = &tp_fill<CC>;
        std::lock_guard<std::mutex> lk(tp_mu());
        tp_registry()[A + B + CC].push_back(k);
    }
};

// (a, b, c, pass-1 columns, pass-2 columns, pass-3 rows): tiles of 2048 -
// 4096 points, runs of 16 - 64 points.  The first layout of a length is
// the default, the others are selected by GFFT_3PASS_VARIANT.  Measured on
// GB300 (GB/s, 1 GB batches, forward + inverse; 2^19 and 2^20 run two
// passes by default, 2029 and 2136):
//   2^19  (6,6,7 | 64,64,16) 2085   (6,7,6 | 64,32,32) 1886, (5,7,7) 1652
//   2^20  (6,6,8 | 64,64,16) 2102   (7,6,7 | 32,64,16) 2065, (6,7,7) 2056
//   2^21  (7,7,7 | 32,32,16) 2118   (7,6,8 | 32,64,16) 2057
//   2^22  (7,7,8 | 32,32,16) 2095   (7,8,7 | 32,16,16) 2040, four other
//         shapes 1951-2044
//   2^23  (7,8,8 | 32,16,16) 2017   (8,7,8 | 16,32,16) 1978
TpReg<6, 6, 7, 64, 64, 16> tp19;
TpReg<6, 7, 6, 64, 32, 32> tp19_1;
TpReg<6, 6, 8, 64, 64, 16> tp20;
TpReg<7, 6, 7, 32, 64, 16> tp20_1;
TpReg<7, 7, 7, 32, 32, 16> tp21;
TpReg<7, 6, 8, 32, 64, 16> tp21_1;
TpReg<7, 7, 8, 32, 32, 16> tp22;
TpReg<7, 8, 7, 32, 16, 16> tp22_1;
TpReg<7, 8, 8, 32, 16, 16> tp23;
TpReg<8, 7, 8, 16, 32, 16> tp23_1;
TpReg<8, 8, 8, 16, 16, 16> tp24;

}  // namespace

const ThreePass *threepass_find(int dtype, int logn)
{
    if (dtype != GFFT_F32) return nullptr;
    static const int variant = [] {
        const char *v = std::getenv("GFFT_3PASS_VARIANT");
        return (v && *v) ? std::atoi(v) : 0;
    }();
    std::lock_guard<std::mutex> lk(tp_mu());
    auto it = tp_registry().find(logn);
    if (it == tp_registry().end() || it->second.empty()) return nullptr;
    return &it->second[variant >= 0 && variant < (int)it->second.size() ? variant : 0];
}

cudaError_t launch_threepass(const ThreePass &k, int inverse, const ThreePassArgs &a, cudaStream_t st)
{
    if (a.batch <= 0) return cudaSuccess;
    const long long A = 1LL << k.la, B = 1LL << k.lb, C = 1LL << k.lc, M = B * C, N = A * M;
    const void *const *fn = inverse ? k.inv : k.fwd;
    for (int p = 0; p < 3; p++) {
        const cudaError_t e = ensure_smem(fn[p], k.smem[p]);
        if (e != cudaSuccess) return e;
    }
    const unsigned nmask1 = (unsigned)(N - 1), nmask2 = (unsigned)(M - 1);
    // pass 1: A-point columns over the M columns of every transform
    {
        const void *in = a.in;
        void *out = a.ws;
        long long ld = M, idist = a.idist, odist = N, y0 = 0;
        const void *tw = a.tw[0], *lo = a.lo1, *hi = a.hi1;
        int bits = a.bits1;
        unsigned nmask = nmask1;
        void *args[] = {(void *)&in, (void *)&out, (void *)&ld, (void *)&idist, (void *)&odist, (void *)&y0,
                        (void *)&tw, (void *)&lo, (void *)&hi, (void *)&bits, (void *)&nmask};
        for (long long b0 = 0; b0 < a.batch; b0 += 65535) {
            y0 = b0;
            const cudaError_t e = launch_pdl(fn[0], dim3((unsigned)(M / k.c1), (unsigned)std::min(65535LL, a.batch - b0)),
                                             dim3(k.threads[0]), args, k.smem[0], st);
            if (e != cudaSuccess) return e;
        }
    }
    // pass 2: B-point columns over the C columns of every (transform, k1)
    // block of M points, in place in the workspace
    {
        const void *in = a.ws;
        void *out = a.ws;
        long long ld = C, idist = M, odist = M, y0 = 0;
        const void *tw = a.tw[1], *lo = a.lo2, *hi = a.hi2;
        int bits = a.bits2;
        unsigned nmask = nmask2;
        void *args[] = {(void *)&in, (void *)&out, (void *)&ld, (void *)&idist, (void *)&odist, (void *)&y0,
                        (void *)&tw, (void *)&lo, (void *)&hi, (void *)&bits, (void *)&nmask};
        const long long items = a.batch * A;
        for (long long b0 = 0; b0 < items; b0 += 65535) {
            y0 = b0;
            const cudaError_t e = launch_pdl(fn[1], dim3((unsigned)(C / k.c2), (unsigned)std::min(65535LL, items - b0)),
                                             dim3(k.threads[1]), args, k.smem[1], st);
            if (e != cudaSuccess) return e;
        }
    }
    // pass 3: C-point rows r = k1 + A k2, stored transposed
    for (long long b0 = 0; b0 < a.batch; b0 += 65535) {
        const void *in = static_cast<const c32 *>(a.ws) + b0 * N;
        void *out = static_cast<c32 *>(a.out) + b0 * a.odist;
        int la = k.la;
        long long lda = M, ldb = C, ostride = A * B, idist = N, odist = a.odist;
        const void *tw = a.tw[2];
        float scale = (float)a.scale;
        void *args[] = {(void *)&in,      (void *)&out,   (void *)&la,    (void *)&lda, (void *)&ldb,
                        (void *)&ostride, (void *)&idist, (void *)&odist, (void *)&tw,  (void *)&scale};
        const cudaError_t e = launch_pdl(fn[2], dim3((unsigned)(A * B / k.r3), (unsigned)std::min(65535LL, a.batch - b0)),
                                         dim3(k.threads[2]), args, k.smem[2], st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace gfft
