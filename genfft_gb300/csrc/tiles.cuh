// tiles.cuh -- tile kernels built on the Stockham engine: a CTA transforms
// C independent sub-transforms of L = 2^LOGL points that are strided in
// global memory.  They are the passes of the multi-pass (four-step) C2C for
// sizes above the shared-memory limit, the column pass of the 2D transforms
// and the column transform (FFTVert, fft.h:115-171).
//
// Four-step split of N = A * B (n = B a + b, k = k1 + A k2):
//   X[k1 + A k2] = sum_b W_B^(b k2) * ( W_N^(b k1) * sum_a x[B a + b] W_A^(a k1) )
//   column pass : for every column b, an A-point FFT down x[B a + b], times
//                 W_N^(b k1), stored back at Y[B k1 + b]         (k_colpass)
//   row pass    : for every row k1, a B-point FFT along Y[B k1 + b], stored
//                 transposed at X[k1 + A k2]                      (k_rowpass)
#pragma once

#include "stockham.cuh"

namespace gfft {

// Column-major tile layout: column s occupies PITCH slots starting at
// s*PITCH and is addressed like a fused transform (spad).  PITCH is chosen
// so that the C columns a half-warp (fp32) or quarter-warp (fp64) touches
// start in different banks: PITCH = 16/C (mod 16) slots of 8 B for fp32,
// 8/C (mod 8) slots of 16 B for fp64.
template <typename T>
__host__ __device__ constexpr int tile_pitch(int n, int c)
{
    const int base = spad_size<T>(n);
    const int per = sizeof(T) == 4 ? 16 : 8;
    const int want = (per / (c < per ? c : per)) % per;
    return base + ((want - base % per) % per + per) % per;
}

template <typename T, int LOGL, int C, int E_>
struct ColCfg {
    using SP = StockhamPlan<T, LOGL, E_>;
    static constexpr int THREADS = SP::G * C;
    static constexpr int PITCH = tile_pitch<T>(SP::N, C);
    static constexpr int SMEM_ELEMS = (SP::P > 1) ? PITCH * C : 0;
    static constexpr size_t SMEM = (size_t)SMEM_ELEMS * sizeof(cpx<T>);
};

// Column pass.  Column s of the tile (global column col = blockIdx.x*C + s)
// of batch item b = blockIdx.y holds element i at
//     in [b*idist + row(i)*ld_in + col]       row(i) = BITREV ? bitrev(i) : i
// and its transform goes to out[b*odist + i*ld_out + col], multiplied by
// W_N^(f*i) when TWM != 0 (a four-step inter-pass twiddle, from the split
// tables tw_hi[e >> lo_bits] * tw_lo[e & lo_mask], e = f*i mod N) with
// f = col (TWM 1: the columns are the second factor) or f = b (TWM 2: the
// batch index is; one launch covers fewer than 65536 batch items).
// HERM (real 2D output, RealFFT2D::forward, FFTReal.h:90-103): the tile runs
// over the W/2+1 non-redundant columns (ncols = W/2+1) and also stores the
// Hermitian mirror X[(L-i) mod L][W-col] = conj X[i][col] for 0 < col < W/2.
// Threads are numbered t*C + s, so a warp touches C consecutive columns of
// a row and global accesses come in C-element runs.
template <typename T, int LOGL, int C, int E_, bool INV, int TWM, bool BITREV, bool HERM = false>
__global__ void __launch_bounds__(ColCfg<T, LOGL, C, E_>::THREADS)
    k_colpass(const cpx<T> *__restrict__ in, cpx<T> *__restrict__ out, long long ncols, long long ld_in,
              long long ld_out, long long idist, long long odist,
              const cpx<T> *__restrict__ tw, const cpx<T> *__restrict__ tw_lo,
              const cpx<T> *__restrict__ tw_hi, int lo_bits, unsigned nmask, T scale)
{
    using Cfg = ColCfg<T, LOGL, C, E_>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G;
    extern __shared__ unsigned char smem_raw[];
    cpx<T> *sm = reinterpret_cast<cpx<T> *>(smem_raw);

    const int s = threadIdx.x % C;
    const int t = threadIdx.x / C;
    const long long col = (long long)blockIdx.x * C + s;
    const bool active = col < ncols;
    const unsigned lo_mask = (1u << lo_bits) - 1u;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel

    {
        const long long b = blockIdx.y;
        cpx<T> v[E];
        if (active) {
            if constexpr (BITREV) {
                const cpx<T> *src = in + b * idist + col;
#pragma unroll
                for (int q = 0; q < E; q++) v[q] = ldcs_c(src + (long long)bitrev(t + q * G, LOGL) * ld_in);
            } else {
                const cpx<T> *src = in + b * idist + col + (long long)t * ld_in;
                const long long step = (long long)G * ld_in;
#pragma unroll
                for (int q = 0; q < E; q++, src += step) v[q] = ldcs_c(src);
            }
        } else {
#pragma unroll
            for (int q = 0; q < E; q++) v[q] = cpx<T>{(T)0, (T)0};
        }
        cpx<T> *my = sm + s * Cfg::PITCH;
        stockham_run<T, LOGL, E_, INV>(
            v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
        if (active) {
            cpx<T> *dst = out + b * odist + col + (long long)t * ld_out;
            const long long step = (long long)G * ld_out;
            const unsigned ecol = TWM == 2 ? (unsigned)b : (unsigned)col;
#pragma unroll
            for (int q = 0; q < E; q++, dst += step) {
                cpx<T> val = v[q];
                if constexpr (TWM != 0) {
                    const unsigned e = (ecol * (unsigned)(t + q * G)) & nmask;
                    const cpx<T> w = cmul(ldg_c(tw_hi + (e >> lo_bits)), ldg_c(tw_lo + (e & lo_mask)));
                    val = twmul<INV>(val, w);
                    // keep the twiddle loads of later points from being hoisted
                    // (each hoisted pair costs four live registers)
                    if ((q & 3) == 3) asm volatile("" ::: "memory");
                }
                st_c(dst, scl(val, scale));
            }
            if constexpr (HERM) {
                const long long W = 2 * (ncols - 1);
                if (col > 0 && 2 * col < W) {
                    cpx<T> *mir = out + b * odist + (W - col);
#pragma unroll
                    for (int q = 0; q < E; q++) {
                        const int i = t + q * G;
                        st_c(mir + (long long)((SP::N - i) & (SP::N - 1)) * ld_out, scl(conj(v[q]), scale));
                    }
                }
            }
        }
    }
}

template <typename T, int LOGL, int C, int E_>
struct RowCfg {
    using SP = StockhamPlan<T, LOGL, E_>;
    static constexpr int THREADS = SP::G * C;
    static constexpr int ROW = (SP::P > 1) ? SP::SMEM : 0;
    static constexpr int XPOSE = spad_size<T>(SP::N * C);
    static constexpr int SMEM_ELEMS = (ROW * C > XPOSE) ? ROW * C : XPOSE;
    static constexpr size_t SMEM = (size_t)SMEM_ELEMS * sizeof(cpx<T>);
};

// Row pass with transposed store.  Row s of the tile (global row
// row = blockIdx.x*C + s) of item b = blockIdx.y holds element i at
//     in[b*idist + row*ld_in + i]
// and output element k goes to out[b*odist + row + k*ostride].  Loads are
// contiguous along each row; the result is transposed through shared memory
// so the store writes C-element runs.
template <typename T, int LOGL, int C, int E_, bool INV>
__global__ void __launch_bounds__(RowCfg<T, LOGL, C, E_>::THREADS)
    k_rowpass(const cpx<T> *__restrict__ in, cpx<T> *__restrict__ out, long long nrows, long long ld_in,
              long long ostride, long long idist, long long odist,
              const cpx<T> *__restrict__ tw, T scale)
{
    using Cfg = RowCfg<T, LOGL, C, E_>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G, N = SP::N;
    extern __shared__ unsigned char smem_raw[];
    cpx<T> *sm = reinterpret_cast<cpx<T> *>(smem_raw);

    const int s = threadIdx.x / G;
    const int t = threadIdx.x - s * G;
    const long long row0 = (long long)blockIdx.x * C;
    const long long row = row0 + s;
    const bool active = row < nrows;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel

    {
        const long long b = blockIdx.y;
        cpx<T> v[E];
        const cpx<T> *src = in + b * idist + row * ld_in + t;
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = active ? ld_c(src + q * G) : cpx<T>{(T)0, (T)0};
        cpx<T> *my = sm + s * Cfg::ROW;
        stockham_run<T, LOGL, E_, INV>(
            v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
        __syncthreads();
#pragma unroll
        for (int q = 0; q < E; q++) sm[spad<T>((t + q * G) * C + s)] = v[q];
        __syncthreads();
        cpx<T> *dst = out + b * odist + row0;
#pragma unroll
        for (int m = 0; m < E; m++) {
            const int idx = threadIdx.x + m * Cfg::THREADS;
            const int s2 = idx % C;
            const int k = idx / C;
            if (k < N && row0 + s2 < nrows) stcs_c(dst + s2 + (long long)k * ostride, scl(sm[spad<T>(idx)], scale));
        }
    }
}

}  // namespace gfft
