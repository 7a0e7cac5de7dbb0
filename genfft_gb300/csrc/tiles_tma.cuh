// tiles_tma.cuh -- persistent, TMA-pipelined versions of the tile kernels.
//
// One CTA per SM walks the tiles of a launch.  Each CTA owns two shared
// stage buffers: while it transforms the tile in one buffer, the TMA engine
// fills the other with the next tile, so HBM stays busy through the
// compute phase (the plain tile kernels load, compute and store in turn and
// leave HBM idle in between).  Tiles too wide for two buffers get one
// (NSTG = 1): the next tile's copy starts as soon as this tile's last
// shared-memory read is done, and overlaps the rest of its work.
//   row pass    : the C rows of a tile are C contiguous bulk copies
//                 (cp.async.bulk, one per row);
//   column pass : the C x L tile is L/BOXR boxes of a 3D tensor map
//                 (cp.async.bulk.tensor), ncols x rows x batch.
// The arithmetic is the Stockham engine of the plain kernels, with the same
// twiddle tables, so results are identical.
#pragma once

#include "tiles.cuh"
#include "tma.cuh"

namespace gfft {

template <int A, int B>
struct cmax {
    static constexpr int value = A > B ? A : B;
};

// elements of one stage buffer, rounded to 128 bytes
template <typename T, int ELEMS>
struct StageRound {
    static constexpr int per = 128 / (int)sizeof(cpx<T>);
    static constexpr int value = (ELEMS + per - 1) / per * per;
};

// ---------------------------------------------------------------------------
// row pass: C rows of L points, stored transposed (see k_rowpass)

// NSTG as for the column pass below (1: the next tile's copies start once
// the transposed tile has been read back into registers, before the stores)
template <typename T, int LOGL, int C, int E_, int NSTG = 2>
struct RowTmaCfg {
    using SP = StockhamPlan<T, LOGL, E_>;
    static constexpr int N = SP::N;
    static constexpr int THREADS = SP::G * C;
    static constexpr int ROW = (SP::P > 1) ? SP::SMEM : 0;
    static constexpr int XPOSE = spad_size<T>(N * C);
    static constexpr int STAGE =
        StageRound<T, cmax<cmax<ROW * C, XPOSE>::value, N * C>::value>::value;  // elements
    static constexpr size_t SMEM = NSTG * (size_t)STAGE * sizeof(cpx<T>) + 64;
};

template <typename T, int LOGL, int C, int E_, bool INV, int NSTG = 2>
__global__ void __launch_bounds__(RowTmaCfg<T, LOGL, C, E_, NSTG>::THREADS, 1)
    k_rowpass_tma(const cpx<T> *__restrict__ in, cpx<T> *__restrict__ out, long long nrows, long long ld_in,
                  long long ostride, long long idist, long long odist, long long nbatch,
                  const cpx<T> *__restrict__ tw, unsigned *err, T scale)
{
    static_assert(NSTG == 1 || NSTG == 2, "one or two stages");
    using Cfg = RowTmaCfg<T, LOGL, C, E_, NSTG>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G, N = SP::N;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    cpx<T> *const stage0 = reinterpret_cast<cpx<T> *>(smem_raw);
    uint64_t *const bars = reinterpret_cast<uint64_t *>(smem_raw + NSTG * (size_t)Cfg::STAGE * sizeof(cpx<T>));

    const int s = threadIdx.x / G;
    const int t = threadIdx.x - s * G;
    const long long tiles = (nrows + C - 1) / C;
    const long long total = tiles * nbatch;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel

    if (threadIdx.x == 0) {
        for (int i = 0; i < NSTG; i++) mbar_init(&bars[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](long long w, int buf) {  // thread 0: load tile w into buffer buf
        const long long b = w / tiles, row0 = (w - b * tiles) * C;
        const int rows = (int)((nrows - row0) < C ? (nrows - row0) : C);
        cpx<T> *dst = stage0 + buf * Cfg::STAGE;
        mbar_arrive_expect_tx(&bars[buf], (uint32_t)(rows * N * sizeof(cpx<T>)));
        const cpx<T> *src = in + b * idist + row0 * ld_in;
        for (int r = 0; r < rows; r++) bulk_load(dst + r * N, src + r * ld_in, N * sizeof(cpx<T>), &bars[buf]);
    };

    long long w = blockIdx.x;
    if (threadIdx.x == 0 && w < total) issue(w, 0);
    for (int k = 0; w < total; w += gridDim.x, k++) {
        const int cur = NSTG == 2 ? (k & 1) : 0;
        const uint32_t par = (uint32_t)(NSTG == 2 ? ((k >> 1) & 1) : (k & 1));
        const bool ok = mbar_wait(&bars[cur], par);
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) {
                atomicOr(err, DEV_ERR_TMA_TIMEOUT);
                mbar_wait(&bars[cur], par);  // let this CTA's copy land before exit
            }
            return;
        }
        // the other buffer is free (every thread finished the previous tile)
        if (NSTG == 2 && threadIdx.x == 0 && w + gridDim.x < total) {
            fence_proxy_async_smem();
            issue(w + gridDim.x, cur ^ 1);
        }
        cpx<T> *S = stage0 + cur * Cfg::STAGE;
        const long long b = w / tiles, row0 = (w - b * tiles) * C;
        const bool active = row0 + s < nrows;
        cpx<T> v[E];
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = active ? S[s * N + t + q * G] : cpx<T>{(T)0, (T)0};
        __syncthreads();
        cpx<T> *my = S + s * Cfg::ROW;
        stockham_run<T, LOGL, E_, INV>(
            v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
        __syncthreads();
#pragma unroll
        for (int q = 0; q < E; q++) S[spad<T>((t + q * G) * C + s)] = v[q];
        __syncthreads();
        cpx<T> *dst = out + b * odist + row0;
        if constexpr (NSTG == 1) {
            // read the transposed tile back, free the buffer for the next
            // tile's copies, then store
            cpx<T> o[E];
#pragma unroll
            for (int m = 0; m < E; m++) o[m] = S[spad<T>(threadIdx.x + m * Cfg::THREADS)];
            __syncthreads();
            if (threadIdx.x == 0 && w + gridDim.x < total) {
                fence_proxy_async_smem();
                issue(w + gridDim.x, 0);
            }
#pragma unroll
            for (int m = 0; m < E; m++) {
                const int idx = threadIdx.x + m * Cfg::THREADS;
                const int s2 = idx % C;
                const int kk = idx / C;
                if (kk < N && row0 + s2 < nrows) stcs_c(dst + s2 + (long long)kk * ostride, scl(o[m], scale));
            }
        } else {
#pragma unroll
            for (int m = 0; m < E; m++) {
                const int idx = threadIdx.x + m * Cfg::THREADS;
                const int s2 = idx % C;
                const int kk = idx / C;
                if (kk < N && row0 + s2 < nrows)
                    stcs_c(dst + s2 + (long long)kk * ostride, scl(S[spad<T>(idx)], scale));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// column pass: C columns of L points (see k_colpass); the tensor map views
// the input as [batch][rows][ncols] elements of `unit` bytes (8 for fp32
// complex; fp64 complex is two 8-byte units)

// NSTG = 2: double-buffered (the next tile lands while this one is
// transformed).  NSTG = 1, for tiles whose two buffers do not fit: the
// next tile's copy starts once every thread has read its last exchange
// values, so it overlaps the twiddle and the stores of this tile, and the
// loads cost no load instructions either way.
template <typename T, int LOGL, int C, int E_, int NSTG = 2>
struct ColTmaCfg {
    using SP = StockhamPlan<T, LOGL, E_>;
    static constexpr int N = SP::N;
    static constexpr int THREADS = SP::G * C;
    static constexpr int PITCH = tile_pitch<T>(N, C);
    static constexpr int BOXR = N < 256 ? N : 256;  // rows per tensor box
    static constexpr int STAGE = StageRound<T, cmax<PITCH * C, N * C>::value>::value;
    static constexpr size_t SMEM = NSTG * (size_t)STAGE * sizeof(cpx<T>) + 64;
};

template <typename T, int LOGL, int C, int E_, bool INV, int TWM, bool HERM, int NSTG = 2>
__global__ void __launch_bounds__(ColTmaCfg<T, LOGL, C, E_, NSTG>::THREADS, 1)
    k_colpass_tma(const __grid_constant__ CUtensorMap map, cpx<T> *__restrict__ out, long long ncols,
                  long long ld_out, long long odist, long long nbatch, const cpx<T> *__restrict__ tw,
                  const cpx<T> *__restrict__ tw_lo, const cpx<T> *__restrict__ tw_hi, int lo_bits, unsigned nmask,
                  unsigned *err, T scale)
{
    static_assert(NSTG == 1 || NSTG == 2, "one or two stages");
    using Cfg = ColTmaCfg<T, LOGL, C, E_, NSTG>;
    using SP = typename Cfg::SP;
    constexpr int E = SP::E, G = SP::G, N = SP::N;
    constexpr int UNITS = sizeof(cpx<T>) / 8;  // 8-byte tensor elements per complex value
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    cpx<T> *const stage0 = reinterpret_cast<cpx<T> *>(smem_raw);
    uint64_t *const bars = reinterpret_cast<uint64_t *>(smem_raw + NSTG * (size_t)Cfg::STAGE * sizeof(cpx<T>));

    const int s = threadIdx.x % C;
    const int t = threadIdx.x / C;
    const long long tiles = (ncols + C - 1) / C;
    const long long total = tiles * nbatch;
    const unsigned lo_mask = (1u << lo_bits) - 1u;
    pdl_enter();  // launched by launch_pdl: waits for the previous kernel

    if (threadIdx.x == 0) {
        for (int i = 0; i < NSTG; i++) mbar_init(&bars[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](long long w, int buf) {  // thread 0: load tile w into buffer buf
        const long long b = w / tiles, col0 = (w - b * tiles) * C;
        cpx<T> *dst = stage0 + buf * Cfg::STAGE;
        // out-of-range columns of the last tile are zero-filled and still counted
        mbar_arrive_expect_tx(&bars[buf], (uint32_t)(N * C * sizeof(cpx<T>)));
        for (int r = 0; r < N; r += Cfg::BOXR)
            tensor_load_3d(dst + r * C, &map, (int)(col0 * UNITS), r, (int)b, &bars[buf]);
    };

    long long w = blockIdx.x;
    if (threadIdx.x == 0 && w < total) issue(w, 0);
    for (int k = 0; w < total; w += gridDim.x, k++) {
        const int cur = NSTG == 2 ? (k & 1) : 0;
        const uint32_t par = (uint32_t)(NSTG == 2 ? ((k >> 1) & 1) : (k & 1));
        const bool ok = mbar_wait(&bars[cur], par);
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) {
                atomicOr(err, DEV_ERR_TMA_TIMEOUT);
                mbar_wait(&bars[cur], par);
            }
            return;
        }
        if (NSTG == 2 && threadIdx.x == 0 && w + gridDim.x < total) {
            fence_proxy_async_smem();
            issue(w + gridDim.x, cur ^ 1);
        }
        cpx<T> *S = stage0 + cur * Cfg::STAGE;
        const long long b = w / tiles, col = (w - b * tiles) * C + s;
        cpx<T> v[E];
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = S[(t + q * G) * C + s];
        __syncthreads();
        cpx<T> *my = S + s * Cfg::PITCH;
        stockham_run<T, LOGL, E_, INV>(
            v, t, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, tw, []() { __syncthreads(); });
        if constexpr (NSTG == 1) {
            // every thread has read its last exchange values: the buffer
            // takes the next tile while this one is twiddled and stored
            __syncthreads();
            if (threadIdx.x == 0 && w + gridDim.x < total) {
                fence_proxy_async_smem();
                issue(w + gridDim.x, 0);
            }
        }
        if (col < ncols) {
            cpx<T> *dst = out + b * odist + col + (long long)t * ld_out;
            const long long step = (long long)G * ld_out;
            const unsigned ecol = TWM == 2 ? (unsigned)b : (unsigned)col;
#pragma unroll
            for (int q = 0; q < E; q++, dst += step) {
                cpx<T> val = v[q];
                if constexpr (TWM != 0) {
                    const unsigned e = (ecol * (unsigned)(t + q * G)) & nmask;
                    const cpx<T> wv = cmul(ldg_c(tw_hi + (e >> lo_bits)), ldg_c(tw_lo + (e & lo_mask)));
                    val = twmul<INV>(val, wv);
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
                        st_c(mir + (long long)((N - i) & (N - 1)) * ld_out, scl(conj(v[q]), scale));
                    }
                }
            }
        }
    }
}

}  // namespace gfft
