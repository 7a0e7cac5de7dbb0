// fourstep.cuh -- one persistent launch for a batch of four-step C2C
// transforms of N = A * B points (sizes above the single-CTA limit), with
// the intermediate array kept in a small ring of L2-resident slots.
//
// The reference transforms these sizes with its recursive radix-2 levels
// over a bit-reversed copy (fft.h:80-85, FFTUtil.h:51-83,
// fft_impl_generic.h:36-63), touching the whole array once per level.  Here
// every transform is two tile passes (see tiles.cuh for the split):
//   COL tile (t, j): CC columns of A points of transform t, read from HBM,
//                    FFT + W_N twiddle, written to ring slot t % S;
//   ROW tile (t, r): CR rows of B points of slot t % S, FFT, stored
//                    transposed to the output in HBM.
// Work items are claimed in a fixed order through one atomic counter:
// phase p holds the COL tiles of transform p followed by the ROW tiles of
// transform p - LAG.  A ROW tile waits (bounded) until every COL tile of its
// transform is done; a COL tile waits, before its stores, until every ROW
// tile of the slot's previous transform (t - S) has read it.  Both waits
// point at items with lower claim numbers (LAG < S), which are held by
// running CTAs, so the schedule cannot deadlock.  With S slots small enough
// to stay in L2, the intermediate never reaches HBM: the HBM traffic is one
// read of the input and one write of the output, the algorithmic bytes.
//
// Each CTA is warp-specialised.  One producer thread claims items, resolves
// the ROW dependencies and fills a ring of NS shared-memory stages with TMA
// copies (3D tensor boxes for COL tiles, one bulk copy per row for ROW
// tiles), running ahead of the compute warps.  The compute warps take the
// stages in order (full/empty mbarriers), synchronise among themselves
// with a named barrier, and never wait on the claim or on global counters
// except the rare COL slot-free check.  Every wait is bounded.
#pragma once

#include "dit.cuh"
#include "fourstep.h"
#include "tiles.cuh"
#include "tma.cuh"

namespace gfft {

template <int A_, int B_>
struct imax {
    static constexpr int value = A_ > B_ ? A_ : B_;
};
template <int A_, int B_>
struct imin {
    static constexpr int value = A_ < B_ ? A_ : B_;
};

template <typename T, int LA, int LB, int CC, int E_, int NS_>
struct FourStepCfg {
    using SPA = StockhamPlan<T, LA, E_>;
    using SPB = StockhamPlan<T, LB, E_>;
    static constexpr int NS = NS_;                 // shared-memory stages
    static constexpr int CT = SPA::G * CC;         // compute threads
    static constexpr int THREADS = CT + 32;        // + the producer warp
    static constexpr int CR = CT / SPB::G;         // rows per ROW tile
    static constexpr long long A = 1LL << LA, B = 1LL << LB, N = A * B;
    static constexpr int NC = (int)(B / CC), NR = (int)(A / CR);
    // real-input mode: row items pair CH = CR/2 rows with their mirrors
    // (A / CR pair items) plus one item for the self-paired row 0
    static constexpr int CH = CR / 2, NRP = (int)(A / CR) + 1;
    static constexpr int BOXR = A < 256 ? (int)A : 256;  // rows per tensor box
    // COL stage: A rows of CC landed by the tensor copies, then the padded
    // column-major exchange layout of tiles.cuh
    static constexpr int PITCH = tile_pitch<T>(SPA::N, CC);
    static constexpr int COL_ELEMS = imax<(int)(A * CC), (SPA::P > 1 ? PITCH * CC : 0)>::value;
    // ROW stage: CR rows of B landed back to back, then padded rows, then
    // the transpose of the store
    static constexpr int ROWP = SPB::P > 1 ? SPB::SMEM : 0;
    static constexpr int XPOSE = spad_size<T>(SPB::N * CR);
    static constexpr int ROW_ELEMS = imax<(int)(B * CR), imax<ROWP * CR, XPOSE>::value>::value;
    static constexpr int PER_LINE = 128 / (int)sizeof(cpx<T>);  // stages start on 128-byte lines
    static constexpr int STAGE = (imax<COL_ELEMS, ROW_ELEMS>::value + PER_LINE - 1) / PER_LINE * PER_LINE;
    // twiddle tables staged in shared memory once per CTA: the Stockham
    // tables of both tile lengths (one when equal) and the W_N split tables
    static constexpr int LO_BITS = (LA + LB + 1) / 2;
    static constexpr int TWA = SPA::TW, TWB = LA == LB ? 0 : SPB::TW;
    static constexpr int NLO = 1 << LO_BITS, NHI = (int)(N >> LO_BITS);
    static constexpr int TABLES = (TWA + TWB + NLO + NHI + PER_LINE - 1) / PER_LINE * PER_LINE;
    static constexpr size_t BAR_OFF = ((size_t)NS * STAGE + TABLES) * sizeof(cpx<T>);
    static constexpr size_t SMEM = BAR_OFF + 128;  // + barriers and item slots
    static constexpr int SMEM_BLOCKS = (int)((228 * 1024) / (SMEM + 1024));  // 1 KB reserved per CTA
    static constexpr int REG_BLOCKS = 65536 / (THREADS * 56);  // at least 56 registers a thread
    static constexpr int MIN_BLOCKS = imax<1, imin<SMEM_BLOCKS, REG_BLOCKS>::value>::value;
    static_assert(CR >= 1 && CR * SPB::G == CT, "row tile must use every compute thread");
    static_assert(B % CC == 0 && A % CR == 0 && A % BOXR == 0, "tiles must divide the array");
    static_assert(CT % 32 == 0, "compute threads are whole warps");
    static constexpr bool FITS = SMEM <= 227 * 1024;  // stages and tables fit one CTA
};

// named barrier over the compute warps (id 1; id 0 is __syncthreads)
__device__ __forceinline__ void bar_compute(int nthreads)
{
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}
// same, returning the AND of every compute thread's predicate
__device__ __forceinline__ bool bar_compute_and(int nthreads, bool pred)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.and.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(nthreads)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// make data another SM published through the generic proxy (and acquired
// here) visible to this thread's later TMA (async proxy) reads of global memory
__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// wait until *p >= target (bounded; false on timeout or abort)
__device__ __forceinline__ bool fs_wait_geq(const int *p, int target, const int *abort)
{
    const volatile int *v = p;
    if (*v >= target) return true;
    const unsigned long long t0 = global_ns();
    while (*v < target) {
        if (*(const volatile int *)abort) return false;
        if (global_ns() - t0 > TMA_WAIT_NS) return false;
        __nanosleep(64);
    }
    return true;
}

// DIT: the real-input transform (forward, half spectrum): the input is the
// n reals read as N = n/2 complex values, and the row items apply the DIT
// adjustment (dit.cuh) to bin pairs (k, N - k) before storing the N + 1
// bins.  Bin k = k1 + A k2 pairs with row A - k1, column B - 1 - k2 (row 0
// with itself, column B - k2), so a row item transforms CH rows and their
// mirrors together.
template <typename T, int LA, int LB, int CC, int E_, int NS_, bool INV, bool DIT = false>
__global__ void __launch_bounds__(FourStepCfg<T, LA, LB, CC, E_, NS_>::THREADS,
                                  FourStepCfg<T, LA, LB, CC, E_, NS_>::MIN_BLOCKS)
    k_fourstep(const __grid_constant__ CUtensorMap map, const FourStepArgs a)
{
    using Cfg = FourStepCfg<T, LA, LB, CC, E_, NS_>;
    using SPA = typename Cfg::SPA;
    using SPB = typename Cfg::SPB;
    constexpr int EA = SPA::E, GA = SPA::G, EB = SPB::E, GB = SPB::G;
    constexpr int CT = Cfg::CT, CR = Cfg::CR, NC = Cfg::NC, NS = Cfg::NS;
    constexpr int NR = DIT ? Cfg::NRP : Cfg::NR, CH = Cfg::CH;
    static_assert(!DIT || (CH >= 1 && !INV), "real-input mode: forward, at least two rows per item");
    static_assert(!DIT || (sizeof(T) == 4 && Cfg::ROWP >= SPB::N + SPB::N / 16), "real-input mode: padded fp32 rows");
    constexpr long long A = Cfg::A, B = Cfg::B, N = Cfg::N;
    constexpr int UNITS = (int)sizeof(cpx<T>) / 8;  // 8-byte tensor elements per complex value
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    cpx<T> *const stage0 = reinterpret_cast<cpx<T> *>(smem_raw);
    cpx<T> *const twa = stage0 + (size_t)NS * Cfg::STAGE;
    cpx<T> *const twb = LA == LB ? twa : twa + Cfg::TWA;
    cpx<T> *const tlo = twa + Cfg::TWA + Cfg::TWB;
    cpx<T> *const thi = tlo + Cfg::NLO;
    uint64_t *const full = reinterpret_cast<uint64_t *>(smem_raw + Cfg::BAR_OFF);
    uint64_t *const empty = full + NS;
    int *const item_of = reinterpret_cast<int *>(empty + NS);
    int *const s_flag = item_of + NS;

    int *const abort_flag = a.ctr + 1;
    int *const col_done = a.ctr + 2;
    int *const row_done = a.ctr + 2 + a.slots;
    const int per_phase = NC + NR;

    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        fence_barrier_init();
    }
    {
        // stage the twiddle tables (read by every tile this CTA runs)
        auto copy = [](cpx<T> *d, const void *src, int n) {
            const cpx<T> *g = static_cast<const cpx<T> *>(src);
            for (int i = threadIdx.x; i < n; i += Cfg::THREADS) d[i] = ldg_c(g + i);
        };
        copy(twa, a.tw_a, Cfg::TWA);
        if (LA != LB) copy(twb, a.tw_b, Cfg::TWB);
        copy(tlo, a.tw_lo, Cfg::NLO);
        copy(thi, a.tw_hi, Cfg::NHI);
    }
    __syncthreads();

    if (threadIdx.x >= CT) {
        // ================= producer (one thread)
        if (threadIdx.x != CT) return;
        int k = 0;
        bool failed = false;
        for (;;) {
            const int item = *(volatile int *)abort_flag ? a.nitems : atomicAdd(a.ctr, 1);
            const bool done = item >= a.nitems;
            int p = 0, j = 0;
            if (!done) {
                p = item / per_phase;
                j = item - p * per_phase;
                if (j < NC ? p >= a.batch : p < a.lag) continue;  // empty place of the schedule
            }
            const int st = k % NS;
            const uint32_t ph = (uint32_t)((k / NS) & 1);
            if (!mbar_wait(&empty[st], ph ^ 1u)) {
                failed = true;
                break;
            }
            if (done) {
                item_of[st] = -1;
                mbar_arrive(&full[st]);
                break;
            }
            cpx<T> *S = stage0 + (size_t)st * Cfg::STAGE;
            if (j < NC) {
                const long long col0 = (long long)j * CC;
                item_of[st] = item;
                mbar_arrive_expect_tx(&full[st], (uint32_t)(A * CC * sizeof(cpx<T>)));
#pragma unroll 1
                for (int r = 0; r < (int)A; r += Cfg::BOXR)
                    tensor_load_3d(S + (size_t)r * CC, &map, (int)(col0 * UNITS), r, p, &full[st]);
            } else {
                const long long t = p - a.lag;
                const int slot = (int)(t % a.slots), use = (int)(t / a.slots);
                if (!fs_wait_geq(col_done + slot, (use + 1) * NC, abort_flag)) {
                    item_of[st] = -1;  // the stage is ours: tell the compute warps to stop
                    mbar_arrive(&full[st]);
                    failed = true;
                    break;
                }
                __threadfence();
                fence_proxy_async_global();
                const cpx<T> *slot_base = static_cast<const cpx<T> *>(a.ws) + (long long)slot * N;
                item_of[st] = item;
                if (DIT) {
                    const int r = j - NC;
                    if (r < NR - 1) {
                        // rows 1 + CH r .. + CH - 1, then their mirrors A - CH r - CH .. A - CH r - 1
                        mbar_arrive_expect_tx(&full[st], (uint32_t)(2 * CH * B * sizeof(cpx<T>)));
                        bulk_load(S, slot_base + (1 + (long long)CH * r) * B, (uint32_t)(CH * B * sizeof(cpx<T>)),
                                  &full[st]);
                        bulk_load(S + (size_t)CH * B, slot_base + (A - (long long)CH * r - CH) * B,
                                  (uint32_t)(CH * B * sizeof(cpx<T>)), &full[st]);
                    } else {  // row 0
                        mbar_arrive_expect_tx(&full[st], (uint32_t)(B * sizeof(cpx<T>)));
                        bulk_load(S, slot_base, (uint32_t)(B * sizeof(cpx<T>)), &full[st]);
                    }
                } else {
                    const long long row0 = (long long)(j - NC) * CR;
                    const cpx<T> *src = slot_base + row0 * B;
                    mbar_arrive_expect_tx(&full[st], (uint32_t)(CR * B * sizeof(cpx<T>)));
#pragma unroll 1
                    for (int s = 0; s < CR; s++)
                        bulk_load(S + (size_t)s * B, src + (long long)s * B, (uint32_t)(B * sizeof(cpx<T>)),
                                  &full[st]);
                }
            }
            k++;
        }
        if (failed) {
            atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
            atomicExch(abort_flag, 1);
            // let this CTA's copies in flight land before it exits
            for (int i = k - NS < 0 ? 0 : k - NS; i < k; i++) mbar_wait(&full[i % NS], (uint32_t)((i / NS) & 1));
        }
        return;
    }

    // ===================== compute warps
    const int tid = threadIdx.x;
    for (int k = 0;; k++) {
        const int st = k % NS;
        const uint32_t ph = (uint32_t)((k / NS) & 1);
        if (!bar_compute_and(CT, mbar_wait(&full[st], ph))) {
            if (tid == 0) {
                atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                atomicExch(abort_flag, 1);
            }
            break;
        }
        const int item = item_of[st];
        if (item < 0) break;
        const int p = item / per_phase;
        const int j = item - p * per_phase;
        cpx<T> *S = stage0 + (size_t)st * Cfg::STAGE;
        if (j < NC) {
            // ---------------- COL tile j of transform p
            const long long t = p;
            const int slot = (int)(t % a.slots), use = (int)(t / a.slots);
            const int s = tid % CC, tt = tid / CC;
            const long long col = (long long)j * CC + s;
            cpx<T> v[EA];
#pragma unroll
            for (int q = 0; q < EA; q++) v[q] = S[(tt + q * GA) * CC + s];
            bar_compute(CT);
            cpx<T> *my = S + s * Cfg::PITCH;
            stockham_run<T, LA, E_, INV, TwShared>(
                v, tt, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, twa, []() { bar_compute(CT); });
            // the slot is free once every ROW tile of transform t - S read it
            if (use > 0) {
                if (tid == 0) {
                    *s_flag = fs_wait_geq(row_done + slot, use * NR, abort_flag);
                    __threadfence();
                }
                bar_compute(CT);
                if (!*s_flag) {
                    if (tid == 0) {
                        atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                        atomicExch(abort_flag, 1);
                    }
                    break;
                }
            }
            constexpr unsigned lo_mask = (1u << Cfg::LO_BITS) - 1u;
            cpx<T> *dst = static_cast<cpx<T> *>(a.ws) + (long long)slot * N + col + (long long)tt * B;
            const unsigned ecol = (unsigned)col;
#pragma unroll
            for (int q = 0; q < EA; q++) {
                const unsigned e = (ecol * (unsigned)(tt + q * GA)) & (unsigned)(N - 1);
                const cpx<T> w = cmul(thi[e >> Cfg::LO_BITS], tlo[e & lo_mask]);
                st_c(dst + (long long)q * GA * B, twmul<INV>(v[q], w));
                if ((q & 3) == 3) asm volatile("" ::: "memory");
            }
            // publish: the barrier orders every compute thread's stores
            // before thread 0's release of the count
            bar_compute(CT);
            if (tid == 0) {
                __threadfence();
                atomicAdd(col_done + slot, 1);
                mbar_arrive(&empty[st]);
            }
        } else {
            // ---------------- ROW tile r of transform p - LAG
            const long long t = p - a.lag;
            const int slot = (int)(t % a.slots);
            const int s = tid / GB, tt = tid - s * GB;
            if constexpr (DIT) {
                // ---- real-input row item: CH rows and their mirrors (or row 0)
                const int r = j - NC;
                const bool row0 = r == NR - 1;
                const cpx<T> *slot_base = static_cast<const cpx<T> *>(a.ws) + (long long)slot * N;
                {
                    // drop the copied rows' L2 lines without a write-back
                    auto drop = [tid](const cpx<T> *base, long long elems) {
                        const char *c = reinterpret_cast<const char *>(base);
                        const int lines = (int)(elems * (long long)sizeof(cpx<T>) / 128);
                        for (int i = tid; i < lines; i += CT)
                            asm volatile("discard.global.L2 [%0], 128;" ::"l"(c + (size_t)i * 128) : "memory");
                    };
                    if (row0) {
                        drop(slot_base, B);
                    } else {
                        drop(slot_base + (1 + (long long)CH * r) * B, (long long)CH * B);
                        drop(slot_base + (A - (long long)CH * r - CH) * B, (long long)CH * B);
                    }
                }
                cpx<T> v[EB];
#pragma unroll
                for (int q = 0; q < EB; q++) v[q] = S[s * B + tt + q * GB];
                bar_compute(CT);
                if (tid == 0) {
                    __threadfence();
                    atomicAdd(row_done + slot, 1);
                }
                cpx<T> *my = S + s * Cfg::ROWP;
                stockham_run<T, LB, E_, false, TwShared>(
                    v, tt, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, twb, []() { bar_compute(CT); });
                bar_compute(CT);
                // Z tile: slot s, column k2 rotated by s * ZROT (so that the
                // CH slots a warp reads at once fall on different banks), then
                // padded like the exchange
                constexpr int ZROT = CH >= 2 ? 32 / CH : 0;
                auto zpos = [](int slot_, int k2) {
                    const int c = (k2 + slot_ * ZROT) & ((int)B - 1);
                    return slot_ * Cfg::ROWP + c + (c >> 4);
                };
#pragma unroll
                for (int q = 0; q < EB; q++) S[zpos(s, tt + q * GB)] = v[q];
                bar_compute(CT);
                auto Z = [S, zpos](int slot_, int k2) { return S[zpos(slot_, k2)]; };
                cpx<T> *dst = static_cast<cpx<T> *>(a.out) + t * a.odist;
                const cpx<T> *dtw = static_cast<const cpx<T> *>(a.dtw);
                const T scale = (T)a.scale;
                if (!row0) {
                    // lo slot s2 (row 1 + CH r + s2) pairs with hi slot
                    // 2 CH - 1 - s2 (row A - 1 - CH r - s2), column B - 1 - k2;
                    // consecutive threads take consecutive rows: runs of CH bins
                    for (int idx = tid; idx < CH * (int)B; idx += CT) {
                        const int s2 = idx % CH, k2 = idx / CH;
                        const long long k = 1 + (long long)CH * r + s2 + A * k2, jj = N - k;
                        const cpx<T> zk = Z(s2, k2), zj = Z(2 * CH - 1 - s2, (int)B - 1 - k2);
                        stcs_c(dst + k, scl(dit_value(zk, zj, ldg_c(dtw + k)), scale));
                        stcs_c(dst + jj, scl(dit_value(zj, zk, ldg_c(dtw + jj)), scale));
                    }
                } else {
                    // row 0: bins A k2 and A (B - k2), k2 = 0 .. B/2 (k2 = 0 also
                    // gives the Nyquist bin N)
                    for (int k2 = tid; k2 <= (int)B / 2; k2 += CT) {
                        const long long k = A * k2, jj = N - k;
                        const cpx<T> zk = Z(0, k2), zj = Z(0, ((int)B - k2) & ((int)B - 1));
                        stcs_c(dst + k, scl(dit_value(zk, zj, ldg_c(dtw + k)), scale));
                        stcs_c(dst + jj, scl(dit_value(zj, zk, ldg_c(dtw + jj)), scale));
                    }
                }
                bar_compute(CT);
                if (tid == 0) mbar_arrive(&empty[st]);
                continue;
            }
            const long long row0 = (long long)(j - NC) * CR;
            // the rows are in shared memory: drop their L2 lines without a
            // write-back (the slot is rewritten before it is read again),
            // then release this tile's share of the slot
            {
                const char *base =
                    reinterpret_cast<const char *>(static_cast<const cpx<T> *>(a.ws) + (long long)slot * N + row0 * B);
                constexpr int LINES = (int)(CR * B * sizeof(cpx<T>) / 128);
                for (int i = tid; i < LINES; i += CT)
                    asm volatile("discard.global.L2 [%0], 128;" ::"l"(base + (size_t)i * 128) : "memory");
            }
            cpx<T> v[EB];
#pragma unroll
            for (int q = 0; q < EB; q++) v[q] = S[s * B + tt + q * GB];
            bar_compute(CT);
            if (tid == 0) {
                __threadfence();
                atomicAdd(row_done + slot, 1);
            }
            cpx<T> *my = S + s * Cfg::ROWP;
            stockham_run<T, LB, E_, INV, TwShared>(
                v, tt, [my](int i) -> cpx<T> & { return my[spad<T>(i)]; }, twb, []() { bar_compute(CT); });
            bar_compute(CT);
#pragma unroll
            for (int q = 0; q < EB; q++) S[spad<T>((tt + q * GB) * CR + s)] = v[q];
            bar_compute(CT);
            cpx<T> *dst = static_cast<cpx<T> *>(a.out) + t * a.odist + row0;
            const T scale = (T)a.scale;
#pragma unroll
            for (int m = 0; m < EB; m++) {
                const int idx = tid + m * CT;
                const int s2 = idx % CR;
                const int kk = idx / CR;
                stcs_c(dst + s2 + (long long)kk * A, scl(S[spad<T>(idx)], scale));
            }
            bar_compute(CT);
            if (tid == 0) mbar_arrive(&empty[st]);
        }
    }
}

}  // namespace gfft
