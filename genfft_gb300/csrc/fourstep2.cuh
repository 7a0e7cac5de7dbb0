// fourstep2.cuh -- the persistent four-step C2C (fourstep.cuh) with two
// sub-transforms per thread on packed FP32 instructions (pair.cuh), for
// fp32 n = A * B with A, B = 2^8 .. 2^12.  Opt-in (GFFT_FS_PAIR=1):
// measured on GB300 it is slower than the default paths except at 2^18.
//
// Same split, schedule and intermediate ring as k_fourstep: COL items (CC
// columns of A points of transform p: HBM -> FFT -> W_N twiddle -> ring
// slot) and ROW items (CR rows of B points of a slot -> FFT -> transposed
// store to HBM), claimed in a fixed order through one counter, with bounded
// waits on the COL -> ROW and slot-reuse dependencies; the ring stays in
// L2, so HBM sees one read of the input and one write of the output.
//
// What changes is the tile work, which bounds k_fourstep at these sizes:
//   * each thread holds E pair points: two adjacent columns of a COL item,
//     two adjacent rows of a ROW item, so the butterflies, rotations and
//     twiddle products of two transforms issue as one packed instruction;
//   * each pair of sub-transforms exchanges through its own padded buffer,
//     separate from the stage, under its own barrier (__syncwarp where the
//     pair is one warp's), so a warp hands the stage back to the producer
//     as soon as it has read its points and the next item's copy overlaps
//     the whole transform of this one;
//   * both epilogues go through shared memory so that every store writes
//     whole 32-byte sectors: a COL item writes CC * 8 contiguous bytes of
//     each ring row, a ROW item CR * 8 contiguous bytes of each output run
//     (k = k1 + A k2 with its CR rows k1 neighbours);
//   * the compute warps never fence: a publisher warp takes each finished
//     item (mbarrier hand-off, release / acquire within the CTA), makes it
//     visible to the GPU and counts it, so the item's stores drain while
//     the compute warps start the next one;
//   * L2 policies keep the ring resident: the input's tensor copies are
//     evict-first, the ring's stores evict-last;
//   * variants of 8 pair points a thread and up to about 113 KB of shared
//     memory run two CTAs an SM.
// Accounting: col_done[slot] and row_done[slot] count COL and ROW items, as
// in k_fourstep; a ROW item is counted once its rows are in shared memory
// (and their L2 lines dropped), a COL item once its stores are visible.
#pragma once

#include "fourstep.cuh"
#include "pair.cuh"

namespace gfft {

template <int LA, int LB, int E_, int CT_, int NS_>
struct Fs2Cfg {
    using SPA = StockhamPlan<float, LA, E_>;
    using SPB = StockhamPlan<float, LB, E_>;
    static constexpr int E = E_, CT = CT_, NS = NS_;
    static constexpr int GA = SPA::G, GB = SPB::G;  // threads per pair unit
    static constexpr int UA = CT / GA, UB = CT / GB;  // pair units per item
    static constexpr int CC = 2 * UA, CR = 2 * UB;    // columns / rows per item
    static constexpr long long A = 1LL << LA, B = 1LL << LB, N = A * B;
    static constexpr int NC = (int)(B / CC), NR = (int)(A / CR);
    static constexpr int WARPS = CT / 32;
    static constexpr int THREADS = CT + 64;  // + producer warp + publisher warp
    static constexpr int BOXR = A < 256 ? (int)A : 256;
    static constexpr int STAGE = 2 * E * CT;  // complex elements: CC * A == CR * B
    static constexpr size_t STAGE_BYTES = (size_t)STAGE * 8;
    // exchange buffers (pair units side by side), reused by the epilogue
    static constexpr int XA = ppad_size((int)A), XB = ppad_size((int)B);
    static constexpr size_t XCH_OFF = (size_t)NS * STAGE_BYTES;
    static constexpr size_t XCH_BYTES = (size_t)imax<UA * XA, UB * XB>::value * 16;
    // epilogue layout: row k of RB bytes at k * RB + (k * RB / 128) * 16
    static constexpr size_t xpos_bytes(int rows, int rb) { return (size_t)rows * rb + (size_t)rows * rb / 128 * 16; }
    static constexpr bool EPI_FITS =
        xpos_bytes((int)A, CC * 8) <= XCH_BYTES && xpos_bytes((int)B, CR * 8) <= XCH_BYTES;
    static constexpr int LO_BITS = (LA + LB + 1) / 2;
    static constexpr int NLO = 1 << LO_BITS, NHI = (int)(N >> LO_BITS);
    static constexpr int TWA = SPA::TW, TWB = LA == LB ? 0 : SPB::TW;
    static constexpr size_t TAB_OFF = XCH_OFF + XCH_BYTES;
    static constexpr size_t TAB_BYTES = (size_t)(TWA + TWB + NLO + NHI) * 8;
    // twiddle tables in shared memory when they fit beside the stages and
    // the exchange buffers, else read through the L1 cache
    static constexpr int NP = 4;  // publisher hand-off ring
    static constexpr size_t BAR_BYTES = (size_t)(2 * NS + 2 * NP) * 8 + (NS + NP) * 4 + 16;
    static constexpr bool TAB_SMEM = TAB_OFF + TAB_BYTES + BAR_BYTES <= 227 * 1024;
    static constexpr size_t BAR_OFF = (TAB_OFF + (TAB_SMEM ? TAB_BYTES : 0) + 15) / 16 * 16;
    static constexpr size_t SMEM = BAR_OFF + BAR_BYTES;
    // a pair unit of one warp exchanges under __syncwarp; longer units use
    // named barriers 2 .. 2 + units - 1 (1 is the compute warps' barrier)
    static constexpr bool SYNC_FITS = (GA == 32 || (GA % 32 == 0 && UA <= 14)) && (GB == 32 || (GB % 32 == 0 && UB <= 14));
    static constexpr bool FITS = SMEM <= 227 * 1024 && CT % 32 == 0 && CT % GA == 0 && CT % GB == 0 && UA >= 1 &&
                                 UB >= 1 && CC <= 16 && CR <= 16 && B % CC == 0 && A % CR == 0 && A % BOXR == 0 &&
                                 EPI_FITS && SYNC_FITS;
    // two CTAs an SM where their shared memory fits (8 pair points a
    // thread keep the registers within half the file)
    static constexpr int MIN_BLOCKS = (E <= 8 && THREADS <= 320 && 2 * (SMEM + 1024) <= 228 * 1024) ? 2 : 1;
};

// named barrier `id` over `n` threads
__device__ __forceinline__ void bar_named(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// the exchange barrier of pair unit u (G threads)
template <int G>
__device__ __forceinline__ void unit_sync(int u)
{
    if constexpr (G == 32) __syncwarp();
    else bar_named(2 + u, G);
}

template <int LA, int LB, int E_, int CT_, int NS_, bool INV>
__global__ void __launch_bounds__(Fs2Cfg<LA, LB, E_, CT_, NS_>::THREADS, Fs2Cfg<LA, LB, E_, CT_, NS_>::MIN_BLOCKS)
    k_fs2(const __grid_constant__ CUtensorMap map, const FourStepArgs a)
{
    using Cfg = Fs2Cfg<LA, LB, E_, CT_, NS_>;
    constexpr int E = Cfg::E, CT = Cfg::CT, NS = Cfg::NS, NP = Cfg::NP, GA = Cfg::GA, GB = Cfg::GB;
    constexpr int CC = Cfg::CC, CR = Cfg::CR, NC = Cfg::NC, NR = Cfg::NR;
    constexpr long long A = Cfg::A, B = Cfg::B, N = Cfg::N;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    float2 *const stage0 = reinterpret_cast<float2 *>(smem_raw);
    unsigned char *const xch = smem_raw + Cfg::XCH_OFF;
    float2 *const s_tab = reinterpret_cast<float2 *>(smem_raw + Cfg::TAB_OFF);
    uint64_t *const full = reinterpret_cast<uint64_t *>(smem_raw + Cfg::BAR_OFF);
    uint64_t *const empty = full + NS;
    uint64_t *const stored = empty + NS;   // compute warps -> publisher
    uint64_t *const pubfree = stored + NP;  // publisher -> compute thread 0
    int *const item_of = reinterpret_cast<int *>(pubfree + NP);
    int *const pub_slot = item_of + NS;

    // the twiddle tables, read through the shared-memory copies or the L1
    const float2 *const g_twa = static_cast<const float2 *>(a.tw_a);
    const float2 *const g_twb = static_cast<const float2 *>(a.tw_b);
    const float2 *const g_lo = static_cast<const float2 *>(a.tw_lo);
    const float2 *const g_hi = static_cast<const float2 *>(a.tw_hi);
    constexpr int O_TWB = LA == LB ? 0 : Cfg::TWA, O_LO = Cfg::TWA + Cfg::TWB, O_HI = O_LO + Cfg::NLO;
    auto tw_a = [&](int i) -> float2 {
        if constexpr (Cfg::TAB_SMEM) return s_tab[i];
        else return __ldg(g_twa + i);
    };
    auto tw_b = [&](int i) -> float2 {
        if constexpr (Cfg::TAB_SMEM) return s_tab[O_TWB + i];
        else return __ldg(g_twb + i);
    };
    auto tw_lo = [&](unsigned i) -> float2 {
        if constexpr (Cfg::TAB_SMEM) return s_tab[O_LO + i];
        else return __ldg(g_lo + i);
    };
    auto tw_hi = [&](unsigned i) -> float2 {
        if constexpr (Cfg::TAB_SMEM) return s_tab[O_HI + i];
        else return __ldg(g_hi + i);
    };
    if constexpr (Cfg::TAB_SMEM) {
        auto copy = [](float2 *d, const float2 *s, int n) {
            for (int i = threadIdx.x; i < n; i += Cfg::THREADS) d[i] = __ldg(s + i);
        };
        copy(s_tab, g_twa, Cfg::TWA);
        if (LA != LB) copy(s_tab + Cfg::TWA, g_twb, Cfg::TWB);
        copy(s_tab + O_LO, g_lo, Cfg::NLO);
        copy(s_tab + O_HI, g_hi, Cfg::NHI);
    }

    int *const abort_flag = a.ctr + 1;
    int *const col_done = a.ctr + 2;
    int *const row_done = a.ctr + 2 + a.slots;
    const int per_phase = NC + NR;

    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], Cfg::WARPS);
        }
        for (int i = 0; i < NP; i++) {
            mbar_init(&stored[i], Cfg::WARPS);
            mbar_init(&pubfree[i], 1);
        }
        fence_barrier_init();
    }
    __syncthreads();

    if (threadIdx.x >= CT + 32) {
        // ================= publisher (one thread): item k's hand-off
        // (pub_slot: col slot >= 0, -1 - slot for a ROW item, END) ->
        // fence -> count; in item order
        constexpr int END = -0x40000000;
        if (threadIdx.x != CT + 32) return;
        for (int k = 0;; k++) {
            const int s = k % NP;
            if (!mbar_wait(&stored[s], (uint32_t)((k / NP) & 1))) {
                atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                atomicExch(abort_flag, 1);
                break;
            }
            const int v = pub_slot[s];
            if (v == END) break;
            __threadfence();
            if (v >= 0) atomicAdd(col_done + v, 1);
            else atomicAdd(row_done + (-1 - v), 1);
            mbar_arrive(&pubfree[s]);
        }
        return;
    }
    if (threadIdx.x >= CT) {
        // ================= producer (one thread), as in k_fourstep
        if (threadIdx.x != CT) return;
        // the input is read once: its L2 lines go first, before the ring's
        const uint64_t in_policy = l2_policy_evict_first();
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
            float2 *S = stage0 + (size_t)st * Cfg::STAGE;
            if (j < NC) {
                item_of[st] = item;
                mbar_arrive_expect_tx(&full[st], (uint32_t)(A * CC * 8));
#pragma unroll 1
                for (int r = 0; r < (int)A; r += Cfg::BOXR)
                    tensor_load_3d_hint(S + (size_t)r * CC, &map, j * CC, r, p, &full[st], in_policy);
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
                const float2 *src =
                    static_cast<const float2 *>(a.ws) + (long long)slot * N + (long long)(j - NC) * CR * B;
                item_of[st] = item;
                mbar_arrive_expect_tx(&full[st], (uint32_t)(CR * B * 8));
#pragma unroll 1
                for (int s = 0; s < CR; s++)
                    bulk_load(S + (size_t)s * B, src + (long long)s * B, (uint32_t)(B * 8), &full[st]);
            }
            k++;
        }
        if (failed) {
            atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
            atomicExch(abort_flag, 1);
            for (int i = k - NS < 0 ? 0 : k - NS; i < k; i++) mbar_wait(&full[i % NS], (uint32_t)((i / NS) & 1));
        }
        return;
    }

    // ===================== compute warps
    const int tid = threadIdx.x, lane = tid & 31;
    constexpr int END = -0x40000000;
    // hand item k to the publisher: thread 0 records what to count (after
    // the publisher has taken item k - NP from the same place), then every
    // warp arrives once its own stores are issued
    auto publish = [&](int k, int what) -> bool {
        bool ok = true;
        if (tid == 0) {
            if (k >= NP) ok = mbar_wait(&pubfree[k % NP], (uint32_t)(((k / NP) - 1) & 1));
            pub_slot[k % NP] = what;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&stored[k % NP]);
        return ok;
    };
    const float scale = (float)a.scale;
    for (int k = 0;; k++) {
        const int st = k % NS;
        const uint32_t ph = (uint32_t)((k / NS) & 1);
        bool ok = mbar_wait(&full[st], ph);
        const int item = ok ? item_of[st] : -1;
        int p = 0, j = 0;
        if (item >= 0) {
            p = item / per_phase;
            j = item - p * per_phase;
        }
        if (ok && item >= 0) {
            if (j < NC) {
                // COL: the slot must be free (every ROW item of transform
                // p - S counted) before this item stores into it
                const int use = p / a.slots;
                if (tid == 0 && use > 0) ok = fs_wait_geq(row_done + p % a.slots, use * NR, abort_flag);
            } else {
                // ROW: its rows are in shared memory; drop their L2 lines
                // without a write-back (the slot is rewritten before it is
                // read again)
                const long long t = p - a.lag;
                const char *base = reinterpret_cast<const char *>(static_cast<const float2 *>(a.ws) +
                                                                  (long long)(t % a.slots) * N +
                                                                  (long long)(j - NC) * CR * B);
                constexpr int LINES = (int)(CR * B * 8 / 128);
                for (int i = tid; i < LINES; i += CT)
                    asm volatile("discard.global.L2 [%0], 128;" ::"l"(base + (size_t)i * 128) : "memory");
            }
        }
        // every compute thread agrees, and is done with the last item's
        // exchange buffers
        if (!bar_compute_and(CT, ok)) {
            if (tid == 0) {
                atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                atomicExch(abort_flag, 1);
            }
            break;
        }
        if (item < 0) {
            publish(k, END);
            break;
        }
        const float2 *S = stage0 + (size_t)st * Cfg::STAGE;
        if (j < NC) {
            // ---------------- COL item j of transform p
            const int slot = p % a.slots;
            const int u = tid / GA, tt = tid - u * GA;  // pair unit: columns 2u, 2u + 1
            pcx v[E];
#pragma unroll
            for (int q = 0; q < E; q++) {
                const float4 x = *reinterpret_cast<const float4 *>(S + (size_t)(tt + q * GA) * CC + 2 * u);
                v[q] = pcx{make_float2(x.x, x.z), make_float2(x.y, x.w)};
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            pcx *my = reinterpret_cast<pcx *>(xch) + (size_t)u * Cfg::XA;
            pstockham_run<LA, E, INV>(
                v, tt, [my](int i) -> pcx & { return my[ppad(i)]; }, tw_a, [u]() { unit_sync<GA>(u); });
            // W_N^(col k1) twiddle, then the tile through shared memory:
            // row k1 holds the item's CC columns (CC * 8 bytes)
            const unsigned col = (unsigned)(j * CC + 2 * u);
            constexpr unsigned lo_mask = (1u << Cfg::LO_BITS) - 1u;
            constexpr int RB = CC * 8;
            bar_compute(CT);
#pragma unroll
            for (int q = 0; q < E; q++) {
                const unsigned k1 = (unsigned)(tt + q * GA);
                const unsigned e0 = (col * k1) & (unsigned)(N - 1), e1 = (e0 + k1) & (unsigned)(N - 1);
                const float2 h0 = tw_hi(e0 >> Cfg::LO_BITS), l0 = tw_lo(e0 & lo_mask);
                const float2 h1 = tw_hi(e1 >> Cfg::LO_BITS), l1 = tw_lo(e1 & lo_mask);
                const cpx<float> w0 = cmul(cpx<float>{h0.x, h0.y}, cpx<float>{l0.x, l0.y});
                const cpx<float> w1 = cmul(cpx<float>{h1.x, h1.y}, cpx<float>{l1.x, l1.y});
                const pcx r = ptw2<INV>(v[q], make_float2(w0.x, w1.x), make_float2(w0.y, w1.y));
                const size_t off = (size_t)k1 * RB + (size_t)k1 * RB / 128 * 16 + (size_t)u * 16;
                *reinterpret_cast<float4 *>(xch + off) = make_float4(r.re.x, r.im.x, r.re.y, r.im.y);
            }
            bar_compute(CT);
            // 16-byte chunk c of the tile: row c / (CC/2), columns 2 (c % (CC/2)) + 0, 1
            // the ring stays in L2 until its ROW items read it (and drop it)
            float2 *wsl = static_cast<float2 *>(a.ws) + (long long)slot * N + (long long)j * CC;
            const uint64_t ring_policy = l2_policy_evict_last();
#pragma unroll 4
            for (int c = tid; c < Cfg::STAGE / 2; c += CT) {
                const int k1 = c / (CC / 2), h = c - k1 * (CC / 2);
                const size_t off = (size_t)k1 * RB + (size_t)k1 * RB / 128 * 16 + (size_t)h * 16;
                st_global_v4_hint(wsl + (long long)k1 * B + 2 * h, *reinterpret_cast<const float4 *>(xch + off),
                                  ring_policy);
            }
            if (!publish(k, slot)) {
                atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                atomicExch(abort_flag, 1);
            }
        } else {
            // ---------------- ROW item: rows k1 .. k1 + CR - 1 of transform p - LAG
            const long long t = p - a.lag;
            if (!publish(k, -1 - (int)(t % a.slots))) {
                atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                atomicExch(abort_flag, 1);
            }
            const int u = tid / GB, tt = tid - u * GB;  // pair unit: rows 2u, 2u + 1
            pcx v[E];
#pragma unroll
            for (int q = 0; q < E; q++) {
                const int b = tt + q * GB;
                const float2 x0 = S[(size_t)(2 * u) * B + b], x1 = S[(size_t)(2 * u + 1) * B + b];
                v[q] = pcx{make_float2(x0.x, x1.x), make_float2(x0.y, x1.y)};
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            pcx *my = reinterpret_cast<pcx *>(xch) + (size_t)u * Cfg::XB;
            pstockham_run<LB, E, INV>(
                v, tt, [my](int i) -> pcx & { return my[ppad(i)]; }, tw_b, [u]() { unit_sync<GB>(u); });
            // through shared memory: row k2 holds the item's CR rows k1
            constexpr int RB = CR * 8;
            const bool scaled = scale != 1.0f;
            bar_compute(CT);
#pragma unroll
            for (int q = 0; q < E; q++) {
                const int k2 = tt + q * GB;
                const pcx r = scaled ? pscl(v[q], scale) : v[q];
                const size_t off = (size_t)k2 * RB + (size_t)k2 * RB / 128 * 16 + (size_t)u * 16;
                *reinterpret_cast<float4 *>(xch + off) = make_float4(r.re.x, r.im.x, r.re.y, r.im.y);
            }
            bar_compute(CT);
            float2 *dst = static_cast<float2 *>(a.out) + t * a.odist + (long long)(j - NC) * CR;
#pragma unroll 4
            for (int c = tid; c < Cfg::STAGE / 2; c += CT) {
                const int k2 = c / (CR / 2), h = c - k2 * (CR / 2);
                const size_t off = (size_t)k2 * RB + (size_t)k2 * RB / 128 * 16 + (size_t)h * 16;
                __stcs(reinterpret_cast<float4 *>(dst + (long long)k2 * A + 2 * h),
                       *reinterpret_cast<const float4 *>(xch + off));
            }
        }
    }
}

}  // namespace gfft
