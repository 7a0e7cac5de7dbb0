// fourstep2.cuh -- the persistent four-step C2C (fourstep.cuh) with two
// sub-transforms per thread on packed FP32 instructions (pair.cuh), for
// fp32 n = A * B with A, B = 2^9 .. 2^12 (n = 2^18 .. 2^24).
//
// Same split, schedule and intermediate ring as k_fourstep: COL items (CC
// columns of A points of transform p, HBM -> FFT -> W_N twiddle -> ring slot)
// and ROW items (CR rows of B points of a slot -> FFT -> transposed store to
// HBM), claimed in a fixed order through one counter, with bounded waits on
// the COL -> ROW and slot-reuse dependencies; the ring stays in L2, so HBM
// sees one read of the input and one write of the output.
//
// What changes is the tile work, which bounds k_fourstep at these sizes:
//   * each thread holds 16 pair points (two adjacent columns of a COL item,
//     two adjacent rows of a ROW item), so the butterflies, rotations and
//     twiddle products of two transforms issue as one packed instruction;
//   * the compute threads form groups of GS = max(A, B)/16 threads (one
//     pair of sub-transforms, or two of the shorter length), each with its
//     own padded exchange buffer and its own named barrier, so a group never
//     waits for another group's exchanges;
//   * a warp hands the stage back to the producer as soon as it has read its
//     points (the exchanges use the group buffers), so the next item's copy
//     overlaps the whole transform of this one;
//   * a ROW item stores each pair point as one 16-byte store: its two rows
//     k1, k1 + 1 are neighbours in the output (k = k1 + A k2), and the
//     item's CR rows fill whole 32-byte sectors.
// Accounting: col_done[slot] counts warps that stored their part of a COL
// item, row_done[slot] counts groups that read their part of a ROW item.
#pragma once

#include "fourstep.cuh"
#include "pair.cuh"

namespace gfft {

template <int LA, int LB, int CT_, int NS_>
struct Fs2Cfg {
    using SPA = StockhamPlan<float, LA, 16>;
    using SPB = StockhamPlan<float, LB, 16>;
    static constexpr int CT = CT_, NS = NS_;
    static constexpr int GA = SPA::G, GB = SPB::G;
    static constexpr int GS = GA > GB ? GA : GB;  // threads per barrier group
    static constexpr int NG = CT / GS;             // groups
    static constexpr int UA = GS / GA, UB = GS / GB;  // pair units per group (COL / ROW)
    static constexpr int CC = 2 * CT / GA;  // columns per COL item
    static constexpr int CR = 2 * CT / GB;  // rows per ROW item
    static constexpr long long A = 1LL << LA, B = 1LL << LB, N = A * B;
    static constexpr int NC = (int)(B / CC), NR = (int)(A / CR);
    static constexpr int WARPS = CT / 32;
    static constexpr int THREADS = CT + 32;
    static constexpr int BOXR = A < 256 ? (int)A : 256;
    static constexpr int STAGE = 32 * CT;  // complex elements: CC * A == CR * B
    static constexpr size_t STAGE_BYTES = (size_t)STAGE * 8;
    // exchange buffer of one group, in pair points
    static constexpr int XG = imax<UA * ppad_size((int)A), UB * ppad_size((int)B)>::value;
    static constexpr size_t XCH_OFF = (size_t)NS * STAGE_BYTES;
    static constexpr size_t XCH_BYTES = (size_t)NG * XG * 16;
    static constexpr int LO_BITS = (LA + LB + 1) / 2;
    static constexpr int NLO = 1 << LO_BITS, NHI = (int)(N >> LO_BITS);
    static constexpr int TWA = SPA::TW, TWB = LA == LB ? 0 : SPB::TW;
    static constexpr size_t TAB_OFF = XCH_OFF + XCH_BYTES;
    static constexpr size_t TAB_BYTES = (size_t)(TWA + TWB + NLO + NHI) * 8;
    // twiddle tables in shared memory when they fit beside the stages and
    // the exchange buffers, else read through the L1 cache
    static constexpr bool TAB_SMEM = TAB_OFF + TAB_BYTES + 128 <= 227 * 1024;
    static constexpr size_t BAR_OFF = (TAB_OFF + (TAB_SMEM ? TAB_BYTES : 0) + 15) / 16 * 16;
    static constexpr size_t SMEM = BAR_OFF + 128;
    static constexpr bool FITS = SMEM <= 227 * 1024 && CT % 32 == 0 && GS >= 32 && CT % GS == 0 && NG >= 1 &&
                                 NG <= 15 && CC >= 2 && CR >= 2 && B % CC == 0 && A % CR == 0 && A % BOXR == 0;
};

// named barrier `id` over `n` threads, and the same returning the AND of a
// predicate over them
__device__ __forceinline__ void bar_named(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ bool bar_named_and(int id, int n, bool pred)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}

template <int LA, int LB, int CT_, int NS_, bool INV>
__global__ void __launch_bounds__(Fs2Cfg<LA, LB, CT_, NS_>::THREADS, 1)
    k_fs2(const __grid_constant__ CUtensorMap map, const FourStepArgs a)
{
    using Cfg = Fs2Cfg<LA, LB, CT_, NS_>;
    constexpr int CT = Cfg::CT, NS = Cfg::NS, GS = Cfg::GS, GA = Cfg::GA, GB = Cfg::GB;
    constexpr int CC = Cfg::CC, CR = Cfg::CR, NC = Cfg::NC, NR = Cfg::NR, NG = Cfg::NG;
    constexpr long long A = Cfg::A, B = Cfg::B, N = Cfg::N;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    float2 *const stage0 = reinterpret_cast<float2 *>(smem_raw);
    pcx *const xch0 = reinterpret_cast<pcx *>(smem_raw + Cfg::XCH_OFF);
    uint64_t *const full = reinterpret_cast<uint64_t *>(smem_raw + Cfg::BAR_OFF);
    uint64_t *const empty = full + NS;
    int *const item_of = reinterpret_cast<int *>(empty + NS);

    // twiddle tables: shared-memory copies or the global ones
    const float2 *twa = static_cast<const float2 *>(a.tw_a), *twb = static_cast<const float2 *>(a.tw_b);
    const float2 *tlo = static_cast<const float2 *>(a.tw_lo), *thi = static_cast<const float2 *>(a.tw_hi);
    if constexpr (Cfg::TAB_SMEM) {
        float2 *t0 = reinterpret_cast<float2 *>(smem_raw + Cfg::TAB_OFF);
        auto copy = [](float2 *d, const float2 *s, int n) {
            for (int i = threadIdx.x; i < n; i += Cfg::THREADS) d[i] = __ldg(s + i);
        };
        copy(t0, twa, Cfg::TWA);
        if (LA != LB) copy(t0 + Cfg::TWA, twb, Cfg::TWB);
        copy(t0 + Cfg::TWA + Cfg::TWB, tlo, Cfg::NLO);
        copy(t0 + Cfg::TWA + Cfg::TWB + Cfg::NLO, thi, Cfg::NHI);
        twa = t0;
        twb = LA == LB ? t0 : t0 + Cfg::TWA;
        tlo = t0 + Cfg::TWA + Cfg::TWB;
        thi = tlo + Cfg::NLO;
    }
    auto ldtw = [](const float2 *p) -> float2 {
        if constexpr (Cfg::TAB_SMEM) return *p;
        else return __ldg(p);
    };

    int *const abort_flag = a.ctr + 1;
    int *const col_done = a.ctr + 2;
    int *const row_done = a.ctr + 2 + a.slots;
    const int per_phase = NC + NR;

    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], Cfg::WARPS);
        }
        fence_barrier_init();
    }
    __syncthreads();

    if (threadIdx.x >= CT) {
        // ================= producer (one thread), as in k_fourstep
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
            float2 *S = stage0 + (size_t)st * Cfg::STAGE;
            if (j < NC) {
                item_of[st] = item;
                mbar_arrive_expect_tx(&full[st], (uint32_t)(A * CC * 8));
#pragma unroll 1
                for (int r = 0; r < (int)A; r += Cfg::BOXR)
                    tensor_load_3d(S + (size_t)r * CC, &map, j * CC, r, p, &full[st]);
            } else {
                const long long t = p - a.lag;
                const int slot = (int)(t % a.slots), use = (int)(t / a.slots);
                if (!fs_wait_geq(col_done + slot, (use + 1) * NC * Cfg::WARPS, abort_flag)) {
                    item_of[st] = -1;  // the stage is ours: tell the compute warps to stop
                    mbar_arrive(&full[st]);
                    failed = true;
                    break;
                }
                __threadfence();
                fence_proxy_async_global();
                const float2 *src = static_cast<const float2 *>(a.ws) + (long long)slot * N + (long long)(j - NC) * CR * B;
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

    // ===================== compute groups
    const int tid = threadIdx.x;
    const int g = tid / GS, gt = tid - g * GS, lane = tid & 31;
    auto gsync = [g]() {
        if constexpr (GS == 32) __syncwarp();
        else bar_named(1 + g, GS);
    };
    auto gsync_and = [g](bool pred) -> bool {
        if constexpr (GS == 32) return __all_sync(0xffffffffu, pred);
        else return bar_named_and(1 + g, GS, pred);
    };
    pcx *const xg = xch0 + (size_t)g * Cfg::XG;
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
                // COL: the slot must be free (every group of every ROW item
                // of transform p - S has read it) before this item stores
                const int use = p / a.slots;
                if (gt == 0 && use > 0) ok = fs_wait_geq(row_done + p % a.slots, use * NR * NG, abort_flag);
            } else {
                // ROW: the rows are in shared memory; drop this group's L2
                // lines of the slot without a write-back (the slot is
                // rewritten before it is read again)
                const long long t = p - a.lag;
                const char *base = reinterpret_cast<const char *>(
                    static_cast<const float2 *>(a.ws) + (long long)(t % a.slots) * N +
                    ((long long)(j - NC) * CR + 2LL * Cfg::UB * g) * B);
                constexpr int LINES = (int)(2 * Cfg::UB * B * 8 / 128);
                for (int i = gt; i < LINES; i += GS)
                    asm volatile("discard.global.L2 [%0], 128;" ::"l"(base + (size_t)i * 128) : "memory");
            }
        }
        // the group agrees (and every thread of it is done with the last
        // item's exchange buffer)
        if (!gsync_and(ok)) {
            if (gt == 0) {
                atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                atomicExch(abort_flag, 1);
            }
            break;
        }
        if (item < 0) break;
        const float2 *S = stage0 + (size_t)st * Cfg::STAGE;
        if (j < NC) {
            // ---------------- COL item j of transform p: columns c0, c0 + 1
            const int slot = p % a.slots;
            const int u = gt / GA, tt = gt - u * GA;
            const int c0 = 2 * (g * Cfg::UA + u);
            pcx v[16];
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const float4 x = *reinterpret_cast<const float4 *>(S + (size_t)(tt + q * GA) * CC + c0);
                v[q] = pcx{make_float2(x.x, x.z), make_float2(x.y, x.w)};
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            pcx *my = xg + (size_t)u * ppad_size((int)A);
            pstockham_run<LA, INV>(
                v, tt, [my](int i) -> pcx & { return my[ppad(i)]; }, [twa, ldtw](int i) { return ldtw(twa + i); },
                gsync);
            const unsigned col = (unsigned)(j * CC + c0);
            float2 *dst = static_cast<float2 *>(a.ws) + (long long)slot * N + col + (long long)tt * B;
            constexpr unsigned lo_mask = (1u << Cfg::LO_BITS) - 1u;
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const unsigned k1 = (unsigned)(tt + q * GA);
                const unsigned e0 = (col * k1) & (unsigned)(N - 1), e1 = (e0 + k1) & (unsigned)(N - 1);
                const float2 h0 = ldtw(thi + (e0 >> Cfg::LO_BITS)), l0 = ldtw(tlo + (e0 & lo_mask));
                const float2 h1 = ldtw(thi + (e1 >> Cfg::LO_BITS)), l1 = ldtw(tlo + (e1 & lo_mask));
                const cpx<float> w0 = cmul(cpx<float>{h0.x, h0.y}, cpx<float>{l0.x, l0.y});
                const cpx<float> w1 = cmul(cpx<float>{h1.x, h1.y}, cpx<float>{l1.x, l1.y});
                const pcx r = ptw2<INV>(v[q], make_float2(w0.x, w1.x), make_float2(w0.y, w1.y));
                *reinterpret_cast<float4 *>(dst + (long long)q * GA * B) = make_float4(r.re.x, r.im.x, r.re.y, r.im.y);
                if ((q & 3) == 3) asm volatile("" ::: "memory");
            }
            __syncwarp();
            if (lane == 0) {
                __threadfence();
                atomicAdd(col_done + slot, 1);
            }
        } else {
            // ---------------- ROW item: rows k1, k1 + 1 of transform p - LAG
            const long long t = p - a.lag;
            const int u = gt / GB, tt = gt - u * GB;
            const int r0 = 2 * (g * Cfg::UB + u);
            if (gt == 0) {
                __threadfence();
                atomicAdd(row_done + (int)(t % a.slots), 1);
            }
            pcx v[16];
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int b = tt + q * GB;
                const float2 x0 = S[(size_t)r0 * B + b], x1 = S[(size_t)(r0 + 1) * B + b];
                v[q] = pcx{make_float2(x0.x, x1.x), make_float2(x0.y, x1.y)};
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            pcx *my = xg + (size_t)u * ppad_size((int)B);
            pstockham_run<LB, INV>(
                v, tt, [my](int i) -> pcx & { return my[ppad(i)]; }, [twb, ldtw](int i) { return ldtw(twb + i); },
                gsync);
            const long long k1 = (long long)(j - NC) * CR + r0;
            float2 *dst = static_cast<float2 *>(a.out) + t * a.odist + k1;
            const bool scaled = scale != 1.0f;
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const long long k2 = tt + q * GB;
                const pcx r = scaled ? pscl(v[q], scale) : v[q];
                __stcs(reinterpret_cast<float4 *>(dst + k2 * A), make_float4(r.re.x, r.im.x, r.re.y, r.im.y));
            }
        }
    }
}

}  // namespace gfft
