// ragged.cu -- one persistent launch for a batch of transforms of uneven
// power-of-two sizes (fp32, n = 2^0 .. 2^18), packed back to back.
//
// The reference transforms one size per FFT<T> object (fft.h:56-113); a
// ragged batch there is a host loop over per-size plans.  Here a single
// persistent kernel walks a device work list of tiles of 4096 points:
//   SMALL (n <= 2^12): up to 4096 / n same-size transforms, one thread
//          group per transform (the fused Stockham engine);
//   COL / ROW (n = 2^13 .. 2^18): the two tile passes of the four-step split
//          n = A * B (tiles.cuh); column tiles write the transform's scratch,
//          and a ROW tile waits (bounded) until every column tile of its
//          transform is done (a per-transform counter).
// Each CTA is warp-specialised like the four-step kernel (fourstep.cuh): a
// producer warp claims items in list order through one atomic counter,
// resolves the ROW dependency and fills a ring of shared-memory stages with
// TMA bulk copies issued by its 32 lanes (one per small transform, one per
// column-tile row, one 32 KB copy per row tile); 256 compute threads take
// the stages in order.  A ROW item only waits on COL items earlier in the
// list, which running CTAs hold, so the schedule cannot deadlock; the list
// places each transform's ROW tiles `lag` items after its COL tiles so that
// they rarely wait, and the scratch a ROW tile has read is dropped from L2
// without a write-back.  Batches whose packing is not 16-byte aligned (sizes
// of one point) load tiles with the compute threads instead of TMA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "fourstep.cuh"
#include "internal.h"
#include "plan.h"
#include "tiles.cuh"
#include "tiles_registry.h"
#include "tma.cuh"
#include "twiddle.h"

namespace gfft {

namespace rg {

constexpr int CT = 256;            // compute threads
constexpr int THREADS = CT + 32;   // + the producer warp
constexpr int E = 16;              // points per thread
constexpr int TILE = 4096;         // points per tile
constexpr int NS = 2;              // shared-memory stages
constexpr int MAX_SMALL_LOGN = 12;
constexpr int MAX_LOGN = 18;

enum ItemType { SMALL = 0, COL = 1, ROW = 2 };

struct Item {
    int type;
    int logn;
    int a;  // SMALL: first index into perm;  COL/ROW: transform index
    int b;  // SMALL: count;                  COL/ROW: tile index
};

// twiddle table offsets (elements) inside one concatenated table
struct Tables {
    int stock[MAX_LOGN + 1];  // Stockham table of length 2^l (E = 16)
    int lo[MAX_LOGN + 1];     // four-step split tables of length 2^l
    int hi[MAX_LOGN + 1];
};

struct Args {
    const cpx<float> *in;
    cpx<float> *out;
    cpx<float> *ws;
    const Item *items;
    const int *perm;            // SMALL items index transforms through perm
    const long long *off;       // element offset of each transform
    const long long *wsoff;     // scratch offset of each large transform
    int *col_done;              // per-transform finished column tiles
    int *counter;               // [0] next item, [1] abort
    unsigned *err;
    const cpx<float> *tw;
    const CUtensorMap *maps;    // per large transform: its input as [A rows][B] (COL tiles), or null
    int nitems;
    int tma;                    // 1: TMA copies into the stages, 0: thread loads
    Tables tab;
};

__host__ __device__ constexpr int split_a(int logn) { return logn / 2; }
__host__ __device__ constexpr int tile_c(int logl) { return TILE >> logl; }  // columns (rows) per tile
// transforms per SMALL tile: one thread group of max(1, n/16) threads each
__host__ __device__ constexpr int small_per_tile(int logn) { return logn <= 4 ? CT : TILE >> logn; }

// shared-memory elements one stage needs for every item layout
__host__ __device__ constexpr int stage_elems()
{
    int m = TILE + TILE / 16 + CT;  // SMALL: transforms in padded slots
    for (int l = 6; l <= 9; l++) {
        const int c = tile_c(l), n = 1 << l;
        const int col = tile_pitch<float>(n, c) * c;              // COL exchange layout
        const int row = (n + n / 16) * c;                         // ROW exchange layout
        m = m > col ? m : col;
        m = m > row ? m : row;
    }
    const int x = spad_size<float>(TILE);  // ROW transpose
    m = m > x ? m : x;
    return (m + 15) / 16 * 16;  // 128-byte multiple
}
constexpr int STAGE = stage_elems();
// Stockham tables of the tile lengths 2^6 .. 2^9, staged once per CTA
template <int L>
struct TwOff {
    static constexpr int value = TwOff<L - 1>::value + StockhamPlan<float, L - 1, E>::TW;
};
template <>
struct TwOff<6> {
    static constexpr int value = 0;
};
constexpr int TW_ELEMS = TwOff<10>::value;
// per stage: the item and, for SMALL items, each transform's output offset
struct StageInfo {
    Item it;
    long long out_off[CT];
};
constexpr size_t TW_OFF = (size_t)NS * STAGE * sizeof(cpx<float>);
constexpr size_t INFO_OFF = (TW_OFF + (size_t)TW_ELEMS * sizeof(cpx<float>) + 127) / 128 * 128;
constexpr size_t BAR_OFF = INFO_OFF + (size_t)NS * sizeof(StageInfo);
constexpr size_t SMEM = BAR_OFF + 64;

// ---- SMALL: count transforms of 2^LOGN points, dense in the stage
template <int LOGN, bool INV>
__device__ void small_tile(const Args &A, const Item &it, cpx<float> *S, const long long *out_off)
{
    using SP = StockhamPlan<float, LOGN, E>;
    constexpr int G = SP::G, EE = SP::E, N = SP::N;
    constexpr int SLOT = spad_size<float>(N);
    const int g = threadIdx.x / G, t = threadIdx.x - g * G;
    const bool active = g < it.b;
    cpx<float> v[EE];
#pragma unroll
    for (int q = 0; q < EE; q++) v[q] = active ? S[g * N + t + q * G] : cpx<float>{0.f, 0.f};
    bar_compute(CT);
    cpx<float> *my = S + g * SLOT;
    stockham_run<float, LOGN, E, INV>(
        v, t, [my](int i) -> cpx<float> & { return my[spad<float>(i)]; }, A.tw + A.tab.stock[LOGN],
        []() { bar_compute(CT); });
    if (active) {
        cpx<float> *dst = A.out + out_off[g] + t;
#pragma unroll
        for (int q = 0; q < EE; q++) stcs_c(dst + q * G, v[q]);
    }
}

// ---- COL: tile it.b of the column pass of transform it.a
template <int LOGN, bool INV>
__device__ void col_tile(const Args &A, const Item &it, cpx<float> *S, const cpx<float> *tws)
{
    constexpr int LA = split_a(LOGN), LB = LOGN - LA;
    constexpr long long B = 1LL << LB;
    using SP = StockhamPlan<float, LA, E>;
    constexpr int G = SP::G, C = tile_c(LA);
    constexpr int PITCH = tile_pitch<float>(SP::N, C);
    const int s = threadIdx.x % C, t = threadIdx.x / C;
    const long long col = (long long)it.b * C + s;
    cpx<float> v[E];
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = S[(t + q * G) * C + s];  // rows of C columns, as copied
    bar_compute(CT);
    cpx<float> *my = S + s * PITCH;
    stockham_run<float, LA, E, INV, TwShared>(
        v, t, [my](int i) -> cpx<float> & { return my[spad<float>(i)]; }, tws + TwOff<LA>::value,
        []() { bar_compute(CT); });
    constexpr unsigned nmask = (1u << LOGN) - 1u;
    constexpr int lo_bits = (LOGN + 1) / 2;
    const cpx<float> *tlo = A.tw + A.tab.lo[LOGN], *thi = A.tw + A.tab.hi[LOGN];
    cpx<float> *dst = A.ws + A.wsoff[it.a] + col + (long long)t * B;
#pragma unroll
    for (int q = 0; q < E; q++) {
        const unsigned e = ((unsigned)col * (unsigned)(t + q * G)) & nmask;
        const cpx<float> w = cmul(ldg_c(thi + (e >> lo_bits)), ldg_c(tlo + (e & ((1u << lo_bits) - 1u))));
        st_c(dst + (long long)q * G * B, twmul<INV>(v[q], w));
        if ((q & 3) == 3) asm volatile("" ::: "memory");
    }
    // publish: the barrier orders every thread's stores before the count moves
    bar_compute(CT);
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(A.col_done + it.a, 1);
    }
}

// ---- ROW: tile it.b of the row pass of transform it.a (transposed store)
template <int LOGN, bool INV>
__device__ void row_tile(const Args &A, const Item &it, cpx<float> *S, const cpx<float> *tws)
{
    constexpr int LA = split_a(LOGN), LB = LOGN - LA;
    constexpr long long Acount = 1LL << LA, B = 1LL << LB;
    using SP = StockhamPlan<float, LB, E>;
    constexpr int G = SP::G, C = tile_c(LB);
    constexpr int ROWP = SP::SMEM;
    const int s = threadIdx.x / G, t = threadIdx.x - s * G;
    const long long row0 = (long long)it.b * C;
    {
        // the rows are in shared memory: drop their scratch lines from L2
        // without a write-back (nothing reads them again)
        const char *base = reinterpret_cast<const char *>(A.ws + A.wsoff[it.a] + row0 * B);
        constexpr int LINES = (int)(C * B * sizeof(cpx<float>) / 128);
        for (int i = threadIdx.x; i < LINES; i += CT)
            asm volatile("discard.global.L2 [%0], 128;" ::"l"(base + (size_t)i * 128) : "memory");
    }
    cpx<float> v[E];
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = S[s * B + t + q * G];
    bar_compute(CT);
    cpx<float> *my = S + s * ROWP;
    stockham_run<float, LB, E, INV, TwShared>(
        v, t, [my](int i) -> cpx<float> & { return my[spad<float>(i)]; }, tws + TwOff<LB>::value,
        []() { bar_compute(CT); });
    bar_compute(CT);
#pragma unroll
    for (int q = 0; q < E; q++) S[spad<float>((t + q * G) * C + s)] = v[q];
    bar_compute(CT);
    cpx<float> *dst = A.out + A.off[it.a] + row0;
#pragma unroll
    for (int m = 0; m < E; m++) {
        const int idx = threadIdx.x + m * CT;
        stcs_c(dst + idx % C + (long long)(idx / C) * Acount, S[spad<float>(idx)]);
    }
}

// bytes of the copies that fill the stage for `it`
__device__ __forceinline__ uint32_t item_bytes(const Item &it)
{
    if (it.type == SMALL) return (uint32_t)it.b << (it.logn + 3);
    return (uint32_t)TILE * 8u;
}

// lane `lane` of the producer warp issues its share of the item's copies
__device__ __forceinline__ void issue_copies(const Args &A, const Item &it, cpx<float> *S, uint64_t *bar, int lane)
{
    if (it.type == SMALL) {
        const int n = 1 << it.logn;
        for (int g = lane; g < it.b; g += 32)
            bulk_load(S + g * n, A.in + A.off[A.perm[it.a + g]], (uint32_t)n * 8u, bar);
    } else if (it.type == COL) {
        const int la = split_a(it.logn), c = tile_c(la);
        if (A.maps) {
            // boxes of c columns x up to 256 rows of the transform's [A][B] view
            const int boxr = la < 8 ? (1 << la) : 256;
            for (int r = lane * boxr; r < (1 << la); r += 32 * boxr)
                tensor_load_3d(S + r * c, A.maps + it.a, it.b * c, r, 0, bar);
        } else {
            const long long b = 1LL << (it.logn - la);
            const cpx<float> *src = A.in + A.off[it.a] + (long long)it.b * c;
            for (int r = lane; r < (1 << la); r += 32) bulk_load(S + r * c, src + r * b, (uint32_t)c * 8u, bar);
        }
    } else if (lane == 0) {
        const int la = split_a(it.logn), lb = it.logn - la;
        const long long row0 = (long long)it.b * tile_c(lb);
        bulk_load(S, A.ws + A.wsoff[it.a] + (row0 << lb), (uint32_t)TILE * 8u, bar);
    }
}

// compute threads load the item's tile themselves (unaligned packing)
__device__ void load_tile(const Args &A, const Item &it, cpx<float> *S)
{
    if (it.type == SMALL) {
        const int n = 1 << it.logn;
        for (int i = threadIdx.x; i < it.b * n; i += CT) S[i] = ld_c(A.in + A.off[A.perm[it.a + i / n]] + (i % n));
    } else if (it.type == COL) {
        const int la = split_a(it.logn), c = tile_c(la);
        const long long b = 1LL << (it.logn - la);
        const cpx<float> *src = A.in + A.off[it.a] + (long long)it.b * c;
        for (int i = threadIdx.x; i < TILE; i += CT) S[i] = ld_c(src + (i / c) * b + i % c);
    } else {
        const int la = split_a(it.logn), lb = it.logn - la;
        const cpx<float> *src = A.ws + A.wsoff[it.a] + (((long long)it.b * tile_c(lb)) << lb);
        for (int i = threadIdx.x; i < TILE; i += CT) {
            const float2 f = __ldcg(reinterpret_cast<const float2 *>(src + i));  // never a stale L1 line
            S[i] = cpx<float>{f.x, f.y};
        }
    }
    bar_compute(CT);
}

template <bool INV>
__global__ void __launch_bounds__(THREADS, 2) k_ragged(const Args A)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    cpx<float> *const stage0 = reinterpret_cast<cpx<float> *>(smem_raw);
    cpx<float> *const tws = reinterpret_cast<cpx<float> *>(smem_raw + TW_OFF);
    StageInfo *const info = reinterpret_cast<StageInfo *>(smem_raw + INFO_OFF);
    uint64_t *const full = reinterpret_cast<uint64_t *>(smem_raw + BAR_OFF);
    uint64_t *const empty = full + NS;
    int *const item_of = reinterpret_cast<int *>(empty + NS);
    int *const abort_flag = A.counter + 1;

    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        fence_barrier_init();
    }
    // Stockham tables of the tile lengths (read by every COL and ROW tile)
    for (int l = 6; l <= 9; l++) {
        const int n = l == 6 ? StockhamPlan<float, 6, E>::TW : l == 7 ? StockhamPlan<float, 7, E>::TW
                    : l == 8 ? StockhamPlan<float, 8, E>::TW : StockhamPlan<float, 9, E>::TW;
        const int o = l == 6 ? TwOff<6>::value : l == 7 ? TwOff<7>::value : l == 8 ? TwOff<8>::value : TwOff<9>::value;
        for (int i = threadIdx.x; i < n; i += THREADS) tws[o + i] = A.tw[A.tab.stock[l] + i];
    }
    __syncthreads();

    if (threadIdx.x >= CT) {
        // ================= producer warp: lane 0 decides, every lane copies
        const int lane = threadIdx.x - CT;
        int k = 0;
        bool failed = false;
        for (;;) {
            int idx = 0, st = k % NS, ok = 1;
            if (lane == 0) {
                idx = *(volatile int *)abort_flag ? A.nitems : atomicAdd(A.counter, 1);
                const uint32_t ph = (uint32_t)((k / NS) & 1);
                ok = mbar_wait(&empty[st], ph ^ 1u);
                if (ok && idx < A.nitems) {
                    const Item it = A.items[idx];
                    if (it.type == ROW) {
                        const int la = split_a(it.logn);
                        const int ncol = (1 << (it.logn - la)) / tile_c(la);
                        if (!fs_wait_geq(A.col_done + it.a, ncol, abort_flag)) {
                            ok = 0;
                            item_of[st] = -1;  // the stage is ours: stop the compute warps
                            mbar_arrive(&full[st]);
                        } else {
                            __threadfence();
                            fence_proxy_async_global();
                        }
                    }
                    if (ok) item_of[st] = idx;
                } else if (ok) {
                    item_of[st] = -1;
                    mbar_arrive(&full[st]);
                }
            }
            idx = __shfl_sync(0xffffffffu, idx, 0);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                failed = true;
                break;
            }
            if (idx >= A.nitems) break;
            // the item and the SMALL output offsets go beside the stage, so
            // the compute threads start without global look-ups
            const Item it = A.items[idx];
            if (lane == 0) info[st].it = it;
            if (it.type == SMALL)
                for (int g = lane; g < it.b; g += 32) info[st].out_off[g] = A.off[A.perm[it.a + g]];
            __syncwarp();
            if (lane == 0) {
                if (A.tma) mbar_arrive_expect_tx(&full[st], item_bytes(it));
                else mbar_arrive(&full[st]);  // the compute threads load this tile
            }
            __syncwarp();
            if (A.tma) issue_copies(A, it, stage0 + (size_t)st * STAGE, &full[st], lane);
            k++;
        }
        if (failed && lane == 0) {
            atomicOr(A.err, DEV_ERR_TMA_TIMEOUT);
            atomicExch(abort_flag, 1);
            for (int i = k - NS < 0 ? 0 : k - NS; i < k; i++) mbar_wait(&full[i % NS], (uint32_t)((i / NS) & 1));
        }
        return;
    }

    // ===================== compute threads
    for (int k = 0;; k++) {
        const int st = k % NS;
        const uint32_t ph = (uint32_t)((k / NS) & 1);
        if (!bar_compute_and(CT, mbar_wait(&full[st], ph))) {
            if (threadIdx.x == 0) {
                atomicOr(A.err, DEV_ERR_TMA_TIMEOUT);
                atomicExch(abort_flag, 1);
            }
            break;
        }
        const int idx = item_of[st];
        if (idx < 0) break;
        const Item it = info[st].it;
        cpx<float> *S = stage0 + (size_t)st * STAGE;
        if (!A.tma) load_tile(A, it, S);
        switch (it.type) {
        case SMALL:
            switch (it.logn) {
#define S_(L) case L: small_tile<L, INV>(A, it, S, info[st].out_off); break;
                S_(0) S_(1) S_(2) S_(3) S_(4) S_(5) S_(6) S_(7) S_(8) S_(9) S_(10) S_(11) S_(12)
#undef S_
            }
            break;
        case COL:
            switch (it.logn) {
#define S_(L) case L: col_tile<L, INV>(A, it, S, tws); break;
                S_(13) S_(14) S_(15) S_(16) S_(17) S_(18)
#undef S_
            }
            break;
        default:
            switch (it.logn) {
#define S_(L) case L: row_tile<L, INV>(A, it, S, tws); break;
                S_(13) S_(14) S_(15) S_(16) S_(17) S_(18)
#undef S_
            }
            break;
        }
        bar_compute(CT);  // the stage is read: hand it back to the producer
        if (threadIdx.x == 0) mbar_arrive(&empty[st]);
    }
}

}  // namespace rg

// ---------------------------------------------------------------------------
// host side

using rg::Item;

struct RaggedPlan {
    int device = 0;
    long long count = 0, total = 0;  // transforms, elements
    std::vector<int> logn;
    std::vector<long long> off;
    // tuning (autotuner-chosen)
    int lag_factor = 2;       // ROW tiles follow their COL tiles by lag_factor x (items in flight)
    int ctas_per_sm = 0;      // 0 = occupancy limit
    int large_first = 1;      // order large transforms before small ones
    int tma = 1;              // packing 16-byte aligned (no one-point transforms)
    // device state
    void *dev_items = nullptr, *dev_perm = nullptr, *dev_off = nullptr, *dev_wsoff = nullptr;
    int *dev_counters = nullptr;  // [0] item counter, [1] abort, [2..count+1] col_done
    void *ws = nullptr;
    size_t ws_bytes = 0;
    const void *tw = nullptr;
    rg::Tables tab{};
    int nitems = 0;
    int grid = 0;
    // captured graphs, keyed by (in, out, inverse)
    std::map<std::tuple<const void *, void *, int>, cudaGraphExec_t> graphs;
    // per input pointer: the tensor maps of the large transforms (COL tiles)
    std::map<const void *, void *> maps;
};

static void ragged_free_graphs(RaggedPlan &p)
{
    for (auto &kv : p.graphs) cudaGraphExecDestroy(kv.second);
    p.graphs.clear();
}

// (re)build the device work list for the current tuning parameters
static void ragged_build_items(RaggedPlan &p)
{
    // persistent grid first: the ROW lag is measured in items in flight
    int per_sm = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rg::k_ragged<false>, rg::THREADS, rg::SMEM),
               "occupancy");
    if (p.ctas_per_sm > 0) per_sm = std::min(per_sm, p.ctas_per_sm);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.device);
    p.grid = std::max(1, per_sm) * sms;
    const long long lag = (long long)p.grid * (rg::NS + 1) * std::max(1, p.lag_factor);

    std::vector<Item> items;
    std::vector<int> perm;
    // large transforms, biggest first; each ROW tile enters the list `lag`
    // items after the last COL tile of its transform
    std::vector<int> large;
    for (long long i = 0; i < p.count; i++)
        if (p.logn[i] > rg::MAX_SMALL_LOGN) large.push_back((int)i);
    std::stable_sort(large.begin(), large.end(), [&](int x, int y) { return p.logn[x] > p.logn[y]; });
    auto cols = [&](int i) {
        const int l = p.logn[i], la = rg::split_a(l);
        return (1 << (l - la)) / rg::tile_c(la);
    };
    auto rows = [&](int i) {
        const int l = p.logn[i], la = rg::split_a(l);
        return (1 << la) / rg::tile_c(l - la);
    };
    std::vector<Item> big;
    std::deque<std::pair<long long, Item>> ready;  // ROW items and the position they may take
    for (int t : large) {
        for (int c = 0; c < cols(t); c++) {
            while (!ready.empty() && ready.front().first <= (long long)big.size()) {
                big.push_back(ready.front().second);
                ready.pop_front();
            }
            big.push_back({rg::COL, p.logn[t], t, c});
        }
        const long long at = (long long)big.size() + lag;
        for (int r = 0; r < rows(t); r++) ready.push_back({at, Item{rg::ROW, p.logn[t], t, r}});
    }
    for (auto &q : ready) big.push_back(q.second);
    // small transforms grouped by size, biggest first, one tile per item
    std::vector<Item> small;
    for (int l = rg::MAX_SMALL_LOGN; l >= 0; l--) {
        std::vector<int> ids;
        for (long long i = 0; i < p.count; i++)
            if (p.logn[i] == l) ids.push_back((int)i);
        if (ids.empty()) continue;
        const int per = rg::small_per_tile(l);
        for (size_t k = 0; k < ids.size(); k += per) {
            const int cnt = (int)std::min<size_t>(per, ids.size() - k);
            small.push_back({rg::SMALL, l, (int)perm.size(), cnt});
            perm.insert(perm.end(), ids.begin() + k, ids.begin() + k + cnt);
        }
    }
    if (p.large_first) {
        items = big;
        items.insert(items.end(), small.begin(), small.end());
    } else {
        items = small;
        items.insert(items.end(), big.begin(), big.end());
    }
    if (perm.empty()) perm.push_back(0);
    if (items.empty()) fail(GFFT_ERR_INVALID_SIZE, "empty ragged batch");
    if (p.dev_items) cudaFree(p.dev_items);
    if (p.dev_perm) cudaFree(p.dev_perm);
    p.dev_items = p.dev_perm = nullptr;
    check_cuda(cudaMalloc(&p.dev_items, items.size() * sizeof(Item)), "cudaMalloc(items)");
    check_cuda(cudaMalloc(&p.dev_perm, perm.size() * sizeof(int)), "cudaMalloc(perm)");
    check_cuda(cudaMemcpy(p.dev_items, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice), "items");
    check_cuda(cudaMemcpy(p.dev_perm, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice), "perm");
    p.nitems = (int)items.size();
    ragged_free_graphs(p);
}

RaggedPlan *ragged_create(int dtype, const long long *sizes, long long count)
{
    if (dtype != GFFT_F32) fail(GFFT_ERR_UNSUPPORTED, "ragged batches are fp32");
    if (count < 1) fail(GFFT_ERR_INVALID_SIZE, "ragged batch needs at least one transform");
    std::unique_ptr<RaggedPlan> p(new RaggedPlan());
    check_cuda(cudaGetDevice(&p->device), "cudaGetDevice");
    p->count = count;
    p->logn.resize(count);
    p->off.resize(count);
    std::vector<long long> wsoff(count, 0);
    long long pos = 0, wpos = 0;
    for (long long i = 0; i < count; i++) {
        if (!is_pow2(sizes[i]) || sizes[i] > (1LL << rg::MAX_LOGN))
            fail(GFFT_ERR_INVALID_SIZE, "ragged sizes must be powers of two in [1, 2^18]");
        p->logn[i] = ilog2ll(sizes[i]);
        p->off[i] = pos;
        pos += sizes[i];
        if (p->logn[i] > rg::MAX_SMALL_LOGN) {
            wsoff[i] = wpos;
            wpos += sizes[i];
        }
    }
    p->total = pos;
    // twiddles: Stockham tables for every small length and tile length,
    // four-step split tables for every large length
    std::vector<cpx<float>> host;
    auto root = [](long long k, long long M, cpx<float> *w) { forward_root<float>(k, M, &w->x, &w->y); };
    auto add_stock = [&](int l, auto fill, size_t cnt) {
        p->tab.stock[l] = (int)host.size();
        host.resize(host.size() + std::max<size_t>(cnt, 1));
        fill(host.data() + p->tab.stock[l]);
    };
#define ST(L) add_stock(L, [&](cpx<float> *o) { stockham_fill_twiddles<float, L, rg::E>(o, root); }, \
                        (size_t)StockhamPlan<float, L, rg::E>::TW);
    ST(0) ST(1) ST(2) ST(3) ST(4) ST(5) ST(6) ST(7) ST(8) ST(9) ST(10) ST(11) ST(12)
#undef ST
    for (int l = rg::MAX_SMALL_LOGN + 1; l <= rg::MAX_LOGN; l++) {
        const long long N = 1LL << l;
        const int lo = (l + 1) / 2;
        p->tab.lo[l] = (int)host.size();
        for (long long e = 0; e < (1LL << lo); e++) { cpx<float> w; root(e, N, &w); host.push_back(w); }
        p->tab.hi[l] = (int)host.size();
        for (long long e = 0; e < (N >> lo); e++) { cpx<float> w; root(e << lo, N, &w); host.push_back(w); }
    }
    p->tw = cached_table("ragged/tw/" + std::to_string(host.size()), GFFT_F32, host.size(),
                         [&host](void *buf) { std::memcpy(buf, host.data(), host.size() * sizeof(cpx<float>)); });
    check_cuda(cudaMalloc(&p->dev_off, count * sizeof(long long)), "cudaMalloc(off)");
    check_cuda(cudaMemcpy(p->dev_off, p->off.data(), count * sizeof(long long), cudaMemcpyHostToDevice), "off");
    check_cuda(cudaMalloc(&p->dev_wsoff, count * sizeof(long long)), "cudaMalloc(wsoff)");
    check_cuda(cudaMemcpy(p->dev_wsoff, wsoff.data(), count * sizeof(long long), cudaMemcpyHostToDevice), "wsoff");
    check_cuda(cudaMalloc(&p->dev_counters, (count + 2) * sizeof(int)), "cudaMalloc(counters)");
    p->ws_bytes = (size_t)std::max<long long>(wpos, 1) * sizeof(cpx<float>);
    check_cuda(cudaMalloc(&p->ws, p->ws_bytes), "cudaMalloc(ragged scratch)");
    // TMA copies need every transform to start on 16 bytes: no one-point sizes
    p->tma = 1;
    for (long long i = 0; i < count; i++)
        if (p->logn[i] == 0) p->tma = 0;
    for (const void *fn : {(const void *)rg::k_ragged<false>, (const void *)rg::k_ragged<true>}) {
        check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rg::SMEM), "smem");
        check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                        cudaSharedmemCarveoutMaxShared),
                   "carveout");
    }
    device_error_word();  // allocate now: never inside a stream capture
    ragged_build_items(*p);
    return p.release();
}

void ragged_destroy(RaggedPlan *p)
{
    if (!p) return;
    ragged_free_graphs(*p);
    for (auto &kv : p->maps) cudaFree(kv.second);
    for (void *q : {p->dev_items, p->dev_perm, p->dev_off, p->dev_wsoff, (void *)p->dev_counters, p->ws})
        if (q) cudaFree(q);
    delete p;
}

long long ragged_total(const RaggedPlan *p) { return p->total; }

// Tensor maps of the large transforms for input `in` (built once per
// pointer, before any capture; nullptr when the batch cannot use TMA)
static const CUtensorMap *ragged_maps(RaggedPlan &p, const void *in, bool build)
{
    if (!p.tma || (uintptr_t)in % 16) return nullptr;
    auto it = p.maps.find(in);
    if (it != p.maps.end()) return static_cast<const CUtensorMap *>(it->second);
    if (!build) return nullptr;
    if (p.maps.size() >= 8) {
        for (auto &kv : p.maps) cudaFree(kv.second);
        p.maps.clear();
    }
    std::vector<CUtensorMap> h((size_t)p.count);
    std::memset(h.data(), 0, h.size() * sizeof(CUtensorMap));
    for (long long t = 0; t < p.count; t++) {
        const int l = p.logn[t];
        if (l <= rg::MAX_SMALL_LOGN) continue;
        const int la = rg::split_a(l);
        const unsigned long long A = 1ULL << la, B = 1ULL << (l - la);
        const char *base = static_cast<const char *>(in) + (size_t)p.off[t] * sizeof(cpx<float>);
        if (!make_tensor_map_3d(&h[t], base, B, A, 1, B * 8, A * B * 8, (unsigned)rg::tile_c(la),
                                (unsigned)std::min<unsigned long long>(A, 256)))
            return nullptr;
    }
    void *d = nullptr;
    check_cuda(cudaMalloc(&d, h.size() * sizeof(CUtensorMap)), "cudaMalloc(tensor maps)");
    check_cuda(cudaMemcpy(d, h.data(), h.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice), "tensor maps");
    p.maps[in] = d;
    return static_cast<const CUtensorMap *>(d);
}

static void ragged_enqueue(RaggedPlan &p, int inverse, void *out, const void *in, cudaStream_t st)
{
    check_cuda(cudaMemsetAsync(p.dev_counters, 0, (p.count + 2) * sizeof(int), st), "reset counters");
    rg::Args a;
    a.in = static_cast<const cpx<float> *>(in);
    a.out = static_cast<cpx<float> *>(out);
    a.ws = static_cast<cpx<float> *>(p.ws);
    a.items = static_cast<const Item *>(p.dev_items);
    a.perm = static_cast<const int *>(p.dev_perm);
    a.off = static_cast<const long long *>(p.dev_off);
    a.wsoff = static_cast<const long long *>(p.dev_wsoff);
    a.counter = p.dev_counters;
    a.col_done = p.dev_counters + 2;
    a.tma = p.tma && ((uintptr_t)in % 16 == 0) ? 1 : 0;
    a.maps = a.tma ? ragged_maps(p, in, false) : nullptr;
    a.err = device_error_word();
    a.tw = static_cast<const cpx<float> *>(p.tw);
    a.nitems = p.nitems;
    a.tab = p.tab;
    void *args[] = {&a};
    const void *fn = inverse ? (const void *)rg::k_ragged<true> : (const void *)rg::k_ragged<false>;
    check_cuda(cudaLaunchKernel(fn, dim3(p.grid), dim3(rg::THREADS), args, rg::SMEM, st), "launch ragged");
}

// One replay of the captured graph (counter reset + the persistent kernel);
// captured on first use for these pointers.
void ragged_exec(RaggedPlan &p, int inverse, void *out, const void *in, cudaStream_t st, bool use_graph)
{
    if (!in || !out) fail(GFFT_ERR_INVALID_VALUE, "NULL pointer");
    if (((uintptr_t)in | (uintptr_t)out) % 8) fail(GFFT_ERR_ALIGN, "pointers must be 8-byte aligned");
    ragged_maps(p, in, true);  // allocations happen here, never inside the capture
    if (!use_graph) {
        ragged_enqueue(p, inverse, out, in, st);
        return;
    }
    auto key = std::make_tuple(in, out, inverse);
    auto it = p.graphs.find(key);
    if (it == p.graphs.end()) {
        if (p.graphs.size() >= 8) ragged_free_graphs(p);
        cudaStream_t cap;
        check_cuda(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "stream");
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            try {
                ragged_enqueue(p, inverse, out, in, cap);
            } catch (...) {
                cudaStreamEndCapture(cap, &g);
                if (g) cudaGraphDestroy(g);
                cudaStreamDestroy(cap);
                throw;
            }
            e = cudaStreamEndCapture(cap, &g);
        }
        cudaStreamDestroy(cap);
        check_cuda(e, "graph capture");
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        check_cuda(e, "graph instantiate");
        it = p.graphs.emplace(key, ex).first;
    }
    check_cuda(cudaGraphLaunch(it->second, st), "graph launch");
}

// Autotuner: times the candidate schedules on the caller's buffers and
// keeps the fastest (cached on disk by GFFT_AUTOTUNE_CACHE when set).
static std::string ragged_key(const RaggedPlan &p)
{
    long long hist[rg::MAX_LOGN + 1] = {};
    for (int l : p.logn) hist[l]++;
    std::string k = "ragged/f32";
    for (int l = 0; l <= rg::MAX_LOGN; l++) k += "/" + std::to_string(hist[l]);
    return k;
}

static bool cache_lookup(const std::string &key, int *a, int *b, int *c)
{
    const char *path = std::getenv("GFFT_AUTOTUNE_CACHE");
    if (!path || !*path) return false;
    FILE *f = std::fopen(path, "r");
    if (!f) return false;
    char line[4096];
    bool found = false;
    while (std::fgets(line, sizeof line, f)) {
        char k[3000];
        int x, y, z;
        if (std::sscanf(line, "%2999s %d %d %d", k, &x, &y, &z) == 4 && key == k) {
            *a = x, *b = y, *c = z;
            found = true;
        }
    }
    std::fclose(f);
    return found;
}

static void cache_store(const std::string &key, int a, int b, int c)
{
    const char *path = std::getenv("GFFT_AUTOTUNE_CACHE");
    if (!path || !*path) return;
    FILE *f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d %d\n", key.c_str(), a, b, c);
    std::fclose(f);
}

double ragged_autotune(RaggedPlan &p, void *out, const void *in, cudaStream_t st, int *best_out)
{
    const std::string key = ragged_key(p);
    int a, b, c;
    if (cache_lookup(key, &a, &b, &c)) {
        p.lag_factor = a, p.ctas_per_sm = b, p.large_first = c;
        ragged_build_items(p);
        if (best_out) best_out[0] = a, best_out[1] = b, best_out[2] = c;
        return 0.0;
    }
    struct Cand {
        int lag, ctas, large_first;
    };
    std::vector<Cand> cands;
    for (int lg : {1, 2, 4})
        for (int ct : {0, 1})
            for (int lf : {1, 0}) cands.push_back({lg, ct, lf});
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    double best = 1e30;
    Cand bc = cands[0];
    for (const Cand &cd : cands) {
        p.lag_factor = cd.lag, p.ctas_per_sm = cd.ctas, p.large_first = cd.large_first;
        ragged_build_items(p);
        ragged_exec(p, 0, out, in, st, false);  // warm-up
        check_cuda(cudaEventRecord(e0, st), "event");
        for (int r = 0; r < 3; r++) ragged_exec(p, 0, out, in, st, false);
        check_cuda(cudaEventRecord(e1, st), "event");
        check_cuda(cudaEventSynchronize(e1), "sync");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms, bc = cd;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p.lag_factor = bc.lag, p.ctas_per_sm = bc.ctas, p.large_first = bc.large_first;
    ragged_build_items(p);
    cache_store(key, bc.lag, bc.ctas, bc.large_first);
    if (best_out) best_out[0] = bc.lag, best_out[1] = bc.ctas, best_out[2] = bc.large_first;
    return best / 3.0;
}

}  // namespace gfft
