// ragged.cu -- one persistent launch for a batch of transforms of uneven
// power-of-two sizes (fp32, n = 2^0 .. 2^18), packed back to back.
//
// The reference transforms one size per FFT<T> object (fft.h:56-113); a
// ragged batch there is a host loop over per-size plans.  Here a single
// persistent kernel walks a device work list:
//   SMALL (n <= 2^12): a run of same-size transforms, one thread group per
//          transform (the fused Stockham engine), many per CTA;
//   COL / ROW (n = 2^13 .. 2^18): the two tile passes of the four-step split
//          n = A * B; every tile is one item.  Column tiles write the
//          scratch, and a ROW item waits until all column tiles of its
//          transform are done (a per-transform counter; the wait is bounded
//          and reports a timeout instead of hanging).
// Items are claimed in list order through one atomic counter, so a ROW
// item only ever waits on COL items already claimed by running CTAs, which
// never wait: the schedule cannot deadlock.  Tiles use all 256 threads of a
// CTA (C = 4096 / L columns of L points, 32 KB of shared memory), so every
// global access comes in runs of at least 8 complex values.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"
#include "plan.h"
#include "tiles.cuh"
#include "tma.cuh"
#include "twiddle.h"

namespace gfft {

namespace rg {

constexpr int THREADS = 256;
constexpr int E = 16;              // points per thread
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
    int *counter;               // next item
    unsigned *err;
    const cpx<float> *tw;
    int nitems;
    Tables tab;
};

__host__ __device__ constexpr int split_a(int logn) { return logn / 2; }
__host__ __device__ constexpr int tile_c(int logl) { return THREADS * E >> logl; }  // columns per tile

// ---- SMALL: transforms of 2^LOGN points, THREADS / G per pass
template <int LOGN, bool INV>
__device__ void small_item(const Args &A, const Item &it, cpx<float> *sm)
{
    using SP = StockhamPlan<float, LOGN, E>;
    constexpr int G = SP::G, EE = SP::E;
    constexpr int TPP = THREADS / G;  // transforms per pass
    constexpr int SM = spad_size<float>(SP::N);
    const int g = threadIdx.x / G, t = threadIdx.x - g * G;
    const cpx<float> *tw = A.tw + A.tab.stock[LOGN];
    cpx<float> *my = sm + g * SM;
    for (int base = 0; base < it.b; base += TPP) {
        const int idx = base + g;
        const bool active = idx < it.b;
        const long long o = active ? A.off[A.perm[it.a + idx]] : 0;
        cpx<float> v[EE];
#pragma unroll
        for (int q = 0; q < EE; q++) v[q] = active ? ldcs_c(A.in + o + t + q * G) : cpx<float>{0.f, 0.f};
        stockham_run<float, LOGN, E, INV>(
            v, t, [my](int i) -> cpx<float> & { return my[spad<float>(i)]; }, tw, []() { __syncthreads(); });
        if (active) {
#pragma unroll
            for (int q = 0; q < EE; q++) stcs_c(A.out + o + t + q * G, v[q]);
        }
        __syncthreads();  // shared memory is reused by the next pass
    }
}

// ---- COL: tile `it.b` of the column pass of transform it.a
template <int LOGN, bool INV>
__device__ void col_item(const Args &A, const Item &it, cpx<float> *sm)
{
    constexpr int LA = split_a(LOGN), LB = LOGN - LA;
    constexpr long long B = 1LL << LB;
    using SP = StockhamPlan<float, LA, E>;
    constexpr int G = SP::G, C = tile_c(LA);
    constexpr int PITCH = tile_pitch<float>(SP::N, C);
    const int s = threadIdx.x % C, t = threadIdx.x / C;
    const long long col = (long long)it.b * C + s;
    const long long o = A.off[it.a], wo = A.wsoff[it.a];
    cpx<float> v[E];
    const cpx<float> *src = A.in + o + col + (long long)t * B;
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = ldcs_c(src + (long long)q * G * B);
    cpx<float> *my = sm + s * PITCH;
    stockham_run<float, LA, E, INV>(
        v, t, [my](int i) -> cpx<float> & { return my[spad<float>(i)]; }, A.tw + A.tab.stock[LA],
        []() { __syncthreads(); });
    constexpr unsigned nmask = (1u << LOGN) - 1u;
    constexpr int lo_bits = (LOGN + 1) / 2;
    const cpx<float> *tlo = A.tw + A.tab.lo[LOGN], *thi = A.tw + A.tab.hi[LOGN];
    cpx<float> *dst = A.ws + wo + col + (long long)t * B;
#pragma unroll
    for (int q = 0; q < E; q++) {
        const unsigned e = ((unsigned)col * (unsigned)(t + q * G)) & nmask;
        const cpx<float> w = cmul(ldg_c(thi + (e >> lo_bits)), ldg_c(tlo + (e & ((1u << lo_bits) - 1u))));
        st_c(dst + (long long)q * G * B, twmul<INV>(v[q], w));
        if ((q & 3) == 3) asm volatile("" ::: "memory");
    }
    // publish: every thread's stores are visible before the counter moves
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(A.col_done + it.a, 1);
}

// ---- ROW: tile `it.b` of the row pass of transform it.a (transposed store)
template <int LOGN, bool INV>
__device__ bool row_item(const Args &A, const Item &it, cpx<float> *sm, int *flag)
{
    constexpr int LA = split_a(LOGN), LB = LOGN - LA;
    constexpr long long Acount = 1LL << LA, B = 1LL << LB;
    constexpr int NCOL = (int)(B / tile_c(LA));  // column tiles per transform
    using SP = StockhamPlan<float, LB, E>;
    constexpr int G = SP::G, C = tile_c(LB);
    constexpr int ROW = SP::SMEM;
    // wait (bounded) until every column tile of this transform is stored
    if (threadIdx.x == 0) {
        const volatile int *cd = A.col_done + it.a;
        bool ok = *cd >= NCOL;
        if (!ok) {
            const unsigned long long t0 = global_ns();
            while (!(ok = (*cd >= NCOL)))
                if (global_ns() - t0 > TMA_WAIT_NS) break;
        }
        __threadfence();
        *flag = ok;
    }
    __syncthreads();
    if (!*flag) return false;
    const int s = threadIdx.x / G, t = threadIdx.x - s * G;
    const long long row0 = (long long)it.b * C;
    const long long o = A.off[it.a], wo = A.wsoff[it.a];
    cpx<float> v[E];
    const cpx<float> *src = A.ws + wo + (row0 + s) * B + t;
#pragma unroll
    for (int q = 0; q < E; q++) {
        const float2 f = __ldcg(reinterpret_cast<const float2 *>(src + q * G));  // L2, never a stale L1 line
        v[q] = cpx<float>{f.x, f.y};
    }
    cpx<float> *my = sm + s * ROW;
    stockham_run<float, LB, E, INV>(
        v, t, [my](int i) -> cpx<float> & { return my[spad<float>(i)]; }, A.tw + A.tab.stock[LB],
        []() { __syncthreads(); });
    __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) sm[spad<float>((t + q * G) * C + s)] = v[q];
    __syncthreads();
    cpx<float> *dst = A.out + o + row0;
#pragma unroll
    for (int m = 0; m < E; m++) {
        const int idx = threadIdx.x + m * THREADS;
        const int s2 = idx % C, k = idx / C;
        stcs_c(dst + s2 + (long long)k * Acount, sm[spad<float>(idx)]);
    }
    return true;
}

template <bool INV>
__global__ void __launch_bounds__(THREADS) k_ragged(Args A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<float> *sm = reinterpret_cast<cpx<float> *>(smem_raw);
    __shared__ int s_item, s_flag;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(A.counter, 1);
        __syncthreads();
        const int i = s_item;
        if (i >= A.nitems) break;
        const Item it = A.items[i];
        bool ok = true;
        switch (it.type) {
        case SMALL:
            switch (it.logn) {
#define S(L) case L: small_item<L, INV>(A, it, sm); break;
                S(0) S(1) S(2) S(3) S(4) S(5) S(6) S(7) S(8) S(9) S(10) S(11) S(12)
#undef S
            }
            break;
        case COL:
            switch (it.logn) {
#define S(L) case L: col_item<L, INV>(A, it, sm); break;
                S(13) S(14) S(15) S(16) S(17) S(18)
#undef S
            }
            break;
        default:
            switch (it.logn) {
#define S(L) case L: ok = row_item<L, INV>(A, it, sm, &s_flag); break;
                S(13) S(14) S(15) S(16) S(17) S(18)
#undef S
            }
            break;
        }
        if (!ok) {
            if (threadIdx.x == 0) atomicOr(A.err, DEV_ERR_TMA_TIMEOUT);
            break;
        }
        __syncthreads();  // s_item and shared memory are reused
    }
}

}  // namespace rg

// ---------------------------------------------------------------------------
// host side

namespace {

using rg::Item;

size_t ragged_smem()
{
    // the largest of: a pass of small transforms, a column tile, a row tile
    size_t m = 0;
    for (int l = 0; l <= rg::MAX_SMALL_LOGN; l++) {
        const int n = 1 << l, e = std::min(rg::E, n), g = n / e;
        m = std::max(m, (size_t)(rg::THREADS / g) * spad_size<float>(n));
    }
    for (int l = 6; l <= 9; l++) {
        const int c = rg::tile_c(l), n = 1 << l;
        m = std::max(m, (size_t)tile_pitch<float>(n, c) * c);
        m = std::max(m, (size_t)(n + n / 16) * c);
        m = std::max(m, (size_t)spad_size<float>(n * c));
    }
    return m * sizeof(cpx<float>);
}

}  // namespace

struct RaggedPlan {
    int device = 0;
    long long count = 0, total = 0;  // transforms, elements
    std::vector<int> logn;
    std::vector<long long> off;
    // tuning (autotuner-chosen)
    int passes_per_item = 4;  // SMALL items hold this many passes of a CTA
    int ctas_per_sm = 0;      // 0 = occupancy limit
    int large_first = 1;      // order large transforms before small ones
    // device state
    void *dev_items = nullptr, *dev_perm = nullptr, *dev_off = nullptr, *dev_wsoff = nullptr;
    int *dev_counters = nullptr;  // [0] item counter, [1..count] col_done
    void *ws = nullptr;
    size_t ws_bytes = 0;
    const void *tw = nullptr;
    rg::Tables tab{};
    int nitems = 0;
    int grid = 0;
    // captured graphs, keyed by (in, out, inverse)
    std::map<std::tuple<const void *, void *, int>, cudaGraphExec_t> graphs;
};

static void ragged_free_graphs(RaggedPlan &p)
{
    for (auto &kv : p.graphs) cudaGraphExecDestroy(kv.second);
    p.graphs.clear();
}

// (re)build the device work list for the current tuning parameters
static void ragged_build_items(RaggedPlan &p)
{
    std::vector<Item> items;
    std::vector<int> perm;
    // large transforms, biggest first: COL tiles of transform j interleaved
    // with the ROW tiles of transform j-1, so ROW items rarely wait
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
    for (size_t j = 0; j <= large.size(); j++) {
        if (j < large.size())
            for (int c = 0; c < cols(large[j]); c++) big.push_back({rg::COL, p.logn[large[j]], large[j], c});
        if (j > 0)
            for (int r = 0; r < rows(large[j - 1]); r++) big.push_back({rg::ROW, p.logn[large[j - 1]], large[j - 1], r});
    }
    // small transforms grouped by size, biggest first
    std::vector<Item> small;
    for (int l = rg::MAX_SMALL_LOGN; l >= 0; l--) {
        std::vector<int> ids;
        for (long long i = 0; i < p.count; i++)
            if (p.logn[i] == l) ids.push_back((int)i);
        if (ids.empty()) continue;
        const int n = 1 << l, e = std::min(rg::E, n), g = n / e;
        const int per = (rg::THREADS / g) * std::max(1, p.passes_per_item);
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
    if (items.empty()) items.push_back({rg::SMALL, 0, 0, 0});
    if (p.dev_items) cudaFree(p.dev_items);
    if (p.dev_perm) cudaFree(p.dev_perm);
    p.dev_items = p.dev_perm = nullptr;
    check_cuda(cudaMalloc(&p.dev_items, items.size() * sizeof(Item)), "cudaMalloc(items)");
    check_cuda(cudaMalloc(&p.dev_perm, perm.size() * sizeof(int)), "cudaMalloc(perm)");
    check_cuda(cudaMemcpy(p.dev_items, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice), "items");
    check_cuda(cudaMemcpy(p.dev_perm, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice), "perm");
    p.nitems = (int)items.size();
    // persistent grid
    int per_sm = 0;
    const size_t smem = ragged_smem();
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rg::k_ragged<false>, rg::THREADS, smem),
               "occupancy");
    if (p.ctas_per_sm > 0) per_sm = std::min(per_sm, p.ctas_per_sm);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p.device);
    p.grid = std::max(1, per_sm) * sms;
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
    check_cuda(cudaMalloc(&p->dev_counters, (count + 1) * sizeof(int)), "cudaMalloc(counters)");
    p->ws_bytes = (size_t)std::max<long long>(wpos, 1) * sizeof(cpx<float>);
    check_cuda(cudaMalloc(&p->ws, p->ws_bytes), "cudaMalloc(ragged scratch)");
    const size_t smem = ragged_smem();
    for (const void *fn : {(const void *)rg::k_ragged<false>, (const void *)rg::k_ragged<true>})
        check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem");
    device_error_word();  // allocate now: never inside a stream capture
    ragged_build_items(*p);
    return p.release();
}

void ragged_destroy(RaggedPlan *p)
{
    if (!p) return;
    ragged_free_graphs(*p);
    for (void *q : {p->dev_items, p->dev_perm, p->dev_off, p->dev_wsoff, (void *)p->dev_counters, p->ws})
        if (q) cudaFree(q);
    delete p;
}

long long ragged_total(const RaggedPlan *p) { return p->total; }

static void ragged_enqueue(RaggedPlan &p, int inverse, void *out, const void *in, cudaStream_t st)
{
    check_cuda(cudaMemsetAsync(p.dev_counters, 0, (p.count + 1) * sizeof(int), st), "reset counters");
    rg::Args a;
    a.in = static_cast<const cpx<float> *>(in);
    a.out = static_cast<cpx<float> *>(out);
    a.ws = static_cast<cpx<float> *>(p.ws);
    a.items = static_cast<const Item *>(p.dev_items);
    a.perm = static_cast<const int *>(p.dev_perm);
    a.off = static_cast<const long long *>(p.dev_off);
    a.wsoff = static_cast<const long long *>(p.dev_wsoff);
    a.counter = p.dev_counters;
    a.col_done = p.dev_counters + 1;
    a.err = device_error_word();
    a.tw = static_cast<const cpx<float> *>(p.tw);
    a.nitems = p.nitems;
    a.tab = p.tab;
    void *args[] = {&a};
    const void *fn = inverse ? (const void *)rg::k_ragged<true> : (const void *)rg::k_ragged<false>;
    check_cuda(cudaLaunchKernel(fn, dim3(p.grid), dim3(rg::THREADS), args, ragged_smem(), st), "launch ragged");
}

// One replay of the captured graph (counter reset + the persistent kernel);
// captured on first use for these pointers.
void ragged_exec(RaggedPlan &p, int inverse, void *out, const void *in, cudaStream_t st, bool use_graph)
{
    if (!in || !out) fail(GFFT_ERR_INVALID_VALUE, "NULL pointer");
    if (((uintptr_t)in | (uintptr_t)out) % 8) fail(GFFT_ERR_ALIGN, "pointers must be 8-byte aligned");
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
        p.passes_per_item = a, p.ctas_per_sm = b, p.large_first = c;
        ragged_build_items(p);
        if (best_out) best_out[0] = a, best_out[1] = b, best_out[2] = c;
        return 0.0;
    }
    struct Cand {
        int passes, ctas, large_first;
    };
    std::vector<Cand> cands;
    for (int ps : {1, 2, 4, 8})
        for (int ct : {0, 2})
            for (int lf : {1, 0}) cands.push_back({ps, ct, lf});
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    double best = 1e30;
    Cand bc = cands[0];
    for (const Cand &cd : cands) {
        p.passes_per_item = cd.passes, p.ctas_per_sm = cd.ctas, p.large_first = cd.large_first;
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
    p.passes_per_item = bc.passes, p.ctas_per_sm = bc.ctas, p.large_first = bc.large_first;
    ragged_build_items(p);
    cache_store(key, bc.passes, bc.ctas, bc.large_first);
    if (best_out) best_out[0] = bc.passes, best_out[1] = bc.ctas, best_out[2] = bc.large_first;
    return best / 3.0;
}

}  // namespace gfft
