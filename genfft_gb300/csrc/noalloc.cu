// noalloc.cu -- an fp32 C2C entry point that allocates no memory.
//
// gfft_fft_transform_noalloc runs the same four-step column + row passes as
// gfft_fft_transform for lengths above the fused single-kernel limit, but
// its scratch (the intermediate between the two passes) and its twiddle
// tables live in file-scope __device__ arrays of fixed size instead of
// cudaMalloc'd buffers.  It is meant for callers that cannot allocate
// device memory at the point they run a transform: code whose device memory
// is owned and budgeted by someone else (a framework's caching allocator or
// a fixed memory pool), or latency-sensitive loops where a cudaMalloc would
// synchronise the device.  The price: every GPU that loads this library
// holds the arrays (32 MiB of scratch plus about 0.3 MiB of tables) until
// the process exits.
//
// Set-up: the first call on each device, with that device current, takes
// the arrays' device addresses with cudaGetSymbolAddress, fills the twiddle
// tables with cudaMemcpy (synchronous) and raises the kernels' shared-memory
// limit.  Make that first call before any stream capture.  Later calls
// only enqueue kernels.
//
// All calls share the one scratch array: calls whose kernels can overlap on
// the GPU (different streams without ordering between them) race on it and
// must be serialised by the caller.  Nothing needs clearing between calls:
// the column pass writes every scratch element the row pass then reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "internal.h"
#include "plan.h"
#include "stockham.cuh"
#include "twiddle.h"

namespace gfft {
namespace {

constexpr int NA_MIN_LOGN = 15;  // first length above the fp32 fused limit
constexpr int NA_MAX_LOGN = 22;  // the scratch holds one 2^22-point transform
constexpr long long NA_SCRATCH = 1LL << NA_MAX_LOGN;  // complex fp32 elements (32 MiB)
constexpr int NA_MIN_L = NA_MIN_LOGN / 2;              // tile lengths used by the split
constexpr int NA_MAX_L = NA_MAX_LOGN - NA_MAX_LOGN / 2;

constexpr int split_lo(int logn) { return (logn + 1) / 2; }

// twiddle layout: Stockham tables of the tile lengths NA_MIN_L..NA_MAX_L
// (E = 16 points per thread, as registered for fp32), then the four-step
// split tables (lo, hi) of every length NA_MIN_LOGN..NA_MAX_LOGN
constexpr int stockham_tw(int logl)
{
    return logl == 7 ? StockhamPlan<float, 7, 16>::TW
         : logl == 8 ? StockhamPlan<float, 8, 16>::TW
         : logl == 9 ? StockhamPlan<float, 9, 16>::TW
         : logl == 10 ? StockhamPlan<float, 10, 16>::TW
                      : StockhamPlan<float, 11, 16>::TW;
}
constexpr long long tw_total()
{
    long long t = 0;
    for (int l = NA_MIN_L; l <= NA_MAX_L; l++) t += stockham_tw(l);
    for (int n = NA_MIN_LOGN; n <= NA_MAX_LOGN; n++) t += (1LL << split_lo(n)) + (1LL << (n - split_lo(n)));
    return t;
}
constexpr long long NA_TW = tw_total();

static __device__ __align__(256) cpx<float> g_noalloc_scratch[NA_SCRATCH];
static __device__ __align__(256) cpx<float> g_noalloc_tw[NA_TW];

struct Setup {
    bool ready = false;
    cpx<float> *scratch = nullptr;        // device address of g_noalloc_scratch
    cpx<float> *tw = nullptr;             // device address of g_noalloc_tw
    long long stock_off[NA_MAX_L + 1] = {};
    long long lo_off[NA_MAX_LOGN + 1] = {}, hi_off[NA_MAX_LOGN + 1] = {};
    const TileKernel *kcol[NA_MAX_LOGN + 1] = {}, *krow[NA_MAX_LOGN + 1] = {};
    int ccol[NA_MAX_LOGN + 1] = {}, crow[NA_MAX_LOGN + 1] = {};
};

constexpr int NA_MAX_DEVICES = 64;
Setup g_setup[NA_MAX_DEVICES];
std::mutex g_setup_mu;

void setup_device(int dev, Setup &s)
{
    void *p = nullptr;
    check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
    s.scratch = static_cast<cpx<float> *>(p);
    check_cuda(cudaGetSymbolAddress(&p, g_noalloc_tw), "cudaGetSymbolAddress(twiddles)");
    s.tw = static_cast<cpx<float> *>(p);

    std::vector<cpx<float>> host((size_t)NA_TW);
    long long off = 0;
    for (int l = NA_MIN_L; l <= NA_MAX_L; l++) {
        s.stock_off[l] = off;
        const TileKernel *k = tile_find(GFFT_F32, TILE_ROW_XPOSE, l, tile_widest(GFFT_F32, TILE_ROW_XPOSE, l, 16));
        if (!k || (long long)k->twcount != stockham_tw(l)) fail(GFFT_ERR_UNSUPPORTED, "tile table mismatch");
        k->fill(host.data() + off);
        off += stockham_tw(l);
    }
    for (int n = NA_MIN_LOGN; n <= NA_MAX_LOGN; n++) {
        const long long N = 1LL << n;
        const int lo = split_lo(n);
        s.lo_off[n] = off;
        for (long long e = 0; e < (1LL << lo); e++) forward_root<float>(e, N, &host[off + e].x, &host[off + e].y);
        off += 1LL << lo;
        s.hi_off[n] = off;
        for (long long e = 0; e < (N >> lo); e++)
            forward_root<float>(e << lo, N, &host[off + e].x, &host[off + e].y);
        off += N >> lo;
        const int la = n / 2, lb = n - la;
        s.ccol[n] = tile_widest(GFFT_F32, TILE_COL_TW4, la, 16);
        s.crow[n] = tile_widest(GFFT_F32, TILE_ROW_XPOSE, lb, 16);
        s.kcol[n] = tile_find(GFFT_F32, TILE_COL_TW4, la, s.ccol[n]);
        s.krow[n] = tile_find(GFFT_F32, TILE_ROW_XPOSE, lb, s.crow[n]);
        if (!s.kcol[n] || !s.krow[n]) fail(GFFT_ERR_UNSUPPORTED, "no tile kernel");
        // tile kernels of the same length must share one Stockham table:
        // the column kernel's own table must equal the one stored for la
        if ((long long)s.kcol[n]->twcount != stockham_tw(la)) fail(GFFT_ERR_UNSUPPORTED, "tile table mismatch");
        std::vector<cpx<float>> mine((size_t)stockham_tw(la));
        s.kcol[n]->fill(mine.data());
        if (std::memcmp(mine.data(), host.data() + s.stock_off[la], mine.size() * sizeof(cpx<float>)) != 0)
            fail(GFFT_ERR_UNSUPPORTED, "tile table mismatch");
        for (const TileKernel *k : {s.kcol[n], s.krow[n]})
            for (const void *fn : {k->fwd, k->inv})
                if (k->smem > 48 * 1024)
                    check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k->smem),
                               "cudaFuncSetAttribute");
    }
    check_cuda(cudaMemcpy(s.tw, host.data(), sizeof(cpx<float>) * (size_t)NA_TW, cudaMemcpyHostToDevice),
               "cudaMemcpy(twiddles)");
    (void)dev;
    s.ready = true;
}

}  // namespace
}  // namespace gfft

using namespace gfft;

extern "C" gfft_status gfft_fft_transform_noalloc(int dtype, int n, long long batch, int inverse, void *out,
                                                  const void *in, void *stream)
{
    try {
        if (dtype != GFFT_F32) fail(GFFT_ERR_UNSUPPORTED, "the allocation-free transform is fp32 only");
        if (!is_pow2(n) || n < (1 << NA_MIN_LOGN) || n > (1 << NA_MAX_LOGN))
            fail(GFFT_ERR_INVALID_SIZE,
                 "the allocation-free transform takes n = 2^15 .. 2^22 (its 32 MiB scratch holds one "
                 "2^22-point transform); smaller sizes need no scratch, use gfft_fft_transform");
        if (batch < 1) fail(GFFT_ERR_INVALID_SIZE, "batch must be >= 1");
        if (!in || !out) fail(GFFT_ERR_INVALID_VALUE, "NULL pointer");
        if (((uintptr_t)in | (uintptr_t)out) % 8) fail(GFFT_ERR_ALIGN, "pointers must be 8-byte aligned");
        check_device();
        int dev = 0;
        check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        if (dev < 0 || dev >= NA_MAX_DEVICES) fail(GFFT_ERR_UNSUPPORTED, "device ordinal out of range");
        Setup &s = g_setup[dev];
        {
            std::lock_guard<std::mutex> lk(g_setup_mu);
            if (!s.ready) setup_device(dev, s);
        }
        const int logn = ilog2ll(n);
        const long long A = 1LL << (logn / 2), B = (long long)n / A, N = n;
        const int lo = split_lo(logn);
        const unsigned nmask = (unsigned)(N - 1);
        const cpx<float> *tw_col = s.tw + s.stock_off[logn / 2];
        const cpx<float> *tw_row = s.tw + s.stock_off[logn - logn / 2];
        const cpx<float> *tw_lo = s.tw + s.lo_off[logn], *tw_hi = s.tw + s.hi_off[logn];
        const TileKernel &kc = *s.kcol[logn], &kr = *s.krow[logn];
        const void *fc = inverse ? kc.inv : kc.fwd, *fr = inverse ? kr.inv : kr.fwd;
        const long long group = NA_SCRATCH / N;
        cudaStream_t st = (cudaStream_t)stream;
        for (long long g0 = 0; g0 < batch; g0 += group) {
            const long long nb = std::min(group, batch - g0);
            const cpx<float> *src = static_cast<const cpx<float> *>(in) + g0 * N;
            cpx<float> *dst = static_cast<cpx<float> *>(out) + g0 * N;
            cpx<float> *ws = s.scratch;
            long long ncols = B, ld_in = B, ld_out = B, idist = N, odist = N;
            int lob = lo;
            unsigned nm = nmask;
            float one = 1.0f;
            void *cargs[] = {&src, &ws, &ncols, &ld_in, &ld_out, &idist, &odist, &tw_col, &tw_lo, &tw_hi, &lob, &nm,
                             &one};
            check_cuda(cudaLaunchKernel(fc, dim3((unsigned)(B / s.ccol[logn]), (unsigned)nb), dim3(kc.threads), cargs,
                                        kc.smem, st),
                       "launch column pass");
            long long nrows = A, rld = B, ostride = A, ridist = N, rodist = N;
            const cpx<float> *wsc = ws;
            void *rargs[] = {&wsc, &dst, &nrows, &rld, &ostride, &ridist, &rodist, &tw_row, &one};
            check_cuda(cudaLaunchKernel(fr, dim3((unsigned)(A / s.crow[logn]), (unsigned)nb), dim3(kr.threads), rargs,
                                        kr.smem, st),
                       "launch row pass");
        }
        return GFFT_OK;
    } catch (const Error &e) {
        set_last_error(e.msg.c_str());
        return e.status;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return GFFT_ERR_ALLOC;
    } catch (...) {
        set_last_error("unexpected exception");
        return GFFT_ERR_INVALID_VALUE;
    }
}
