// api.cpp -- the C ABI of libgenfft_gb300.so: validation, plans, the plan
// cache behind the reference-shaped entry points, twiddle-table cache and
// the host-buffer execution path.
//
// The reference has no C ABI; its backend seam is the factory functions
// backend::GetImpl / GetVertImpl / GetDITImpl (FFTBackend.h:15-45) that
// return cached per-size singletons (FFTLevel.h:51-60).  The plan cache here
// plays that role for the device kernels, with a mutex around creation
// (the reference's GetInstance is not thread-safe, FFTLevel.h:76-88).
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"
#include "tiles_registry.h"
#include "twiddle.h"

enum { ALGO_NONE = 0, ALGO_FUSED = 1, ALGO_FOURSTEP = 2 };

struct gfft_plan_s {
    gfft_desc d;
    int device = 0;
    int logn0 = 0, logn1 = 0;
    int algo = ALGO_NONE;
    const void *tw = nullptr; // fused: device twiddle table (cached, not owned)
    int launches = 0;
    // four-step (N = A * B): column pass over B columns of A points, row
    // pass over A rows of B points; `group` transforms per launch pair so
    // the intermediate (group * N elements) stays in L2
    int logA = 0, logB = 0;
    const gfft::TileKernel *kcol = nullptr, *krow = nullptr;
    int ccol = 0, crow = 0;
    const void *tw_col = nullptr, *tw_row = nullptr, *tw_lo = nullptr, *tw_hi = nullptr;
    int lo_bits = 0;
    long long group = 0;
    void *ws = nullptr;
    size_t ws_bytes = 0;
    unsigned magic = 0x6766u;
    // host-path staging (owned, lazily allocated)
    std::mutex host_mu;
    void *stage[3] = {nullptr, nullptr, nullptr};
    void *stage_out[3] = {nullptr, nullptr, nullptr};
    size_t stage_bytes_in = 0, stage_bytes_out = 0;
    cudaStream_t host_streams[3] = {nullptr, nullptr, nullptr};
};

namespace gfft {

namespace {
thread_local std::string g_last_error;

bool is_pow2(long long n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2ll(long long n)
{
    int l = 0;
    while ((1LL << l) < n) l++;
    return l;
}
size_t cplx_bytes(int dtype) { return dtype == GFFT_F64 ? 16 : 8; }
}  // namespace

void fail(gfft_status st, const std::string &msg) { throw Error{st, msg}; }

void check_cuda(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        cudaGetLastError();  // clear a non-sticky error
        fail(GFFT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

static void check_device()
{
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    static std::mutex mu;
    static std::map<int, bool> ok;
    std::lock_guard<std::mutex> lk(mu);
    auto it = ok.find(dev);
    if (it == ok.end()) {
        int major = 0, minor = 0;
        check_cuda(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev), "attr");
        check_cuda(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev), "attr");
        it = ok.emplace(dev, major == 10 && minor == 3).first;
    }
    if (!it->second) fail(GFFT_ERR_ARCH, "libgenfft_gb300 is built for sm_103a (GB300) only");
}

const void *cached_table(const std::string &key, int dtype, size_t count,
                         const std::function<void(void *)> &fill)
{
    static std::mutex mu;
    static std::map<std::pair<int, std::string>, void *> cache;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(mu);
    auto k = std::make_pair(dev, key);
    auto it = cache.find(k);
    if (it != cache.end()) return it->second;
    const size_t bytes = std::max<size_t>(count, 1) * cplx_bytes(dtype);
    std::vector<unsigned char> host(bytes, 0);
    if (count) fill(host.data());
    void *d = nullptr;
    check_cuda(cudaMalloc(&d, bytes), "cudaMalloc(twiddles)");
    cudaError_t e = cudaMemcpy(d, host.data(), bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        check_cuda(e, "cudaMemcpy(twiddles)");
    }
    cache.emplace(k, d);
    return d;
}

// ---------------------------------------------------------------------------
// planning

static void validate_desc(const gfft_desc &d)
{
    if (d.dtype != GFFT_F32 && d.dtype != GFFT_F64) fail(GFFT_ERR_INVALID_VALUE, "dtype must be GFFT_F32 or GFFT_F64");
    if (d.mode != GFFT_MODE_PLAIN) fail(GFFT_ERR_INVALID_VALUE, "unknown mode");
    if (d.batch < 1) fail(GFFT_ERR_INVALID_SIZE, "batch must be >= 1");
    if (!is_pow2(d.n0)) fail(GFFT_ERR_INVALID_SIZE, "size must be a power of two >= 1 (README.txt:10-11)");
    if (d.istride < 0 || d.ostride < 0 || d.idist < 0 || d.odist < 0)
        fail(GFFT_ERR_INVALID_VALUE, "strides and distances must be >= 0");
    if (d.flags & ~(unsigned)(GFFT_FLAG_HALF_SPECTRUM | GFFT_FLAG_BITREV_INPUT))
        fail(GFFT_ERR_INVALID_VALUE, "unknown flag bits");
}

static const void *tile_table(int dtype, const TileKernel *k, int logl, int c)
{
    return cached_table("tile/" + std::to_string(dtype) + "/" + std::to_string(logl) + "/" + std::to_string(c) +
                            "/" + std::to_string(k->threads),
                        dtype, k->twcount, [k](void *buf) { k->fill(buf); });
}

// W_N^e split as tw_hi[e >> lo_bits] * tw_lo[e & (2^lo_bits - 1)]
static void four_step_tables(gfft_plan_s &p, int logn)
{
    const int dtype = p.d.dtype;
    const int lo_bits = (logn + 1) / 2;
    const long long N = 1LL << logn;
    p.lo_bits = lo_bits;
    auto fill = [dtype, N](long long count, long long mul) {
        return [dtype, N, count, mul](void *buf) {
            for (long long e = 0; e < count; e++) {
                if (dtype == GFFT_F32) {
                    float *o = static_cast<float *>(buf);
                    forward_root<float>(e * mul, N, &o[2 * e], &o[2 * e + 1]);
                } else {
                    double *o = static_cast<double *>(buf);
                    forward_root<double>(e * mul, N, &o[2 * e], &o[2 * e + 1]);
                }
            }
        };
    };
    const std::string key = "4s/" + std::to_string(dtype) + "/" + std::to_string(logn);
    p.tw_lo = cached_table(key + "/lo", dtype, 1LL << lo_bits, fill(1LL << lo_bits, 1));
    p.tw_hi = cached_table(key + "/hi", dtype, N >> lo_bits, fill(N >> lo_bits, 1LL << lo_bits));
}

static long long env_ll(const char *name, long long dflt)
{
    const char *v = std::getenv(name);
    return (v && *v) ? std::atoll(v) : dflt;
}

static void plan_fourstep(gfft_plan_s &p, int logn)
{
    const gfft_desc &d = p.d;
    if (d.istride != 1 || d.ostride != 1)
        fail(GFFT_ERR_UNSUPPORTED, "sizes above the fused limit need unit element strides");
    if (logn > 24) fail(GFFT_ERR_INVALID_SIZE, "size above 2^24 is not supported");
    // A (column-FFT length) and B (row-FFT length), both at most 2^12
    p.logA = logn / 2;
    p.logB = logn - p.logA;
    const long long maxc = env_ll("GFFT_TILE_MAXC", 16);
    p.ccol = tile_widest(d.dtype, TILE_COL_TW4, p.logA, (int)maxc);
    p.crow = tile_widest(d.dtype, TILE_ROW_XPOSE, p.logB, (int)maxc);
    if (!p.ccol || !p.crow) fail(GFFT_ERR_UNSUPPORTED, "no tile kernel for this size");
    p.kcol = tile_find(d.dtype, TILE_COL_TW4, p.logA, p.ccol);
    p.krow = tile_find(d.dtype, TILE_ROW_XPOSE, p.logB, p.crow);
    p.tw_col = tile_table(d.dtype, p.kcol, p.logA, p.ccol);
    p.tw_row = tile_table(d.dtype, p.krow, p.logB, p.crow);
    four_step_tables(p, logn);
    // group so the intermediate fits comfortably in the 129 MB L2
    const long long N = 1LL << logn;
    const long long l2_budget = env_ll("GFFT_L2_BUDGET_MB", 48) << 20;
    p.group = std::max<long long>(1, l2_budget / (N * (long long)cplx_bytes(d.dtype)));
    p.group = std::min(p.group, std::max<long long>(1, d.batch));
    p.ws_bytes = (size_t)(p.group * N) * cplx_bytes(d.dtype);
    check_cuda(cudaMalloc(&p.ws, p.ws_bytes), "cudaMalloc(workspace)");
    p.algo = ALGO_FOURSTEP;
    p.launches = 2 * (int)((d.batch + p.group - 1) / p.group);
}

static void plan_c2c(gfft_plan_s &p)
{
    const gfft_desc &d = p.d;
    if (d.flags & GFFT_FLAG_BITREV_INPUT) fail(GFFT_ERR_UNSUPPORTED, "bit-reversed input not built yet");
    p.logn0 = ilog2ll(d.n0);
    if (p.logn0 <= fused_max_logn(d.dtype)) {
        const int logn = p.logn0, dtype = d.dtype;
        p.algo = ALGO_FUSED;
        p.launches = 1;
        p.tw = cached_table("fused/" + std::to_string(dtype) + "/" + std::to_string(logn), dtype,
                            fused_twiddle_count(dtype, logn),
                            [dtype, logn](void *buf) { fused_twiddle_fill(dtype, logn, buf); });
        return;
    }
    plan_fourstep(p, p.logn0);
}

static gfft_plan_s *make_plan(const gfft_desc &in)
{
    gfft_desc d = in;
    validate_desc(d);
    if (d.istride == 0) d.istride = 1;
    if (d.ostride == 0) d.ostride = 1;
    check_device();
    std::unique_ptr<gfft_plan_s> p(new gfft_plan_s());
    check_cuda(cudaGetDevice(&p->device), "cudaGetDevice");
    switch (d.kind) {
    case GFFT_KIND_C2C:
        if (d.idist == 0) d.idist = d.n0 * d.istride;
        if (d.odist == 0) d.odist = d.n0 * d.ostride;
        p->d = d;
        plan_c2c(*p);
        break;
    default:
        fail(GFFT_ERR_UNSUPPORTED, "transform kind not built yet");
    }
    return p.release();
}

static void check_ptr(const void *ptr, int dtype, const char *name)
{
    if (!ptr) fail(GFFT_ERR_INVALID_VALUE, std::string(name) + " is NULL");
    const uintptr_t a = dtype == GFFT_F64 ? 16 : 8;
    if ((uintptr_t)ptr % a) fail(GFFT_ERR_ALIGN, std::string(name) + " is not aligned to its complex element");
}

static void exec_plan(gfft_plan_s &p, int inverse, void *out, const void *in, cudaStream_t st,
                      long long batch_override = -1)
{
    const gfft_desc &d = p.d;
    check_ptr(in, d.dtype, "in");
    check_ptr(out, d.dtype, "out");
    const long long batch = batch_override >= 0 ? batch_override : d.batch;
    switch (p.algo) {
    case ALGO_FUSED: {
        FusedC2CArgs a{in, out, batch, d.idist, d.odist, d.istride, d.ostride, p.tw};
        check_cuda(launch_fused_c2c(d.dtype, p.logn0, inverse, a, st), "launch fused C2C");
        break;
    }
    case ALGO_FOURSTEP: {
        const long long A = 1LL << p.logA, B = 1LL << p.logB, N = A * B;
        const size_t eb = cplx_bytes(d.dtype);
        const unsigned nmask = (unsigned)(N - 1);
        for (long long g0 = 0; g0 < batch; g0 += p.group) {
            const long long nb = std::min(p.group, batch - g0);
            const char *src = static_cast<const char *>(in) + (size_t)(g0 * d.idist) * eb;
            char *dst = static_cast<char *>(out) + (size_t)(g0 * d.odist) * eb;
            // column pass: B columns of A points, stride B, into the workspace
            check_cuda(launch_colpass(*p.kcol, inverse, B / p.ccol, nb, src, p.ws, B, B, B, d.idist, N,
                                      p.tw_col, p.tw_lo, p.tw_hi, p.lo_bits, nmask, st),
                       "launch column pass");
            // row pass: A rows of B points, stored transposed (stride A)
            check_cuda(launch_rowpass(*p.krow, inverse, A / p.crow, nb, p.ws, dst, A, B, A, N, d.odist,
                                      p.tw_row, st),
                       "launch row pass");
        }
        break;
    }
    default:
        fail(GFFT_ERR_INVALID_PLAN, "plan has no algorithm");
    }
}

// bytes of one transform's input / output, for host staging (dense plans)
static void io_bytes(const gfft_plan_s &p, size_t *ib, size_t *ob)
{
    const gfft_desc &d = p.d;
    *ib = (size_t)d.idist * cplx_bytes(d.dtype);
    *ob = (size_t)d.odist * cplx_bytes(d.dtype);
}

static void exec_host(gfft_plan_s &p, int inverse, void *out, const void *in)
{
    const gfft_desc &d = p.d;
    if (!in || !out) fail(GFFT_ERR_INVALID_VALUE, "NULL host buffer");
    if (d.istride != 1 || d.ostride != 1 || d.idist != d.n0 || d.odist != d.n0)
        fail(GFFT_ERR_UNSUPPORTED, "host execution needs dense batches");
    std::lock_guard<std::mutex> lk(p.host_mu);
    size_t ib, ob;
    io_bytes(p, &ib, &ob);
    // chunks of about 64 MB, at least one transform
    long long per = std::max<long long>(1, (long long)((64u << 20) / std::max<size_t>(ib, 1)));
    per = std::min(per, d.batch);
    if (!p.stage[0] || p.stage_bytes_in < per * ib || p.stage_bytes_out < per * ob) {
        for (int i = 0; i < 3; i++) {
            if (p.stage[i]) cudaFree(p.stage[i]);
            if (p.stage_out[i]) cudaFree(p.stage_out[i]);
            p.stage[i] = p.stage_out[i] = nullptr;
        }
        for (int i = 0; i < 3; i++) {
            check_cuda(cudaMalloc(&p.stage[i], per * ib), "cudaMalloc(stage)");
            check_cuda(cudaMalloc(&p.stage_out[i], per * ob), "cudaMalloc(stage)");
            if (!p.host_streams[i])
                check_cuda(cudaStreamCreateWithFlags(&p.host_streams[i], cudaStreamNonBlocking), "stream");
        }
        p.stage_bytes_in = per * ib;
        p.stage_bytes_out = per * ob;
    }
    const unsigned char *hin = static_cast<const unsigned char *>(in);
    unsigned char *hout = static_cast<unsigned char *>(out);
    int c = 0;
    for (long long b0 = 0; b0 < d.batch; b0 += per, c++) {
        const long long nb = std::min(per, d.batch - b0);
        const int s = c % 3;
        cudaStream_t st = p.host_streams[s];
        check_cuda(cudaMemcpyAsync(p.stage[s], hin + b0 * ib, nb * ib, cudaMemcpyHostToDevice, st), "H2D");
        exec_plan(p, inverse, p.stage_out[s], p.stage[s], st, nb);
        check_cuda(cudaMemcpyAsync(hout + b0 * ob, p.stage_out[s], nb * ob, cudaMemcpyDeviceToHost, st), "D2H");
    }
    for (int i = 0; i < 3; i++) check_cuda(cudaStreamSynchronize(p.host_streams[i]), "sync");
}

// cache of plans for the reference-shaped entry points: one per
// (device, kind, dtype, n0, n1, flags); batch and pointers are per call
static gfft_plan_s *cached_plan(int kind, int dtype, long long n0, long long n1, unsigned flags)
{
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, long long, long long, unsigned>, gfft_plan_s *> cache;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_tuple(dev, kind, dtype, n0, n1, flags);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    gfft_desc d;
    std::memset(&d, 0, sizeof d);
    d.kind = kind;
    d.dtype = dtype;
    d.mode = GFFT_MODE_PLAIN;
    d.flags = flags;
    d.n0 = n0;
    d.n1 = n1;
    d.batch = 1 << 20;  // sizes the workspace for full groups; the batch is per call
    gfft_plan_s *p = make_plan(d);
    cache.emplace(key, p);
    return p;
}

}  // namespace gfft

using namespace gfft;

#define GFFT_GUARD(body)                                               \
    try {                                                              \
        body;                                                          \
        return GFFT_OK;                                                \
    } catch (const Error &e) {                                         \
        g_last_error = e.msg;                                          \
        return e.status;                                               \
    } catch (const std::bad_alloc &) {                                 \
        g_last_error = "host allocation failed";                       \
        return GFFT_ERR_ALLOC;                                         \
    } catch (...) {                                                    \
        g_last_error = "unexpected exception";                         \
        return GFFT_ERR_INVALID_VALUE;                                 \
    }

static gfft_plan_s *checked(gfft_plan p)
{
    if (!p || p->magic != 0x6766u) fail(GFFT_ERR_INVALID_PLAN, "invalid plan handle");
    return p;
}

extern "C" {

gfft_status gfft_plan_create(gfft_plan *plan, const gfft_desc *desc)
{
    GFFT_GUARD({
        if (!plan || !desc) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        *plan = nullptr;
        *plan = make_plan(*desc);
    });
}

gfft_status gfft_plan_destroy(gfft_plan plan)
{
    GFFT_GUARD({
        gfft_plan_s *p = checked(plan);
        for (int i = 0; i < 3; i++) {
            if (p->stage[i]) cudaFree(p->stage[i]);
            if (p->stage_out[i]) cudaFree(p->stage_out[i]);
            if (p->host_streams[i]) cudaStreamDestroy(p->host_streams[i]);
        }
        if (p->ws) cudaFree(p->ws);
        p->magic = 0;
        delete p;
    });
}

gfft_status gfft_exec(gfft_plan plan, int inverse, void *out, const void *in, void *stream)
{
    GFFT_GUARD({ exec_plan(*checked(plan), inverse != 0, out, in, (cudaStream_t)stream); });
}

gfft_status gfft_exec_host(gfft_plan plan, int inverse, void *out, const void *in)
{
    GFFT_GUARD({ exec_host(*checked(plan), inverse != 0, out, in); });
}

gfft_status gfft_plan_launches(gfft_plan plan, int *launches)
{
    GFFT_GUARD({
        if (!launches) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        *launches = checked(plan)->launches;
    });
}

gfft_status gfft_fft_transform(int dtype, int n, long long batch, int inverse, void *out,
                               const void *in, void *stream)
{
    GFFT_GUARD({
        if (batch < 1) fail(GFFT_ERR_INVALID_SIZE, "batch must be >= 1");
        gfft_plan_s *p = cached_plan(GFFT_KIND_C2C, dtype, n, 0, 0);
        exec_plan(*p, inverse != 0, out, in, (cudaStream_t)stream, batch);
    });
}

const char *gfft_status_string(gfft_status s)
{
    switch (s) {
    case GFFT_OK: return "success";
    case GFFT_ERR_INVALID_SIZE: return "invalid size";
    case GFFT_ERR_INVALID_VALUE: return "invalid value";
    case GFFT_ERR_ALIAS: return "output aliases input";
    case GFFT_ERR_ALIGN: return "misaligned pointer";
    case GFFT_ERR_ARCH: return "unsupported device architecture";
    case GFFT_ERR_CUDA: return "CUDA error";
    case GFFT_ERR_TIMEOUT: return "device wait timed out";
    case GFFT_ERR_UNSUPPORTED: return "unsupported";
    case GFFT_ERR_ALLOC: return "allocation failed";
    case GFFT_ERR_INVALID_PLAN: return "invalid plan";
    }
    return "unknown status";
}

const char *gfft_last_error(void) { return g_last_error.c_str(); }

int gfft_version(void) { return GFFT_VERSION; }

int gfft_max_fused_size(int dtype)
{
    if (dtype != GFFT_F32 && dtype != GFFT_F64) return 0;
    return 1 << fused_max_logn(dtype);
}

}  // extern "C"
