// api.cpp -- the C ABI of libgenfft_gb300.so: validation, plan creation per
// gfft_kind, execution, the plan cache behind the reference-shaped entry
// points, the twiddle-table cache and the host-buffer path.
//
// The reference has no C ABI; its backend seam is the factory functions
// backend::GetImpl / GetVertImpl / GetDITImpl (FFTBackend.h:15-45) that
// return cached per-size singletons (FFTLevel.h:51-60).  The plan cache here
// plays that role for the device kernels, with a mutex around creation
// (the reference's GetInstance is not thread-safe, FFTLevel.h:76-88).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"
#include "plan.h"

namespace gfft {

namespace {
thread_local std::string g_last_error;
}

void fail(gfft_status st, const std::string &msg) { throw Error{st, msg}; }

void set_last_error(const char *msg) { g_last_error = msg; }

void check_cuda(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        cudaGetLastError();  // clear a non-sticky error
        fail(GFFT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

void check_device()
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

const void *cached_table(const std::string &key, int dtype, size_t count, const std::function<void(void *)> &fill)
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

static size_t real_bytes(int dtype) { return dtype == GFFT_F64 ? 8 : 4; }

static void validate_desc(const gfft_desc &d)
{
    if (d.kind < GFFT_KIND_C2C || d.kind > GFFT_KIND_VERT) fail(GFFT_ERR_INVALID_VALUE, "unknown transform kind");
    if (d.dtype != GFFT_F32 && d.dtype != GFFT_F64) fail(GFFT_ERR_INVALID_VALUE, "dtype must be GFFT_F32 or GFFT_F64");
    if (d.mode != GFFT_MODE_PLAIN && d.mode != GFFT_MODE_TC_FP16 && d.mode != GFFT_MODE_TC_BF16)
        fail(GFFT_ERR_INVALID_VALUE, "unknown mode");
    if (d.mode != GFFT_MODE_PLAIN) {
        if (d.kind != GFFT_KIND_C2C || d.dtype != GFFT_F32 || (d.flags & GFFT_FLAG_BITREV_INPUT))
            fail(GFFT_ERR_UNSUPPORTED, "tensor-core modes cover fp32 C2C in natural order");
        if (d.n0 != 256 && d.n0 != 4096 && d.n0 != 65536)
            fail(GFFT_ERR_UNSUPPORTED, "tensor-core modes cover n = 256, 4096 and 65536");
    }
    if (d.batch < 1) fail(GFFT_ERR_INVALID_SIZE, "batch must be >= 1");
    if (!is_pow2(d.n0)) fail(GFFT_ERR_INVALID_SIZE, "size must be a power of two >= 1 (README.txt:10-11)");
    if (d.kind == GFFT_KIND_C2C_2D || d.kind == GFFT_KIND_R2C_2D) {
        if (!is_pow2(d.n1)) fail(GFFT_ERR_INVALID_SIZE, "2D height must be a power of two >= 1");
    } else if (d.kind == GFFT_KIND_VERT) {
        if (d.n1 < 1) fail(GFFT_ERR_INVALID_SIZE, "column count must be >= 1");
    }
    if (d.n0 > (1LL << 26) || d.n1 > (1LL << 26)) fail(GFFT_ERR_INVALID_SIZE, "size above 2^26");
    if (d.istride < 0 || d.ostride < 0 || d.idist < 0 || d.odist < 0)
        fail(GFFT_ERR_INVALID_VALUE, "strides and distances must be >= 0");
    const unsigned known = GFFT_FLAG_HALF_SPECTRUM | GFFT_FLAG_BITREV_INPUT;
    if (d.flags & ~known) fail(GFFT_ERR_INVALID_VALUE, "unknown flag bits");
    if ((d.flags & GFFT_FLAG_HALF_SPECTRUM) && d.kind != GFFT_KIND_R2C && d.kind != GFFT_KIND_R2C_2D)
        fail(GFFT_ERR_INVALID_VALUE, "GFFT_FLAG_HALF_SPECTRUM applies to real-input kinds only");
    if ((d.flags & GFFT_FLAG_BITREV_INPUT) && d.kind != GFFT_KIND_C2C && d.kind != GFFT_KIND_VERT)
        fail(GFFT_ERR_INVALID_VALUE, "GFFT_FLAG_BITREV_INPUT applies to C2C and VERT only");
}

// fill in default strides/distances (all in elements of the array's type)
static void apply_defaults(gfft_desc &d)
{
    const bool half = (d.flags & GFFT_FLAG_HALF_SPECTRUM) != 0;
    switch (d.kind) {
    case GFFT_KIND_C2C:
        if (!d.istride) d.istride = 1;
        if (!d.ostride) d.ostride = 1;
        if (!d.idist) d.idist = d.n0 * d.istride;
        if (!d.odist) d.odist = d.n0 * d.ostride;
        break;
    case GFFT_KIND_R2C:
        d.istride = d.ostride = 1;
        if (!d.idist) d.idist = d.n0;
        if (!d.odist) d.odist = half ? d.n0 / 2 + 1 : d.n0;
        break;
    case GFFT_KIND_C2C_2D:  // istride/ostride are row strides
        if (!d.istride) d.istride = d.n0;
        if (!d.ostride) d.ostride = d.n0;
        if (!d.idist) d.idist = d.n1 * d.istride;
        if (!d.odist) d.odist = d.n1 * d.ostride;
        break;
    case GFFT_KIND_R2C_2D:
        if (!d.istride) d.istride = d.n0;
        if (!d.ostride) d.ostride = half ? d.n0 / 2 + 1 : d.n0;
        if (!d.idist) d.idist = d.n1 * d.istride;
        if (!d.odist) d.odist = d.n1 * d.ostride;
        break;
    case GFFT_KIND_VERT:  // n0 rows, n1 columns, row strides
        if (!d.istride) d.istride = d.n1;
        if (!d.ostride) d.ostride = d.n1;
        if (!d.idist) d.idist = d.n0 * d.istride;
        if (!d.odist) d.odist = d.n0 * d.ostride;
        break;
    }
}

static void check_layout(const gfft_desc &d)
{
    const bool half = (d.flags & GFFT_FLAG_HALF_SPECTRUM) != 0;
    switch (d.kind) {
    case GFFT_KIND_R2C:
        if (d.n0 > 1 && (d.idist % 2)) fail(GFFT_ERR_INVALID_VALUE, "R2C input distance must be even");
        if (d.odist < (half ? d.n0 / 2 + 1 : d.n0)) fail(GFFT_ERR_INVALID_VALUE, "R2C output distance too small");
        break;
    case GFFT_KIND_C2C_2D:
        if (d.istride < d.n0 || d.ostride < d.n0) fail(GFFT_ERR_INVALID_VALUE, "2D row stride below the width");
        break;
    case GFFT_KIND_R2C_2D:
        if (d.n0 > 1 && (d.istride % 2)) fail(GFFT_ERR_INVALID_VALUE, "real 2D input row stride must be even");
        if (d.istride < d.n0) fail(GFFT_ERR_INVALID_VALUE, "2D row stride below the width");
        if (d.ostride < (half ? d.n0 / 2 + 1 : d.n0)) fail(GFFT_ERR_INVALID_VALUE, "2D output row stride too small");
        break;
    case GFFT_KIND_VERT:
        if (d.istride < d.n1 || d.ostride < d.n1) fail(GFFT_ERR_INVALID_VALUE, "row stride below the column count");
        break;
    default:
        break;
    }
}

// a profiler range for the lifetime of a scope (NVTX v3, header-only)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

static gfft_plan_s *make_plan(const gfft_desc &in)
{
    NvtxRange range("gfft plan create");
    gfft_desc d = in;
    validate_desc(d);
    apply_defaults(d);
    check_layout(d);
    check_device();
    std::unique_ptr<gfft_plan_s> p(new gfft_plan_s());
    check_cuda(cudaGetDevice(&p->device), "cudaGetDevice");
    p->d = d;
    const bool half = (d.flags & GFFT_FLAG_HALF_SPECTRUM) != 0;
    const bool bitrev = (d.flags & GFFT_FLAG_BITREV_INPUT) != 0;
    try {
        switch (d.kind) {
        case GFFT_KIND_C2C:
            if (d.mode != GFFT_MODE_PLAIN) {
                p->tc.init(d.mode, ilog2ll(d.n0), d.batch);
                p->launches = p->tc.launches(d.batch);
                break;
            }
            p->c2c.init(d.dtype, ilog2ll(d.n0), d.batch);
            p->launches = p->c2c.launches(d.batch) + (bitrev ? 1 : 0);
            break;
        case GFFT_KIND_R2C:
            p->r2c.init(d.dtype, ilog2ll(d.n0), half ? 1 : 0, d.batch);
            p->c2r.init(d.dtype, ilog2ll(d.n0), d.batch);
            p->launches = p->r2c.launches(d.batch);
            p->launches_inv = p->c2r.launches(d.batch);
            break;
        case GFFT_KIND_C2C_2D:
            p->c2c.init(d.dtype, ilog2ll(d.n0), d.batch * d.n1);
            p->col.init(d.dtype, ilog2ll(d.n1), TILE_COL_PLAIN, true, d.n0);
            p->launches = p->c2c.launches(d.batch * d.n1) + (int)p->col.launches(d.n0, d.batch);
            break;
        case GFFT_KIND_R2C_2D:
            p->r2c.init(d.dtype, ilog2ll(d.n0), 1, d.batch * d.n1);
            p->col.init(d.dtype, ilog2ll(d.n1), half ? TILE_COL_PLAIN : TILE_COL_HERM, false, d.n0 / 2 + 1);
            p->launches = p->r2c.launches(d.batch * d.n1) + (int)p->col.launches(d.n0 / 2 + 1, d.batch);
            break;
        case GFFT_KIND_VERT:
            p->col.init(d.dtype, ilog2ll(d.n0), bitrev ? TILE_COL_BITREV : TILE_COL_PLAIN, true, d.n1);
            p->launches = (int)p->col.launches(d.n1, d.batch);
            break;
        }
        if (d.kind != GFFT_KIND_R2C) p->launches_inv = p->launches;
    } catch (...) {
        p->c2c.release();
        p->r2c.release();
        p->c2r.release();
        p->tc.release();
        p->col.release();
        throw;
    }
    return p.release();
}

static void check_ptr(const void *ptr, size_t align, const char *name)
{
    if (!ptr) fail(GFFT_ERR_INVALID_VALUE, std::string(name) + " is NULL");
    if ((uintptr_t)ptr % align) fail(GFFT_ERR_ALIGN, std::string(name) + " is not aligned to its element type");
}

// per-call layout (reference-shaped entry points override the plan's)
struct Layout {
    long long batch, istride, idist, ostride, odist;
};

static Layout plan_layout(const gfft_plan_s &p)
{
    return Layout{p.d.batch, p.d.istride, p.d.idist, p.d.ostride, p.d.odist};
}

static bool overlaps(const void *a, size_t an, const void *b, size_t bn)
{
    const char *x = static_cast<const char *>(a), *y = static_cast<const char *>(b);
    return x < y + bn && y < x + an;
}

// `scale` multiplies every output (norm= scaling), applied by the kernel
// that writes the result
static void exec_body(gfft_plan_s &p, int inverse, void *out, const void *in, const Layout &L, cudaStream_t st,
                      double scale)
{
    const gfft_desc &d = p.d;
    const size_t cb = cplx_bytes(d.dtype), rb = real_bytes(d.dtype);
    const bool real_in = (d.kind == GFFT_KIND_R2C && !inverse) || d.kind == GFFT_KIND_R2C_2D;
    const bool real_out = d.kind == GFFT_KIND_R2C && inverse;
    check_ptr(in, real_in ? rb : cb, "in");
    check_ptr(out, real_out ? rb : cb, "out");
    switch (d.kind) {
    case GFFT_KIND_C2C:
        if (d.flags & GFFT_FLAG_BITREV_INPUT) {
            // transform_no_scramble (fft.h:69-73): permute to natural order in
            // the output buffer, then transform in place
            if (L.istride != 1 || L.ostride != 1 || L.idist != L.odist)
                fail(GFFT_ERR_UNSUPPORTED, "bit-reversed input needs dense batches");
            if (out != in)
                check_cuda(cudaMemcpyAsync(out, in, (size_t)(L.batch * L.idist) * cb, cudaMemcpyDeviceToDevice, st),
                           "copy");
            check_cuda(launch_bitrev_swap(d.dtype, out, p.c2c.logn, L.batch, L.odist, st), "bit reversal");
            p.c2c.run(inverse, out, out, L.batch, L.odist, L.odist, 1, 1, st, scale);
        } else if (d.mode != GFFT_MODE_PLAIN) {
            p.tc.run(inverse, in, out, L.batch, L.idist, L.odist, L.istride, L.ostride, st, scale);
        } else {
            p.c2c.run(inverse, in, out, L.batch, L.idist, L.odist, L.istride, L.ostride, st, scale);
        }
        break;
    case GFFT_KIND_R2C: {
        if (inverse) {
            // half-spectrum inverse: the plan's output layout is the input
            // (bins), its input layout the output (reals); unscaled
            if (overlaps(in, (size_t)(L.batch * L.odist) * cb, out, (size_t)(L.batch * L.idist) * rb))
                fail(GFFT_ERR_ALIAS, "half-spectrum inverse: output must not overlap the input");
            p.c2r.run(in, out, L.batch, L.odist, L.idist, 0, st, scale);
            break;
        }
        if (overlaps(in, (size_t)(L.batch * L.idist) * rb, out, (size_t)(L.batch * L.odist) * cb))
            fail(GFFT_ERR_ALIAS, "real-input transform: output must not overlap the input");
        p.r2c.run(in, out, L.batch, L.idist, L.odist, st, -1, scale);
        break;
    }
    case GFFT_KIND_C2C_2D: {
        const long long W = d.n0, H = d.n1;
        // row FFTs (FFT2D::scramble_row_fft, fft.h:229-241, in natural order)
        if (L.idist == H * L.istride && L.odist == H * L.ostride) {
            p.c2c.run(inverse, in, out, L.batch * H, L.istride, L.ostride, 1, 1, st);
        } else {
            for (long long b = 0; b < L.batch; b++)
                p.c2c.run(inverse, static_cast<const char *>(in) + (size_t)(b * L.idist) * cb,
                          static_cast<char *>(out) + (size_t)(b * L.odist) * cb, H, L.istride, L.ostride, 1, 1, st);
        }
        // column FFTs in place (FFTVert::transform_no_scramble, fft.h:217)
        p.col.run(inverse, out, out, W, L.ostride, L.ostride, L.batch, L.odist, L.odist, st, scale);
        break;
    }
    case GFFT_KIND_R2C_2D: {
        if (inverse) fail(GFFT_ERR_UNSUPPORTED, "RealFFT2D has no inverse (FFTReal.h:127-130)");
        const long long W = d.n0, H = d.n1;
        if (overlaps(in, (size_t)(L.batch * L.idist) * rb, out, (size_t)(L.batch * L.odist) * cb))
            fail(GFFT_ERR_ALIAS, "real 2D transform: output must not overlap the input (FFTReal.h:331)");
        if (L.idist == H * L.istride && L.odist == H * L.ostride) {
            p.r2c.run(in, out, L.batch * H, L.istride, L.ostride, st);
        } else {
            for (long long b = 0; b < L.batch; b++)
                p.r2c.run(static_cast<const char *>(in) + (size_t)(b * L.idist) * rb,
                          static_cast<char *>(out) + (size_t)(b * L.odist) * cb, H, L.istride, L.ostride, st);
        }
        // columns 0 .. W/2 (the non-redundant half), plus the Hermitian
        // mirror of columns 1 .. W/2-1 for the full-width layout
        p.col.run(0, out, out, W / 2 + 1, L.ostride, L.ostride, L.batch, L.odist, L.odist, st, scale);
        break;
    }
    case GFFT_KIND_VERT: {
        const long long cols = d.n1;
        if (out != in && overlaps(in, (size_t)(L.batch * L.idist) * cb, out, (size_t)(L.batch * L.odist) * cb))
            fail(GFFT_ERR_ALIAS, "column transform: output must be the input or not overlap it");
        p.col.run(inverse, in, out, cols, L.istride, L.ostride, L.batch, L.idist, L.odist, st, scale);
        break;
    }
    default:
        fail(GFFT_ERR_INVALID_PLAN, "plan has no transform kind");
    }
}

// A plan's workspace (multi-pass sizes) serves one transform at a time.
// The reference-shaped entry points share one plan per size (as the
// reference shares its per-size singletons, FFTLevel.h:76-88) whose
// workspace the caller never sees, so their execs may come from several
// threads and streams at once.  Those plans carry an event (ws_last): each
// exec waits on its stream for the previous one's event, under a host lock,
// and records its own, so they run in issue order.  Inside a stream capture
// the caller orders the graph's replays; the capture records no wait.
// Plans from gfft_plan_create carry no event: their execs are ordered by
// the caller (one stream, or one plan per stream).
static void exec_plan(gfft_plan_s &p, int inverse, void *out, const void *in, const Layout &L, cudaStream_t st,
                      double scale = 1.0)
{
    // NVTX range per exec (no cost unless a profiler is attached)
    static const char *const names[] = {"gfft exec C2C", "gfft exec R2C", "gfft exec C2C_2D", "gfft exec R2C_2D",
                                        "gfft exec VERT"};
    NvtxRange range(p.d.kind >= 0 && p.d.kind <= 4 ? names[p.d.kind] : "gfft exec");
    if (!p.ws_last) {
        exec_body(p, inverse, out, in, L, st, scale);
        return;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        (void)cudaGetLastError();
        cs = cudaStreamCaptureStatusActive;
    }
    if (cs != cudaStreamCaptureStatusNone) {
        exec_body(p, inverse, out, in, L, st, scale);
        return;
    }
    std::lock_guard<std::mutex> lk(p.ws_mu);
    check_cuda(cudaStreamWaitEvent(st, p.ws_last, 0), "workspace order wait");
    exec_body(p, inverse, out, in, L, st, scale);
    check_cuda(cudaEventRecord(p.ws_last, st), "workspace order record");
}

// Adjoint of the plan's transform in direction `inverse` (reverse-mode
// differentiation: grad_in = A^H grad_out in PyTorch's convention).
static void exec_adjoint(gfft_plan_s &p, int inverse, void *out, const void *in, const Layout &L, cudaStream_t st)
{
    const gfft_desc &d = p.d;
    switch (d.kind) {
    case GFFT_KIND_C2C:
    case GFFT_KIND_C2C_2D:
    case GFFT_KIND_VERT: {
        // the unnormalised DFT's adjoint is the conjugate-direction (unscaled
        // inverse) transform; the output layout becomes the input layout
        if (d.flags & GFFT_FLAG_BITREV_INPUT) fail(GFFT_ERR_UNSUPPORTED, "adjoint of a bit-reversed-input plan");
        Layout A{L.batch, L.ostride, L.odist, L.istride, L.idist};
        exec_plan(p, !inverse, out, in, A, st);
        break;
    }
    case GFFT_KIND_R2C: {
        const size_t cb = cplx_bytes(d.dtype), rb = real_bytes(d.dtype);
        if (!inverse) {
            // adjoint of R2C: C2R of the gradient with interior bins halved
            // (half spectrum) or folded (full spectrum)
            check_ptr(in, cb, "in");
            check_ptr(out, rb, "out");
            const int w = (d.flags & GFFT_FLAG_HALF_SPECTRUM) ? 1 : 2;
            p.c2r.run(in, out, L.batch, L.odist, L.idist, w, st);
        } else {
            // adjoint of the half-spectrum C2R: R2C with interior bins doubled
            check_ptr(in, rb, "in");
            check_ptr(out, cb, "out");
            if (!(d.flags & GFFT_FLAG_HALF_SPECTRUM))
                fail(GFFT_ERR_UNSUPPORTED, "adjoint of the inverse needs a half-spectrum plan");
            p.r2c.run(in, out, L.batch, L.idist, L.odist, st, 2);
        }
        break;
    }
    default:
        fail(GFFT_ERR_UNSUPPORTED, "no adjoint for this transform kind");
    }
}

// bytes of one transform's input and output in the direction run; the
// half-spectrum inverse of an R2C plan reads the plan's output layout
// (bins, odist) and writes its input layout (reals, idist)
static void io_item_bytes(const gfft_plan_s &p, int inverse, size_t *ib, size_t *ob)
{
    const gfft_desc &d = p.d;
    const bool real_in = d.kind == GFFT_KIND_R2C || d.kind == GFFT_KIND_R2C_2D;
    const size_t in_bytes = (size_t)d.idist * (real_in ? real_bytes(d.dtype) : cplx_bytes(d.dtype));
    const size_t out_bytes = (size_t)d.odist * cplx_bytes(d.dtype);
    const bool c2r = d.kind == GFFT_KIND_R2C && inverse;
    *ib = c2r ? out_bytes : in_bytes;
    *ob = c2r ? in_bytes : out_bytes;
}

// The host path stages whole transforms: transform b's input is the block
// of idist elements at b * idist (output likewise), so each transform must
// lie inside its own block (no batch-interleaved layouts there).
static void check_host_layout(const gfft_desc &d)
{
    const bool half = (d.flags & GFFT_FLAG_HALF_SPECTRUM) != 0;
    long long in_span = 0, out_span = 0;
    switch (d.kind) {
    case GFFT_KIND_C2C:
        in_span = (d.n0 - 1) * d.istride + 1;
        out_span = (d.n0 - 1) * d.ostride + 1;
        break;
    case GFFT_KIND_R2C:
        in_span = d.n0;
        out_span = half ? d.n0 / 2 + 1 : d.n0;
        break;
    case GFFT_KIND_C2C_2D:
        in_span = (d.n1 - 1) * d.istride + d.n0;
        out_span = (d.n1 - 1) * d.ostride + d.n0;
        break;
    case GFFT_KIND_R2C_2D:
        in_span = (d.n1 - 1) * d.istride + d.n0;
        out_span = (d.n1 - 1) * d.ostride + (half ? d.n0 / 2 + 1 : d.n0);
        break;
    case GFFT_KIND_VERT:
        in_span = (d.n0 - 1) * d.istride + d.n1;
        out_span = (d.n0 - 1) * d.ostride + d.n1;
        break;
    default:
        fail(GFFT_ERR_INVALID_PLAN, "plan has no transform kind");
    }
    if (in_span > d.idist || out_span > d.odist)
        fail(GFFT_ERR_UNSUPPORTED,
             "host buffers: each transform must lie within its own idist / odist block (use device buffers for "
             "interleaved batches)");
}

// The device reads host memory through the host's page tables (GB300 with
// Grace: NVLink-C2C with address translation), so a kernel may touch any
// valid host buffer; cached per device.
static bool host_tables_device()
{
    static std::mutex mu;
    static std::map<int, bool> ok;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(mu);
    auto it = ok.find(dev);
    if (it == ok.end()) {
        int pageable = 0, tables = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            pageable = tables = 0;
        }
        it = ok.emplace(dev, pageable == 1 && tables == 1).first;
    }
    return it->second;
}

// first and last byte of [p, p + bytes) in page-locked host memory that the
// device sees at the same address
static bool pinned_same_address(const void *ptr, size_t bytes)
{
    const unsigned char *c = static_cast<const unsigned char *>(ptr);
    for (const unsigned char *q : {c, c + bytes - 1}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost || a.devicePointer != (const void *)q) return false;
    }
    return true;
}

static void exec_host(gfft_plan_s &p, int inverse, void *out, const void *in)
{
    const gfft_desc &d = p.d;
    if (!in || !out) fail(GFFT_ERR_INVALID_VALUE, "NULL host buffer");
    check_host_layout(d);
    std::lock_guard<std::mutex> lk(p.host_mu);
    size_t ib, ob;
    io_item_bytes(p, inverse, &ib, &ob);
    // Single-kernel C2C on pinned buffers: the kernel reads the input and
    // writes the output over the host link itself, with no staging copies.
    // Measured on GB300 at 2^12 x 16384: 330 GB/s algorithmic against 304
    // for the staged pipeline (the link carries 165 GB/s each way in both
    // cases; staging loses its chunk seams).  GFFT_HOST_DIRECT=0 turns it off.
    static const bool direct_on = [] {
        const char *v = std::getenv("GFFT_HOST_DIRECT");
        return !(v && *v == '0');
    }();
    if (direct_on && d.kind == GFFT_KIND_C2C && d.mode == GFFT_MODE_PLAIN && p.c2c.algo == 1 &&
        !(d.flags & GFFT_FLAG_BITREV_INPUT) && host_tables_device() &&
        pinned_same_address(in, (size_t)d.batch * ib) && pinned_same_address(out, (size_t)d.batch * ob)) {
        if (!p.compute_stream) {
            check_cuda(cudaStreamCreateWithFlags(&p.compute_stream, cudaStreamNonBlocking), "stream");
            for (int i = 0; i < 3; i++) {
                check_cuda(cudaEventCreateWithFlags(&p.ev_in[i], cudaEventDisableTiming), "event");
                check_cuda(cudaEventCreateWithFlags(&p.ev_done[i], cudaEventDisableTiming), "event");
            }
        }
        exec_plan(p, inverse, out, in, plan_layout(p), p.compute_stream);
        check_cuda(cudaStreamSynchronize(p.compute_stream), "sync");
        return;
    }
    // chunks of about 64 MB (GFFT_HOST_CHUNK_MB), at least one transform
    static const long long chunk = [] {
        const char *v = std::getenv("GFFT_HOST_CHUNK_MB");
        const long long mb = (v && *v) ? std::atoll(v) : 64;
        return std::max<long long>(1, mb) << 20;
    }();
    long long per = std::max<long long>(1, chunk / (long long)std::max<size_t>(std::max(ib, ob), 1));
    per = std::min(per, d.batch);
    if (!p.stage[0] || p.stage_bytes_in < per * ib || p.stage_bytes_out < per * ob) {
        for (int i = 0; i < 3; i++) {
            if (p.stage[i]) cudaFree(p.stage[i]);
            if (p.stage_out[i]) cudaFree(p.stage_out[i]);
            p.stage[i] = p.stage_out[i] = nullptr;
        }
        p.stage_bytes_in = p.stage_bytes_out = 0;
        for (int i = 0; i < 3; i++) {
            check_cuda(cudaMalloc(&p.stage[i], per * ib), "cudaMalloc(stage)");
            check_cuda(cudaMalloc(&p.stage_out[i], per * ob), "cudaMalloc(stage)");
            if (!p.host_streams[i])
                check_cuda(cudaStreamCreateWithFlags(&p.host_streams[i], cudaStreamNonBlocking), "stream");
        }
        p.stage_bytes_in = per * ib;
        p.stage_bytes_out = per * ob;
    }
    if (!p.compute_stream) {
        check_cuda(cudaStreamCreateWithFlags(&p.compute_stream, cudaStreamNonBlocking), "stream");
        for (int i = 0; i < 3; i++) {
            check_cuda(cudaEventCreateWithFlags(&p.ev_in[i], cudaEventDisableTiming), "event");
            check_cuda(cudaEventCreateWithFlags(&p.ev_done[i], cudaEventDisableTiming), "event");
        }
    }
    // copies overlap on three streams; the transforms run in order on one
    // compute stream, because a plan's workspace serves one exec at a time
    const unsigned char *hin = static_cast<const unsigned char *>(in);
    unsigned char *hout = static_cast<unsigned char *>(out);
    int c = 0;
    for (long long b0 = 0; b0 < d.batch; b0 += per, c++) {
        const long long nb = std::min(per, d.batch - b0);
        const int s = c % 3;
        cudaStream_t st = p.host_streams[s];
        check_cuda(cudaMemcpyAsync(p.stage[s], hin + b0 * ib, nb * ib, cudaMemcpyHostToDevice, st), "H2D");
        check_cuda(cudaEventRecord(p.ev_in[s], st), "event");
        check_cuda(cudaStreamWaitEvent(p.compute_stream, p.ev_in[s], 0), "event wait");
        Layout L = plan_layout(p);
        L.batch = nb;
        exec_plan(p, inverse, p.stage_out[s], p.stage[s], L, p.compute_stream);
        check_cuda(cudaEventRecord(p.ev_done[s], p.compute_stream), "event");
        check_cuda(cudaStreamWaitEvent(st, p.ev_done[s], 0), "event wait");
        check_cuda(cudaMemcpyAsync(hout + b0 * ob, p.stage_out[s], nb * ob, cudaMemcpyDeviceToHost, st), "D2H");
    }
    for (int i = 0; i < 3; i++) check_cuda(cudaStreamSynchronize(p.host_streams[i]), "sync");
}

static void destroy_plan(gfft_plan_s *p)
{
    for (int i = 0; i < 3; i++) {
        if (p->stage[i]) cudaFree(p->stage[i]);
        if (p->stage_out[i]) cudaFree(p->stage_out[i]);
        if (p->host_streams[i]) cudaStreamDestroy(p->host_streams[i]);
        if (p->ev_in[i]) cudaEventDestroy(p->ev_in[i]);
        if (p->ev_done[i]) cudaEventDestroy(p->ev_done[i]);
    }
    if (p->compute_stream) cudaStreamDestroy(p->compute_stream);
    if (p->ws_last) cudaEventDestroy(p->ws_last);
    p->c2c.release();
    p->r2c.release();
    p->c2r.release();
    p->tc.release();
    p->col.release();
    p->magic = 0;
    delete p;
}

// Cached plans for the reference-shaped entry points: one per (device,
// kind, dtype, n0, n1, flags); batch, strides and pointers come per call.
// Their workspace (four-step sizes only) is shared: calls that need one
// must not overlap on different streams.
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
    // the batch is per call; this one only sizes the workspace: full groups
    // within 512 MB (these plans live until exit, one per size used)
    const long long elems = std::max<long long>(1, n0) * std::max<long long>(1, n1);
    d.batch = std::max<long long>(1, (512LL << 20) / (elems * (long long)cplx_bytes(dtype)));
    gfft_plan_s *p = make_plan(d);
    if (p->workspace_bytes() > 0) {
        cudaError_t e = cudaEventCreateWithFlags(&p->ws_last, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            destroy_plan(p);
            check_cuda(e, "cudaEventCreate");
        }
    }
    cache.emplace(key, p);
    return p;
}

}  // namespace gfft

using namespace gfft;

#define GFFT_GUARD(...)                          \
    try {                                        \
        __VA_ARGS__;                             \
        return GFFT_OK;                          \
    } catch (const Error &e) {                   \
        g_last_error = e.msg;                    \
        return e.status;                         \
    } catch (const std::bad_alloc &) {           \
        g_last_error = "host allocation failed"; \
        return GFFT_ERR_ALLOC;                   \
    } catch (...) {                              \
        g_last_error = "unexpected exception";   \
        return GFFT_ERR_INVALID_VALUE;           \
    }

static gfft_plan_s *checked(gfft_plan p)
{
    if (!p || p->magic != 0x6766u) fail(GFFT_ERR_INVALID_PLAN, "invalid plan handle");
    return p;
}

static void need_batch(long long batch)
{
    if (batch < 1) fail(GFFT_ERR_INVALID_SIZE, "batch must be >= 1");
}

static void need_dtype(int dtype)
{
    if (dtype != GFFT_F32 && dtype != GFFT_F64) fail(GFFT_ERR_INVALID_VALUE, "dtype must be GFFT_F32 or GFFT_F64");
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
    GFFT_GUARD({ destroy_plan(checked(plan)); });
}

gfft_status gfft_exec(gfft_plan plan, int inverse, void *out, const void *in, void *stream)
{
    GFFT_GUARD({
        gfft_plan_s *p = checked(plan);
        exec_plan(*p, inverse != 0, out, in, plan_layout(*p), (cudaStream_t)stream);
    });
}

gfft_status gfft_exec_scaled(gfft_plan plan, int inverse, double scale, void *out, const void *in, void *stream)
{
    GFFT_GUARD({
        gfft_plan_s *p = checked(plan);
        exec_plan(*p, inverse != 0, out, in, plan_layout(*p), (cudaStream_t)stream, scale);
    });
}

gfft_status gfft_exec_adjoint(gfft_plan plan, int inverse, void *out, const void *in, void *stream)
{
    GFFT_GUARD({
        gfft_plan_s *p = checked(plan);
        exec_adjoint(*p, inverse != 0, out, in, plan_layout(*p), (cudaStream_t)stream);
    });
}

gfft_status gfft_exec_host(gfft_plan plan, int inverse, void *out, const void *in)
{
    GFFT_GUARD({
        NvtxRange range("gfft exec host");
        exec_host(*checked(plan), inverse != 0, out, in);
    });
}

gfft_status gfft_plan_launches_dir(gfft_plan plan, int inverse, int *launches)
{
    GFFT_GUARD({
        if (!launches) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        gfft_plan_s *p = checked(plan);
        *launches = inverse ? p->launches_inv : p->launches;
    });
}

gfft_status gfft_plan_launches(gfft_plan plan, int *launches)
{
    GFFT_GUARD({
        if (!launches) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        *launches = checked(plan)->launches;
    });
}

gfft_status gfft_plan_workspace_size(gfft_plan plan, size_t *bytes)
{
    GFFT_GUARD({
        if (!bytes) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        gfft_plan_s *p = checked(plan);
        *bytes = p->workspace_bytes();
    });
}

// ---- reference-shaped entry points ---------------------------------------

gfft_status gfft_fft_transform(int dtype, int n, long long batch, int inverse, void *out, const void *in,
                               void *stream)
{
    GFFT_GUARD({
        need_batch(batch);
        need_dtype(dtype);
        gfft_plan_s *p = cached_plan(GFFT_KIND_C2C, dtype, n, 0, 0);
        exec_plan(*p, inverse != 0, out, in, Layout{batch, 1, n, 1, n}, (cudaStream_t)stream);
    });
}

gfft_status gfft_fft_transform_no_scramble(int dtype, int n, long long batch, int inverse, void *inout,
                                           void *stream)
{
    GFFT_GUARD({
        need_batch(batch);
        need_dtype(dtype);
        gfft_plan_s *p = cached_plan(GFFT_KIND_C2C, dtype, n, 0, GFFT_FLAG_BITREV_INPUT);
        exec_plan(*p, inverse != 0, inout, inout, Layout{batch, 1, n, 1, n}, (cudaStream_t)stream);
    });
}

gfft_status gfft_fft_transform_real(int dtype, int n, long long batch, void *out, const void *in, void *stream)
{
    GFFT_GUARD({
        need_batch(batch);
        need_dtype(dtype);
        gfft_plan_s *p = cached_plan(GFFT_KIND_R2C, dtype, n, 0, 0);
        exec_plan(*p, 0, out, in, Layout{batch, 1, n, 1, n}, (cudaStream_t)stream);
    });
}

gfft_status gfft_fft_transform_interleave(int dtype, int n, void *out, const void *in1, const void *in2,
                                          void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        gfft_plan_s *p = cached_plan(GFFT_KIND_C2C, dtype, n, 0, 0);
        check_ptr(in1, real_bytes(dtype), "in1");
        check_ptr(in2, real_bytes(dtype), "in2");
        check_ptr(out, cplx_bytes(dtype), "out");
        check_cuda(launch_interleave(dtype, in1, n, in2, n, out, n, 1, n, (cudaStream_t)stream), "interleave");
        exec_plan(*p, 0, out, out, Layout{1, 1, n, 1, n}, (cudaStream_t)stream);
    });
}

gfft_status gfft_vert_transform(int dtype, int n, int inverse, void *out, long long out_stride, const void *in,
                                long long in_stride, int cols, void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        if (cols < 1) fail(GFFT_ERR_INVALID_SIZE, "cols must be >= 1");
        if (out == in) fail(GFFT_ERR_ALIAS, "FFTVert::transform: out must not be in (fft.h:140)");
        if (in_stride < cols || out_stride < cols) fail(GFFT_ERR_INVALID_VALUE, "row stride below cols");
        gfft_plan_s *p = cached_plan(GFFT_KIND_VERT, dtype, n, cols, 0);
        exec_plan(*p, inverse != 0, out, in, Layout{1, in_stride, n * in_stride, out_stride, n * out_stride},
                  (cudaStream_t)stream);
    });
}

gfft_status gfft_vert_transform_no_scramble(int dtype, int n, int inverse, void *data, long long stride, int cols,
                                            void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        if (cols < 1) fail(GFFT_ERR_INVALID_SIZE, "cols must be >= 1");
        if (stride < cols) fail(GFFT_ERR_INVALID_VALUE, "row stride below cols");
        gfft_plan_s *p = cached_plan(GFFT_KIND_VERT, dtype, n, cols, GFFT_FLAG_BITREV_INPUT);
        exec_plan(*p, inverse != 0, data, data, Layout{1, stride, n * stride, stride, n * stride},
                  (cudaStream_t)stream);
    });
}

gfft_status gfft_dit_apply(int dtype, int n, void *out, const void *in, int half, void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        if (!is_pow2(n)) fail(GFFT_ERR_INVALID_SIZE, "size must be a power of two >= 1");
        check_device();
        check_ptr(in, cplx_bytes(dtype), "in");
        check_ptr(out, cplx_bytes(dtype), "out");
        if (n == 1) {
            check_cuda(launch_dit_one(dtype, in, out, (cudaStream_t)stream), "DIT n=1");
        } else {
            const int logn = ilog2ll(n);
            const void *dtw = cached_table("dit/" + std::to_string(dtype) + "/" + std::to_string(logn), dtype,
                                           (size_t)n / 2 + 1,
                                           [dtype, logn](void *buf) { dit_twiddle_fill(dtype, logn, buf); });
            check_cuda(launch_dit(dtype, half ? 0 : 1, in, out, n / 2, 1, n, n, dtw, (cudaStream_t)stream), "DIT");
        }
    });
}

gfft_status gfft_fft2d_transform(int dtype, int width, int height, int inverse, void *out, long long out_stride,
                                 const void *in, long long in_stride, void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        gfft_plan_s *p = cached_plan(GFFT_KIND_C2C_2D, dtype, width, height, 0);
        if (in_stride < width || out_stride < width) fail(GFFT_ERR_INVALID_VALUE, "row stride below width");
        exec_plan(*p, inverse != 0, out, in,
                  Layout{1, in_stride, height * in_stride, out_stride, height * out_stride}, (cudaStream_t)stream);
    });
}

gfft_status gfft_real_fft_forward(int dtype, int n, long long batch, void *out, const void *in, int half,
                                  void *stream)
{
    GFFT_GUARD({
        need_batch(batch);
        need_dtype(dtype);
        gfft_plan_s *p = cached_plan(GFFT_KIND_R2C, dtype, n, 0, half ? GFFT_FLAG_HALF_SPECTRUM : 0);
        // the reference's output buffer holds n complex values either way
        exec_plan(*p, 0, out, in, Layout{batch, 1, n, 1, n}, (cudaStream_t)stream);
    });
}

gfft_status gfft_real_fft2d_forward(int dtype, int width, int height, void *out, long long out_stride,
                                    const void *in, long long in_stride, void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        if (width > 1 && (in_stride % 2)) fail(GFFT_ERR_INVALID_VALUE, "input row stride must be even");
        if (in_stride < width || out_stride < width) fail(GFFT_ERR_INVALID_VALUE, "row stride below width");
        gfft_plan_s *p = cached_plan(GFFT_KIND_R2C_2D, dtype, width, height, 0);
        exec_plan(*p, 0, out, in, Layout{1, in_stride, height * in_stride, out_stride, height * out_stride},
                  (cudaStream_t)stream);
    });
}

gfft_status gfft_real_fft2d_forward_2x(int dtype, int width, int height, void *out, long long out_stride,
                                       const void *in1, long long in_stride1, const void *in2,
                                       long long in_stride2, void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        if (out_stride < width || in_stride1 < width || in_stride2 < width)
            fail(GFFT_ERR_INVALID_VALUE, "row stride below width");
        gfft_plan_s *p = cached_plan(GFFT_KIND_C2C_2D, dtype, width, height, 0);
        check_ptr(in1, real_bytes(dtype), "in1");
        check_ptr(in2, real_bytes(dtype), "in2");
        check_ptr(out, cplx_bytes(dtype), "out");
        // rows hold in1 + i in2, then the complex 2D transform in place
        check_cuda(launch_interleave(dtype, in1, in_stride1, in2, in_stride2, out, out_stride, height, width,
                                     (cudaStream_t)stream),
                   "interleave");
        exec_plan(*p, 0, out, out, Layout{1, out_stride, height * out_stride, out_stride, height * out_stride},
                  (cudaStream_t)stream);
    });
}

gfft_status gfft_separate_2x_real_fft(int dtype, int n, void *out1, void *out2, const void *in, void *stream)
{
    GFFT_GUARD({
        need_dtype(dtype);
        if (!is_pow2(n) || n < 2) fail(GFFT_ERR_INVALID_SIZE, "size must be a power of two >= 2");
        check_device();
        check_ptr(in, cplx_bytes(dtype), "in");
        check_ptr(out1, cplx_bytes(dtype), "out1");
        check_ptr(out2, cplx_bytes(dtype), "out2");
        if (out1 == out2) fail(GFFT_ERR_ALIAS, "out1 and out2 must differ");
        check_cuda(launch_separate2x(dtype, in, out1, out2, n, (cudaStream_t)stream), "separate");
    });
}

// ---- test hook (not declared in the public header) -------------------------
// One persistent four-step launch (fp32, n = 2^16) whose only work items are
// row tiles waiting on column tiles that are never scheduled: their bounded
// dependency wait runs out after about one second, the kernel records
// DEV_ERR_TMA_TIMEOUT in the device error word and every CTA returns.  It
// writes nothing to `out`.  Lets a test check that no wait can hang and
// that the context stays usable.
gfft_status gfft_test_stalled_fourstep(void *out, const void *in, void *stream)
{
    GFFT_GUARD({
        check_device();
        gfft::C2CCore core;
        core.init(GFFT_F32, 16, 1, 1);  // the persistent kernel
        cudaError_t e = cudaSuccess;
        try {
            core.run_stalled(in, out, (cudaStream_t)stream);
            e = cudaStreamSynchronize((cudaStream_t)stream);
        } catch (...) {
            core.release();
            throw;
        }
        core.release();
        check_cuda(e, "stalled four-step");
    });
}

// ---- ragged batches --------------------------------------------------------

gfft_status gfft_ragged_create(gfft_ragged *plan, int dtype, const long long *sizes, long long count)
{
    GFFT_GUARD({
        if (!plan || !sizes) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        *plan = nullptr;
        check_device();
        *plan = reinterpret_cast<gfft_ragged>(ragged_create(dtype, sizes, count));
    });
}

gfft_status gfft_ragged_destroy(gfft_ragged plan)
{
    GFFT_GUARD({
        if (!plan) fail(GFFT_ERR_INVALID_PLAN, "NULL ragged plan");
        ragged_destroy(reinterpret_cast<RaggedPlan *>(plan));
    });
}

gfft_status gfft_ragged_exec(gfft_ragged plan, int inverse, void *out, const void *in, void *stream)
{
    GFFT_GUARD({
        if (!plan) fail(GFFT_ERR_INVALID_PLAN, "NULL ragged plan");
        NvtxRange range("gfft ragged exec");
        ragged_exec(*reinterpret_cast<RaggedPlan *>(plan), inverse != 0, out, in, (cudaStream_t)stream, true);
    });
}

gfft_status gfft_ragged_exec_adjoint(gfft_ragged plan, int inverse, void *out, const void *in, void *stream)
{
    GFFT_GUARD({
        if (!plan) fail(GFFT_ERR_INVALID_PLAN, "NULL ragged plan");
        ragged_exec(*reinterpret_cast<RaggedPlan *>(plan), inverse == 0, out, in, (cudaStream_t)stream, true);
    });
}

gfft_status gfft_ragged_autotune(gfft_ragged plan, void *out, const void *in, void *stream, int *params,
                                 double *ms)
{
    GFFT_GUARD({
        if (!plan) fail(GFFT_ERR_INVALID_PLAN, "NULL ragged plan");
        int best[3] = {0, 0, 0};
        const double t = ragged_autotune(*reinterpret_cast<RaggedPlan *>(plan), out, in, (cudaStream_t)stream, best);
        if (params) params[0] = best[0], params[1] = best[1], params[2] = best[2];
        if (ms) *ms = t;
    });
}

gfft_status gfft_ragged_elements(gfft_ragged plan, long long *elements)
{
    GFFT_GUARD({
        if (!plan || !elements) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        *elements = ragged_total(reinterpret_cast<RaggedPlan *>(plan));
    });
}

gfft_status gfft_device_error(int *code)
{
    GFFT_GUARD({
        if (!code) fail(GFFT_ERR_INVALID_VALUE, "NULL argument");
        unsigned v = 0;
        unsigned *w = device_error_word();
        check_cuda(cudaMemcpy(&v, w, sizeof v, cudaMemcpyDeviceToHost), "read error word");
        check_cuda(cudaMemset(w, 0, sizeof v), "reset error word");
        *code = (int)v;
        if (v) fail(GFFT_ERR_TIMEOUT, "a device-side wait gave up (bounded TMA wait)");
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
