// plan.h -- internal plan objects: reusable transform "cores" and the plan
// that strings them together per gfft_kind.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "internal.h"
#include "fourstep.h"
#include "threepass.h"
#include "tiles_registry.h"

namespace gfft {

size_t cplx_bytes(int dtype);
int ilog2ll(long long n);
bool is_pow2(long long n);

// Batched 1D C2C of n = 2^logn points: one fused kernel up to the shared
// memory limit, else the four-step column + row passes through a workspace.
struct C2CCore {
    int dtype = 0, logn = 0;
    int algo = 0;  // 1 fused, 2 four-step tile launches, 3 persistent four-step, 5 three passes
    const void *tw = nullptr;
    // persistent four-step: kernel, ring of `fs_slots` transforms, counters
    const FourStepKernel *fs = nullptr;
    // algo 5: three passes of short tiles (threepass.cu) through `ws`
    const ThreePass *tp = nullptr;
    const void *tp_tw[3] = {};
    const void *tp_lo2 = nullptr, *tp_hi2 = nullptr;  // W_(n / 2^la) tables of pass 2
    int tp_bits2 = 0;
    int fs_slots = 0, fs_lag = 0, fs_grid = 0;
    int fs_nr = 0;            // row items per transform
    bool fs_real = false;     // real-input mode: the kernel's DIT version
    int *fs_ctr = nullptr;
    const void *tw_a = nullptr, *tw_b = nullptr;
    int logA = 0, logB = 0, ccol = 0, crow = 0, lo_bits = 0;
    const TileKernel *kcol = nullptr, *krow = nullptr;
    const void *tw_col = nullptr, *tw_row = nullptr, *tw_lo = nullptr, *tw_hi = nullptr;
    long long group = 0;       // transforms per column/row launch pair
    void *ws = nullptr;        // group * n (algo 2) or fs_slots * n (algo 3) elements
    size_t ws_bytes = 0;

    // path: -1 the measured default (or GFFT_FS), 1 the persistent
    // four-step kernel, 0 the tile launches.  real_rows (with path 1): a
    // variant with a real-input version, scheduled for its row items
    void init(int dtype, int logn, long long batch_hint, int path = -1, bool real_rows = false);
    void release();
    int launches(long long batch) const;
    // strides in complex elements; four-step needs unit element strides
    void run(int inverse, const void *in, void *out, long long batch, long long idist, long long odist,
             long long istride, long long ostride, cudaStream_t st, double scale = 1.0) const;
    // persistent four-step: the launches over `batch` transforms (dtw: the
    // DIT twiddles in real-input mode); false, with nothing launched, when
    // the input cannot be read by tensor copies (not 16-byte aligned)
    bool run_persistent(int inverse, const void *in, void *out, long long batch, long long idist, long long odist,
                        cudaStream_t st, double scale, const void *dtw = nullptr) const;
    // persistent four-step only: one launch whose row tiles wait on column
    // tiles that are never scheduled (the bounded wait must run out)
    void run_stalled(const void *in, void *out, cudaStream_t st) const;
};

// Column FFTs of length 2^logl over ncols columns (tile kernels).
struct ColCore {
    int dtype = 0, logl = 0, variant = 0, c = 0;
    const TileKernel *k = nullptr;
    const void *tw = nullptr;
    // split column FFTs (columns longer than one tile, 2^13 .. 2^24 points,
    // and fp32 plain columns of 2^10 .. 2^12 on request): each column of
    // H = H1 * H2 points is two launches of short column FFTs per band of
    // columns, through a scratch of one band (see ColCore::run).  Bit-
    // reversed rows first go through a row permutation pass (rows_bitrev);
    // the full-width real 2D layout gets its mirrored half from a fill pass
    // after the plain columns (herm_fill)
    bool split = false, rows_bitrev = false, herm_fill = false;
    int l1 = 0, l2 = 0, c1 = 0, c2 = 0, lo_bits = 0;
    const TileKernel *ka = nullptr, *kb = nullptr;
    const void *tw_a = nullptr, *tw_b = nullptr, *tw_lo = nullptr, *tw_hi = nullptr;
    long long band = 0;  // columns per band
    void *scratch = nullptr;
    size_t ws_bytes = 0;
    // allow_split = false keeps the one-launch tiles where they exist (real
    // 2D, whose half- and full-width results agree bit for bit through the
    // same tiles); max_cols bounds the scratch band (0 = no bound)
    void init(int dtype, int logl, int variant, bool allow_split = true, long long max_cols = 0);
    void release();
    long long launches(long long ncols, long long batch) const
    {
        if (!split) return 1;
        return 2 * batch * ((ncols + band - 1) / band) + (rows_bitrev ? 1 : 0) + (herm_fill ? 1 : 0);
    }
    void run(int inverse, const void *in, void *out, long long ncols, long long ld_in, long long ld_out,
             long long batch, long long idist, long long odist, cudaStream_t st, double scale = 1.0) const;
};

// Row pass of a four-step real-input transform with the DIT adjustment
// fused in (real_4step.cu)
struct RowDitKernel {
    const void *fn = nullptr;
    int threads = 0;
    size_t smem = 0;
    int ch = 0, logb = 0;  // rows per half-block, log2 row length
    size_t twcount = 0;
    void (*fill)(void *) = nullptr;
};
const RowDitKernel *rowdit_find(int dtype, int logb);
cudaError_t launch_rowpass_dit(const RowDitKernel &k, const void *in, void *out, long long A, long long batch,
                               long long idist, long long odist, const void *tw, const void *dtw, cudaStream_t st,
                               double scale = 1.0);

// Real-input 1D transform of n = 2^logn reals (RealFFT<T>::forward).
// mode: 0 half spectrum, 1 full spectrum, 2 half with doubled interior bins
struct R2CCore {
    int dtype = 0, logn = 0, half = 1;
    // 0 n == 1, 1 fused, 2 C2C(n/2) + DIT pass, 3 four-step column pass +
    // row pass with the DIT fused, 4 one persistent four-step launch whose
    // row items apply the DIT (3 and 4: half spectrum; other modes as 2)
    int algo = 0;
    const void *tw = nullptr, *dtw = nullptr;
    const RowDitKernel *rowdit = nullptr;
    const void *tw_rowdit = nullptr;
    C2CCore c2c;
    void init(int dtype, int logn, int half, long long batch_hint);
    void release() { c2c.release(); }
    int launches(long long batch) const;
    // idist in reals (even), odist in complex elements
    void run(const void *in, void *out, long long batch, long long idist, long long odist, cudaStream_t st,
             int mode = -1, double scale = 1.0) const;
};

// Half-spectrum inverse: n/2+1 bins -> n reals, unscaled, Hermitian
// extension (imaginary parts of the DC and Nyquist bins ignored)
struct C2RCore {
    int dtype = 0, logn = 0;
    int algo = 0;  // 0 n == 1, 1 fused, 2 pre-pass + C2C(n/2) inverse
    const void *tw = nullptr, *dtw = nullptr;
    // algo 1 whose folded full-spectrum input (2 n/2 bins) does not fit the
    // fused kernel's shared memory: that mode takes the algo 2 route
    bool fold_split = false;
    C2CCore c2c;
    void init(int dtype, int logn, long long batch_hint);
    void release() { c2c.release(); }
    int launches(long long batch) const;
    // idist in complex elements, odist in reals (even)
    void run(const void *in, void *out, long long batch, long long idist, long long odist, int wmode,
             cudaStream_t st, double scale = 1.0) const;
};

// Split-precision tensor-core C2C (tc.cu): fp32 data, radix-16 DFT blocks
// as FP16 hi+lo or BF16 hi+mid+lo products on tcgen05; n = 256, 4096, 65536
struct TCCore {
    int mode = 0, logn = 0;
    const void *bmat[2] = {nullptr, nullptr};  // DFT-16 split terms, forward / inverse
    const void *tw256 = nullptr, *tw2 = nullptr;  // W_256 and the low-order W_N table
    long long group = 0;  // transforms per column/row launch pair (n = 65536)
    void *ws = nullptr;
    size_t ws_bytes = 0;
    void init(int mode, int logn, long long batch_hint);
    void release();
    int launches(long long batch) const;
    void run(int inverse, const void *in, void *out, long long batch, long long idist, long long odist,
             long long istride, long long ostride, cudaStream_t st, double scale = 1.0) const;
};

// ---- kernels in real.cu --------------------------------------------------
int r2c_fused_max_logh(int dtype);
size_t r2c_twiddle_count(int dtype, int logh);
void r2c_twiddle_fill(int dtype, int logh, void *buf);
void dit_twiddle_fill(int dtype, int logn, void *buf);
// mode: 0 half spectrum, 1 full spectrum, 2 half with doubled interior
// bins (the adjoint of the half-spectrum C2R)
cudaError_t launch_r2c_fused(int dtype, int logh, int mode, const void *in, void *out, long long batch,
                             long long idist, long long odist, const void *tw, const void *dtw, cudaStream_t st,
                             double scale = 1.0);
cudaError_t launch_dit(int dtype, int mode, const void *in, void *out, long long H, long long batch,
                       long long idist, long long odist, const void *dtw, cudaStream_t st, double scale = 1.0);
// C2R (c2r.cu): weighting 0 = as given (Hermitian extension), 1 = interior
// bins halved (adjoint of the half-spectrum R2C), 2 = n-bin input folded
// (g_k + conj g_{n-k}) / 2 (adjoint of the full-spectrum R2C)
int c2r_fused_max_logh(int dtype);
// whether the fused C2R holds a transform of half length 2^logh with the
// input weighting wmode (0 plain, 1 halved interior, 2 folded full spectrum)
// in one CTA's shared memory
bool c2r_fused_fits(int dtype, int logh, int wmode);
cudaError_t launch_c2r_fused(int dtype, int logh, int wmode, const void *in, void *out, long long batch,
                             long long idist, long long odist, const void *tw, const void *dtw, cudaStream_t st,
                             double scale = 1.0);
cudaError_t launch_c2r_pre(int dtype, int wmode, const void *in, void *out, long long H, long long batch,
                           long long idist, long long odist, const void *dtw, cudaStream_t st);
cudaError_t launch_c2r_one(int dtype, const void *in, void *out, long long batch, long long idist, long long odist,
                           cudaStream_t st, double scale = 1.0);
cudaError_t launch_dit_one(int dtype, const void *in, void *out, cudaStream_t st);
cudaError_t launch_r2c_one(int dtype, const void *in, void *out, long long batch, long long idist, long long odist,
                           cudaStream_t st, double scale = 1.0);
cudaError_t launch_separate2x(int dtype, const void *in, void *o1, void *o2, long long n, cudaStream_t st);
cudaError_t launch_interleave(int dtype, const void *a, long long lda, const void *b, long long ldb, void *z,
                              long long ldz, long long rows, long long cols, cudaStream_t st);
cudaError_t launch_bitrev_swap(int dtype, void *x, int logn, long long batch, long long dist, cudaStream_t st);

// ---- passes around the split column FFTs (colsplit.cu) -----------------
// rows i -> bit-reversed rows (in place: swaps; else a copy into out)
cudaError_t launch_rows_bitrev(int dtype, const void *in, void *out, int logh, long long ncols, long long ld_in,
                               long long ld_out, long long batch, long long idist, long long odist, cudaStream_t st);
// full-width real 2D: columns W/2+1 .. W-1 from the conjugate mirror
cudaError_t launch_herm_fill(int dtype, void *out, long long H, long long W, long long ld, long long batch,
                             long long odist, cudaStream_t st);

// ---- ragged batches (ragged.cu) ------------------------------------------
struct RaggedPlan;
RaggedPlan *ragged_create(int dtype, const long long *sizes, long long count);
void ragged_destroy(RaggedPlan *p);
long long ragged_total(const RaggedPlan *p);
void ragged_exec(RaggedPlan &p, int inverse, void *out, const void *in, cudaStream_t st, bool use_graph);
double ragged_autotune(RaggedPlan &p, void *out, const void *in, cudaStream_t st, int *best);

}  // namespace gfft

// the public handle
struct gfft_plan_s {
    gfft_desc d;
    unsigned magic = 0x6766u;
    int device = 0;
    int launches = 0;      // per forward exec
    int launches_inv = 0;  // per inverse exec
    gfft::C2CCore c2c;   // C2C; 2D row pass
    gfft::ColCore col;   // 2D column pass; VERT
    gfft::R2CCore r2c;   // R2C; real-2D row pass
    gfft::C2RCore c2r;   // C2R; adjoint of R2C
    gfft::TCCore tc;     // C2C in a tensor-core mode
    // host-path staging (owned, lazily allocated)
    std::mutex host_mu;
    void *stage[3] = {nullptr, nullptr, nullptr};
    void *stage_out[3] = {nullptr, nullptr, nullptr};
    size_t stage_bytes_in = 0, stage_bytes_out = 0;
    cudaStream_t host_streams[3] = {nullptr, nullptr, nullptr};  // copies
    cudaStream_t compute_stream = nullptr;                        // transforms, in order
    cudaEvent_t ev_in[3] = {nullptr, nullptr, nullptr}, ev_done[3] = {nullptr, nullptr, nullptr};
    // execs that use the workspace are ordered on the GPU in issue order,
    // whatever their streams: each waits for the last one's event
    std::mutex ws_mu;
    cudaEvent_t ws_last = nullptr;
    size_t workspace_bytes() const
    {
        return c2c.ws_bytes + r2c.c2c.ws_bytes + c2r.c2c.ws_bytes + tc.ws_bytes + col.ws_bytes;
    }
};
