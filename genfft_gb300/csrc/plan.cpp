// plan.cpp -- transform cores (C2C, column, real-input) and their launch
// sequences.  All device work is stream-ordered on the caller's stream.
//
// Path per size (the defaults, each measured on GB300; the environment
// knobs read below override them):
//   C2C  n <= 2^14 (fp32) / 2^13 (fp64)  one fused kernel (c2c_fused.cu)
//        fp32 2^16 .. 2^19               the persistent four-step kernel
//                                        (fourstep.cuh), one launch a batch
//        fp32 2^21 .. 2^24               three passes of short tiles
//                                        (threepass.cu) per workspace group
//        otherwise                       column + row tile launches per
//                                        workspace group (tiles*.cuh), the
//                                        widest TMA-pipelined tile that fits
//   R2C  n/2 within the fused limit      one fused kernel (real.cu)
//        fp32 half spectrum above it     tile column pass + row pass with
//                                        the DIT fused (real_4step.cu)
//        otherwise                       C2C of n/2 + the DIT pass
//   C2R  n/2 within the fused limit      one fused kernel (c2r.cu)
//        otherwise                       pre-pass + C2C of n/2, inverse
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "plan.h"
#include "twiddle.h"

namespace gfft {

bool is_pow2(long long n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog2ll(long long n)
{
    int l = 0;
    while ((1LL << l) < n) l++;
    return l;
}
size_t cplx_bytes(int dtype) { return dtype == GFFT_F64 ? 16 : 8; }

static long long env_ll(const char *name, long long dflt)
{
    const char *v = std::getenv(name);
    return (v && *v) ? std::atoll(v) : dflt;
}

// the four-step inter-pass twiddle W_N^e = hi[e >> lo_bits] * lo[e & (2^lo_bits - 1)]
// of N = 2^logn, cached per (type, N)
static void wn_tables(int dtype, int logn, int *lo_bits, const void **lo, const void **hi)
{
    const long long N = 1LL << logn;
    const int d = dtype;
    auto fill = [d, N](long long count, long long mul) {
        return [d, N, count, mul](void *buf) {
            for (long long e = 0; e < count; e++) {
                if (d == GFFT_F32) forward_root<float>(e * mul, N, &((float *)buf)[2 * e], &((float *)buf)[2 * e + 1]);
                else forward_root<double>(e * mul, N, &((double *)buf)[2 * e], &((double *)buf)[2 * e + 1]);
            }
        };
    };
    *lo_bits = (logn + 1) / 2;
    const std::string key = "4s/" + std::to_string(dtype) + "/" + std::to_string(logn);
    *lo = cached_table(key + "/lo", dtype, 1LL << *lo_bits, fill(1LL << *lo_bits, 1));
    *hi = cached_table(key + "/hi", dtype, N >> *lo_bits, fill(N >> *lo_bits, 1LL << *lo_bits));
}

static const void *tile_table(int dtype, const TileKernel *k, int logl, int c)
{
    return cached_table("tile/" + std::to_string(dtype) + "/" + std::to_string(logl) + "/" + std::to_string(c) +
                            "/" + std::to_string(k->threads),
                        dtype, k->twcount, [k](void *buf) { k->fill(buf); });
}

// ---------------------------------------------------------------------------
// C2C

void C2CCore::init(int dtype_, int logn_, long long batch_hint, int path, bool real_rows)
{
    dtype = dtype_;
    logn = logn_;
    if (logn <= fused_max_logn(dtype)) {
        algo = 1;
        const int d = dtype, l = logn;
        tw = cached_table("fused/" + std::to_string(d) + "/" + std::to_string(l), d, fused_twiddle_count(d, l),
                          [d, l](void *buf) { fused_twiddle_fill(d, l, buf); });
        return;
    }
    if (logn > 24) fail(GFFT_ERR_INVALID_SIZE, "transform length above 2^24 is not supported");
    // N = A * B, A = column-FFT length, B = row-FFT length, both <= 2^12
    logA = logn / 2;
    logB = logn - logA;
    const long long N = 1LL << logn;
    const int d = dtype;
    // inter-pass twiddle W_N^e = tw_hi[e >> lo_bits] * tw_lo[e & (2^lo_bits - 1)]
    wn_tables(dtype, logn, &lo_bits, &tw_lo, &tw_hi);

    // the two-launch tile path: always set up (the persistent kernel needs
    // 16-byte aligned inputs for its tensor copies and uses it otherwise)
    const int maxc = (int)env_ll("GFFT_TILE_MAXC", 16);
    ccol = tile_widest(dtype, TILE_COL_TW4, logA, maxc);
    crow = tile_widest(dtype, TILE_ROW_XPOSE, logB, maxc);
    if (!ccol || !crow) fail(GFFT_ERR_UNSUPPORTED, "no tile kernel for this length");
    kcol = tile_find(dtype, TILE_COL_TW4, logA, ccol);
    krow = tile_find(dtype, TILE_ROW_XPOSE, logB, crow);
    tw_col = tile_table(dtype, kcol, logA, ccol);
    tw_row = tile_table(dtype, krow, logB, crow);

    // three passes of short tiles (threepass.cu), through a workspace of the
    // tile launches' size (GFFT_3PASS=1 / 0 overrides the measured default)
    const ThreePass *tpk = threepass_find(dtype, logn);
    // measured on GB300 (1 GB batches, forward + inverse, GB/s, two passes
    // against three): 2^19 2028 / 1892, 2^20 2136 / 2067, 2^21 2006 / 2117,
    // 2^22 1870 / 2041, 2^23 1789 / 1978, 2^24 1554 / 1934
    const bool tp_default = logn >= 21;
    // (an explicit request for the persistent kernels, GFFT_FS=1 or
    // GFFT_FS_PAIR=1, keeps them)
    const long long want_tp = env_ll("GFFT_3PASS", -1);
    const bool fs_asked = env_ll("GFFT_FS", 0) != 0 || env_ll("GFFT_FS_PAIR", 0) != 0;
    if (tpk && path < 0 && !real_rows && (want_tp > 0 || (want_tp < 0 && tp_default && !fs_asked))) {
        tp = tpk;
        for (int p = 0; p < 3; p++) {
            const int l = p == 0 ? tp->la : p == 1 ? tp->lb : tp->lc;
            const ThreePass *k = tp;
            tp_tw[p] = cached_table("tp/" + std::to_string(d) + "/" + std::to_string(l), d, k->tw_count[p],
                                    [k, p](void *buf) { k->tw_fill[p](buf); });
        }
        wn_tables(dtype, tp->lb + tp->lc, &tp_bits2, &tp_lo2, &tp_hi2);
        const long long budget = env_ll("GFFT_WS_BUDGET_MB", 1024) << 20;
        group = std::max<long long>(1, budget / (N * (long long)cplx_bytes(dtype)));
        group = std::min(group, std::max<long long>(1, batch_hint));
        ws_bytes = (size_t)(group * N) * cplx_bytes(dtype);
        check_cuda(cudaMalloc(&ws, ws_bytes), "cudaMalloc(workspace)");
        algo = 5;
        return;
    }

    int nall = 0;
    const FourStepKernel *const *all = fourstep_variants(dtype, logn, &nall);
    // the pair-packed kernels (fourstep2.cuh) apart from the others
    std::vector<const FourStepKernel *> plain_vars, pair_vars;
    for (int i = 0; i < nall; i++) (all[i]->pair ? pair_vars : plain_vars).push_back(all[i]);
    const bool want_pair = !real_rows && !pair_vars.empty() && env_ll("GFFT_FS_PAIR", 0) != 0;
    const FourStepKernel *const *vars = want_pair ? pair_vars.data() : plain_vars.data();
    int nvar = (int)(want_pair ? pair_vars.size() : plain_vars.size());
    // measured on GB300 (batches of 770 transforms of 2^15 .. 2^18 points,
    // 385 of 2^19, ...): the persistent kernel is the faster one for fp32
    // n = 2^16 .. 2^19; the tile launches for 2^15, for 2^20 and above, and
    // for fp64
    const bool fs_default = dtype == GFFT_F32 && logn >= 16 && logn <= 19;
    const bool use_fs = path >= 0 ? path == 1 : (want_pair || env_ll("GFFT_FS", fs_default ? 1 : 0) != 0);
    std::vector<const FourStepKernel *> dit_vars;
    if (real_rows) {
        // only the variants with a real-input version
        for (int i = 0; i < nvar; i++)
            if (vars[i]->dit) dit_vars.push_back(vars[i]);
        vars = dit_vars.data();
        nvar = (int)dit_vars.size();
        if (!nvar) fail(GFFT_ERR_UNSUPPORTED, "no real-input four-step kernel for this length");
    }
    if (nvar > 0 && use_fs) {
        // persistent four-step (the tile width / stage count GFFT_FS_CC /
        // GFFT_FS_NS name, else the rule below)
        fs = vars[0];
        const long long want_cc = env_ll("GFFT_FS_CC", 0), want_ns = env_ll("GFFT_FS_NS", 0);
        const long long want_thr = env_ll("GFFT_FS_THREADS", 0);
        if (want_cc || want_ns || want_thr) {
            for (int i = 0; i < nvar; i++)
                if ((!want_cc || vars[i]->cc == want_cc) && (!want_ns || vars[i]->ns == want_ns) &&
                    (!want_thr || vars[i]->threads == want_thr)) {
                    fs = vars[i];
                    break;
                }
        } else if (real_rows) {
            // real input: row items of 8 or more rows (runs of 4+ bins per
            // store) with 256 compute threads, else the most rows per item
            const FourStepKernel *best = nullptr;
            for (int i = 0; i < nvar; i++)
                if (vars[i]->threads == 256 + 32 && vars[i]->cr >= 8) {
                    best = vars[i];
                    break;
                }
            if (!best)
                for (int i = 0; i < nvar; i++)
                    if (!best || vars[i]->cr > best->cr) best = vars[i];
            fs = best;
        } else if (want_pair) {
            // pair-packed: the first registered (GFFT_FS_NS picks another)
            fs = vars[0];
        } else {
            // 256 compute threads (two or three CTAs per SM) with column
            // runs of 64 bytes or more, else the widest tile
            for (int i = 0; i < nvar; i++)
                if (vars[i]->threads == 256 + 32 && vars[i]->cc * (int)cplx_bytes(dtype) >= 64) {
                    fs = vars[i];
                    break;
                }
        }
        const int l_a = fs->la, l_b = fs->lb;
        const FourStepKernel *k = fs;
        tw_a = cached_table("fs/" + std::to_string(d) + "/" + std::to_string(l_a) + "/" + std::to_string(k->twa), d,
                            k->twa, [k](void *buf) { k->fill_a(buf); });
        tw_b = cached_table("fs/" + std::to_string(d) + "/" + std::to_string(l_b) + "/" + std::to_string(k->twb), d,
                            k->twb, [k](void *buf) { k->fill_b(buf); });
        fs_real = real_rows;
        fs_nr = real_rows ? fs->nrp : fs->nr;
        fs_grid = fourstep_grid(*fs, real_rows);
        fourstep_schedule((size_t)N * cplx_bytes(dtype), std::max<long long>(1, batch_hint), fs_grid, fs->ns + 1,
                          fs->nc + fs_nr, &fs_slots, &fs_lag);
        group = fs_slots;  // the tile path reuses the ring as its workspace
        ws_bytes = (size_t)fs_slots * (size_t)N * cplx_bytes(dtype);
        check_cuda(cudaMalloc(&ws, ws_bytes), "cudaMalloc(workspace)");
        check_cuda(cudaMalloc(&fs_ctr, (size_t)(2 + 2 * fs_slots) * sizeof(int)), "cudaMalloc(counters)");
        device_error_word();  // allocated now, never inside a stream capture
        algo = 3;
        return;
    }
    // transforms per launch pair, bounded by the workspace budget: fewer,
    // larger launch pairs (measured on GB300, 1 GB against 512 MB: +2 % for
    // n = 2^20 .. 2^23, e.g. 2^22 x 32 in one pair instead of two)
    const long long budget = env_ll("GFFT_WS_BUDGET_MB", 1024) << 20;
    group = std::max<long long>(1, budget / (N * (long long)cplx_bytes(dtype)));
    group = std::min(group, std::max<long long>(1, batch_hint));
    ws_bytes = (size_t)(group * N) * cplx_bytes(dtype);
    check_cuda(cudaMalloc(&ws, ws_bytes), "cudaMalloc(workspace)");
    algo = 2;
}

void C2CCore::release()
{
    if (ws) cudaFree(ws);
    if (fs_ctr) cudaFree(fs_ctr);
    ws = nullptr;
    fs_ctr = nullptr;
}

// transforms per persistent launch: the item count stays far below 2^31
static long long fs_chunk(int items_per_transform, int lag)
{
    return std::max<long long>(1, (1LL << 30) / items_per_transform - lag);
}

int C2CCore::launches(long long batch) const
{
    if (algo == 1) return 1;
    if (algo == 5) return 3 * (int)((batch + group - 1) / group);
    if (algo == 3) {
        const long long chunk = fs_chunk(fs->nc + fs_nr, fs_lag);
        return (int)((batch + chunk - 1) / chunk);
    }
    return 2 * (int)((batch + group - 1) / group);
}

void C2CCore::run(int inverse, const void *in, void *out, long long batch, long long idist, long long odist,
                  long long istride, long long ostride, cudaStream_t st, double scale) const
{
    if (algo == 1) {
        FusedC2CArgs a{in, out, batch, idist, odist, istride, ostride, tw, scale};
        check_cuda(launch_fused_c2c(dtype, logn, inverse, a, st), "launch fused C2C");
        return;
    }
    if (istride != 1 || ostride != 1)
        fail(GFFT_ERR_UNSUPPORTED, "lengths above the fused limit need unit element strides");
    if (algo == 5) {
        const size_t eb5 = cplx_bytes(dtype);
        for (long long g0 = 0; g0 < batch; g0 += group) {
            const long long nb = std::min(group, batch - g0);
            ThreePassArgs a{static_cast<const char *>(in) + (size_t)(g0 * idist) * eb5,
                            static_cast<char *>(out) + (size_t)(g0 * odist) * eb5,
                            ws, nb, idist, odist, {tp_tw[0], tp_tw[1], tp_tw[2]}, tw_lo, tw_hi, lo_bits,
                            tp_lo2, tp_hi2, tp_bits2, scale};
            check_cuda(launch_threepass(*tp, inverse, a, st), "launch three-pass C2C");
        }
        return;
    }
    if (algo == 3 && !fs_real && run_persistent(inverse, in, out, batch, idist, odist, st, scale)) return;
    const long long A = 1LL << logA, B = 1LL << logB, N = A * B;
    const size_t eb = cplx_bytes(dtype);
    const unsigned nmask = (unsigned)(N - 1);
    for (long long g0 = 0; g0 < batch; g0 += group) {
        const long long nb = std::min(group, batch - g0);
        const char *src = static_cast<const char *>(in) + (size_t)(g0 * idist) * eb;
        char *dst = static_cast<char *>(out) + (size_t)(g0 * odist) * eb;
        // column pass: B columns of A points (row stride B) into the workspace
        check_cuda(launch_colpass(*kcol, inverse, B / ccol, nb, src, ws, B, B, B, idist, N, tw_col, tw_lo, tw_hi,
                                  lo_bits, nmask, st),
                   "launch column pass");
        // row pass: A rows of B points, stored transposed (stride A)
        check_cuda(launch_rowpass(*krow, inverse, A / crow, nb, ws, dst, A, B, A, N, odist, tw_row, st, scale),
                   "launch row pass");
    }
}

bool C2CCore::run_persistent(int inverse, const void *in, void *out, long long batch, long long idist,
                             long long odist, cudaStream_t st, double scale, const void *dtw) const
{
    const size_t eb = cplx_bytes(dtype);
    const long long chunk = fs_chunk(fs->nc + fs_nr, fs_lag);
    const long long A = 1LL << fs->la, B = 1LL << fs->lb;
    const unsigned units = (unsigned)(eb / 8);
    for (long long b0 = 0; b0 < batch; b0 += chunk) {
        const long long nb = std::min(chunk, batch - b0);
        FourStepArgs a;
        a.in = static_cast<const char *>(in) + (size_t)(b0 * idist) * eb;
        a.out = static_cast<char *>(out) + (size_t)(b0 * odist) * eb;
        // the pair-packed kernel stores two neighbouring outputs at once
        if (fs->pair && ((((uintptr_t)a.out) & 15u) != 0 || (nb > 1 && (odist & 1) != 0))) {
            if (b0 > 0) fail(GFFT_ERR_ALIGN, "output chunk not 16-byte aligned");
            return false;
        }
        // the input as [batch][A rows][B columns] of 8-byte units
        CUtensorMap map;
        if (!make_tensor_map_3d(&map, a.in, (unsigned long long)B * units, (unsigned long long)A,
                                (unsigned long long)nb, (unsigned long long)(B * eb),
                                (unsigned long long)((nb > 1 ? idist : A * B) * eb), (unsigned)(fs->cc * units),
                                (unsigned)fs->boxr)) {
            if (b0 > 0) fail(GFFT_ERR_ALIGN, "input chunk not 16-byte aligned");
            return false;
        }
        a.ws = ws;
        a.batch = nb;
        a.idist = idist;
        a.odist = odist;
        a.ctr = fs_ctr;
        a.err = device_error_word();
        a.tw_a = tw_a;
        a.tw_b = tw_b;
        a.tw_lo = tw_lo;
        a.tw_hi = tw_hi;
        a.lo_bits = lo_bits;
        a.slots = fs_slots;
        a.lag = fs_lag;
        a.nitems = (int)((nb + fs_lag) * (fs->nc + fs_nr));
        a.scale = scale;
        a.dtw = dtw;
        check_cuda(launch_fourstep(*fs, inverse, map, a, fs_grid, st, fs_real), "launch persistent four-step");
    }
    return true;
}

void C2CCore::run_stalled(const void *in, void *out, cudaStream_t st) const
{
    if (algo != 3) fail(GFFT_ERR_UNSUPPORTED, "not a persistent four-step plan");
    const size_t eb = cplx_bytes(dtype);
    const long long A = 1LL << fs->la, B = 1LL << fs->lb;
    const unsigned units = (unsigned)(eb / 8);
    CUtensorMap map;
    if (!make_tensor_map_3d(&map, in, (unsigned long long)B * units, (unsigned long long)A, 1,
                            (unsigned long long)(B * eb), (unsigned long long)(A * B * eb), (unsigned)(fs->cc * units),
                            (unsigned)fs->boxr))
        fail(GFFT_ERR_ALIGN, "input not 16-byte aligned");
    FourStepArgs a;
    a.in = in;
    a.out = out;
    a.ws = ws;
    a.batch = 0;  // no column tile is ever scheduled ...
    a.idist = a.odist = A * B;
    a.ctr = fs_ctr;
    a.err = device_error_word();
    a.tw_a = tw_a;
    a.tw_b = tw_b;
    a.tw_lo = tw_lo;
    a.tw_hi = tw_hi;
    a.lo_bits = lo_bits;
    a.slots = 1;
    a.lag = 1;  // ... but the row tiles of transform 0 are (phase 1)
    a.nitems = 2 * (fs->nc + fs->nr);
    a.scale = 1.0;
    a.dtw = nullptr;
    check_cuda(launch_fourstep(*fs, 0, map, a, fs_grid, st), "launch persistent four-step");
}

// ---------------------------------------------------------------------------
// column FFTs

void ColCore::init(int dtype_, int logl_, int variant_, bool allow_split, long long max_cols)
{
    dtype = dtype_;
    logl = logl_;
    variant = variant_;
    // Columns of up to 2^12 points run in one launch of tiles.  Longer ones
    // (the reference's FFTVert goes to 2^23 rows, fft_impl_generic.h:281-315)
    // run split; fp32 plain columns of 2^10 .. 2^12 also do on request
    // (GFFT_COL_SPLIT=1): measured on GB300 for 4096 x 4096 the split column
    // pass is no faster (2D C2C 1887 against 1899 GB/s with the one-launch
    // 4096-point tiles)
    constexpr int ONE_LAUNCH_MAX = 12;
    const bool opt_split = allow_split && variant == TILE_COL_PLAIN && dtype == GFFT_F32 && logl >= 10 &&
                           env_ll("GFFT_COL_SPLIT", 0) != 0;
    if (logl > ONE_LAUNCH_MAX || opt_split) {
        if (logl > 24) fail(GFFT_ERR_INVALID_SIZE, "column length above 2^24 is not supported");
        rows_bitrev = variant == TILE_COL_BITREV;
        herm_fill = variant == TILE_COL_HERM;
        l1 = logl / 2;
        l2 = logl - l1;
        c1 = tile_widest(dtype, TILE_COL_TWB, l1, 64);
        c2 = tile_widest(dtype, TILE_COL_PLAIN, l2, 64);
        ka = c1 ? tile_find(dtype, TILE_COL_TWB, l1, c1) : nullptr;
        kb = c2 ? tile_find(dtype, TILE_COL_PLAIN, l2, c2) : nullptr;
        if (!ka || !kb) fail(GFFT_ERR_UNSUPPORTED, "no split column kernels for this length");
        tw_a = tile_table(dtype, ka, l1, c1);
        tw_b = tile_table(dtype, kb, l2, c2);
        wn_tables(dtype, logl, &lo_bits, &tw_lo, &tw_hi);
        // bands of columns, H x band elements of scratch each
        // (GFFT_COL_BAND_MB): measured on GB300 at 4096 x 4096 the launch
        // count dominates, not the scratch's L2 residency (2D C2C 1238 /
        // 1592 / 1747 / 1887 GB/s with 16 / 32 / 64 / 128 MB bands), so the
        // default is 128 MB.  A band holds at least one tile of each step
        // and at most the columns there are.
        const long long H = 1LL << logl;
        const long long band_bytes = std::max<long long>(1, env_ll("GFFT_COL_BAND_MB", 128)) << 20;
        const long long q = std::max(c1, c2);
        band = std::max<long long>(q, (band_bytes / (H * (long long)cplx_bytes(dtype))) / q * q);
        if (max_cols > 0) band = std::min(band, max_cols);
        ws_bytes = (size_t)(H * band) * cplx_bytes(dtype);
        check_cuda(cudaMalloc(&scratch, ws_bytes), "cudaMalloc(column scratch)");
        split = true;
        return;
    }
    c = tile_widest(dtype, variant, logl, (int)env_ll("GFFT_COL_MAXC", 16));
    if (!c) fail(GFFT_ERR_UNSUPPORTED, "no column kernel for this length");
    k = tile_find(dtype, variant, logl, c);
    tw = tile_table(dtype, k, logl, c);
}

void ColCore::release()
{
    if (scratch) cudaFree(scratch);
    scratch = nullptr;
}

void ColCore::run(int inverse, const void *in, void *out, long long ncols, long long ld_in, long long ld_out,
                  long long batch, long long idist, long long odist, cudaStream_t st, double scale) const
{
    if (!split) {
        check_cuda(launch_colpass(*k, inverse, (ncols + c - 1) / c, batch, in, out, ncols, ld_in, ld_out, idist,
                                  odist, tw, nullptr, nullptr, 0, 0u, st, scale),
                   "launch column FFT");
        return;
    }
    // rows in bit-reversed order: into natural order first (into out, or
    // in place), then the plain split in place on out
    if (rows_bitrev) {
        check_cuda(launch_rows_bitrev(dtype, in, out, logl, ncols, ld_in, ld_out, batch, idist, odist, st),
                   "launch row bit reversal");
        in = out;
        ld_in = ld_out;
        idist = odist;
    }
    // Column FFT of H = H1 H2 points with rows r = H2 r1 + r2 and bins
    // k = k1 + H1 k2 (the four-step split along the column):
    //   A: for each r2 (batch index), H1-point FFTs over r1, times
    //      W_H^(r2 k1), into scratch[k1][r2][column];
    //   B: for each k1 (batch index), H2-point FFTs over r2 of the scratch,
    //      into rows k1 + H1 k2 of the output.
    // A band of columns at a time (the scratch holds one band); A reads
    // every row of its band before B writes it, so out may be in.
    const long long H1 = 1LL << l1, H2 = 1LL << l2;
    const size_t eb = cplx_bytes(dtype);
    for (long long b2 = 0; b2 < batch; b2++) {
        for (long long c0 = 0; c0 < ncols; c0 += band) {
            const long long wb = std::min(band, ncols - c0);
            const char *src = static_cast<const char *>(in) + (size_t)(b2 * idist + c0) * eb;
            char *dst = static_cast<char *>(out) + (size_t)(b2 * odist + c0) * eb;
            check_cuda(launch_colpass(*ka, inverse, (wb + c1 - 1) / c1, H2, src, scratch, wb, H2 * ld_in, H2 * wb,
                                      ld_in, wb, tw_a, tw_lo, tw_hi, lo_bits, (unsigned)((H1 * H2) - 1), st, 1.0),
                       "launch split column pass A");
            check_cuda(launch_colpass(*kb, inverse, (wb + c2 - 1) / c2, H1, scratch, dst, wb, wb, H1 * ld_out,
                                      H2 * wb, ld_out, tw_b, nullptr, nullptr, 0, 0u, st, scale),
                       "launch split column pass B");
        }
    }
    // full-width real 2D: ncols = W/2 + 1 columns done, the rest mirrored
    if (herm_fill)
        check_cuda(launch_herm_fill(dtype, out, H1 * H2, 2 * (ncols - 1), ld_out, batch, odist, st),
                   "launch Hermitian fill");
}

// ---------------------------------------------------------------------------
// real input

void R2CCore::init(int dtype_, int logn_, int half_, long long batch_hint)
{
    dtype = dtype_;
    logn = logn_;
    half = half_;
    if (logn == 0) {
        algo = 0;
        return;
    }
    const int d = dtype, l = logn, lh = logn - 1;
    dtw = cached_table("dit/" + std::to_string(d) + "/" + std::to_string(l), d, (1LL << lh) + 1,
                       [d, l](void *buf) { dit_twiddle_fill(d, l, buf); });
    if (lh <= r2c_fused_max_logh(dtype)) {
        algo = 1;
        tw = cached_table("r2c/" + std::to_string(d) + "/" + std::to_string(lh), d, r2c_twiddle_count(d, lh),
                          [d, lh](void *buf) { r2c_twiddle_fill(d, lh, buf); });
        return;
    }
    // the DIT fused into the row pass of a four-step split of n/2 (fp32)
    const RowDitKernel *k = rowdit_find(dtype, lh - lh / 2);
    if (k && env_ll("GFFT_R2C_FUSED_DIT", 1) != 0) {
        rowdit = k;
        tw_rowdit = cached_table("rowdit/" + std::to_string(d) + "/" + std::to_string(k->logb), d, k->twcount,
                                 [k](void *buf) { k->fill(buf); });
        // the persistent four-step kernel's real-input version (its row
        // items apply the DIT), on request (GFFT_R2C_FS=1): measured on
        // GB300 at n = 2^16 .. 2^22 (batches of 512 MB) it is 2-20 % slower
        // than the tile launches below, which stay the default
        int nvar = 0;
        const FourStepKernel *const *vars = fourstep_variants(dtype, lh, &nvar);
        bool has_dit = false;
        for (int i = 0; i < nvar; i++) has_dit = has_dit || vars[i]->dit;
        if (has_dit && env_ll("GFFT_R2C_FS", 0) != 0) {
            c2c.init(dtype, lh, batch_hint, 1, true);
            if (c2c.algo == 3 && c2c.fs_real) {
                algo = 4;
                return;
            }
            c2c.release();
            c2c = C2CCore();
        }
        c2c.init(dtype, lh, batch_hint, 0);  // column pass, tables and workspace of the tile path
        algo = 3;
        return;
    }
    algo = 2;
    c2c.init(dtype, lh, batch_hint);
}

int R2CCore::launches(long long batch) const
{
    if (algo == 2) return c2c.launches(batch) + 1;
    if (algo == 3 || algo == 4) return c2c.launches(batch);
    return 1;
}

void R2CCore::run(const void *in, void *out, long long batch, long long idist, long long odist, cudaStream_t st,
                  int mode, double scale) const
{
    if (mode < 0) mode = half ? 0 : 1;
    if (algo == 0) {
        check_cuda(launch_r2c_one(dtype, in, out, batch, idist, odist, st, scale), "launch R2C n=1");
    } else if (algo == 1) {
        check_cuda(launch_r2c_fused(dtype, logn - 1, mode, in, out, batch, idist, odist, tw, dtw, st, scale),
                   "launch fused R2C");
    } else if (algo == 4 && mode == 0 && c2c.run_persistent(0, in, out, batch, idist / 2, odist, st, scale, dtw)) {
        // one persistent launch: column items, then row items that apply
        // the DIT adjustment and store the half spectrum
    } else if ((algo == 3 || algo == 4) && mode == 0) {
        // column pass of the n/2-point split into the workspace, then the
        // row pass with the DIT adjustment fused, straight into the spectrum
        // (also the persistent plan's path for inputs its tensor copies
        // cannot read)
        const long long A = 1LL << c2c.logA, B = 1LL << c2c.logB, N = A * B;
        const size_t eb = cplx_bytes(dtype);
        for (long long g0 = 0; g0 < batch; g0 += c2c.group) {
            const long long nb = std::min(c2c.group, batch - g0);
            const char *src = static_cast<const char *>(in) + (size_t)(g0 * (idist / 2)) * eb;
            char *dst = static_cast<char *>(out) + (size_t)(g0 * odist) * eb;
            check_cuda(launch_colpass(*c2c.kcol, 0, B / c2c.ccol, nb, src, c2c.ws, B, B, B, idist / 2, N, c2c.tw_col,
                                      c2c.tw_lo, c2c.tw_hi, c2c.lo_bits, (unsigned)(N - 1), st),
                       "launch column pass");
            check_cuda(launch_rowpass_dit(*rowdit, c2c.ws, dst, A, nb, N, odist, tw_rowdit, dtw, st, scale),
                       "launch row pass with DIT");
        }
    } else {
        const long long H = 1LL << (logn - 1);
        // n reals are n/2 complex; transform them into the output buffer,
        // then adjust in place (the reference's order, FFTReal.h:209-211)
        c2c.run(0, in, out, batch, idist / 2, odist, 1, 1, st);
        check_cuda(launch_dit(dtype, mode, out, out, H, batch, odist, odist, dtw, st, scale), "launch DIT pass");
    }
}

// ---------------------------------------------------------------------------
// half-spectrum inverse

void C2RCore::init(int dtype_, int logn_, long long batch_hint)
{
    dtype = dtype_;
    logn = logn_;
    if (logn == 0) {
        algo = 0;
        return;
    }
    const int d = dtype, l = logn, lh = logn - 1;
    dtw = cached_table("dit/" + std::to_string(d) + "/" + std::to_string(l), d, (1LL << lh) + 1,
                       [d, l](void *buf) { dit_twiddle_fill(d, l, buf); });
    if (c2r_fused_fits(dtype, lh, 0)) {
        // the fused C2R runs the same Stockham plan (points per thread) as
        // the fused R2C of this half length, so it shares that table
        algo = 1;
        tw = cached_table("r2c/" + std::to_string(d) + "/" + std::to_string(lh), d, r2c_twiddle_count(d, lh),
                          [d, lh](void *buf) { r2c_twiddle_fill(d, lh, buf); });
        if (!c2r_fused_fits(dtype, lh, 2)) {
            fold_split = true;
            c2c.init(dtype, lh, batch_hint);
        }
        return;
    }
    algo = 2;
    c2c.init(dtype, lh, batch_hint);
}

int C2RCore::launches(long long batch) const
{
    if (algo == 2) return c2c.launches(batch) + 1;
    return 1;
}

void C2RCore::run(const void *in, void *out, long long batch, long long idist, long long odist, int wmode,
                  cudaStream_t st, double scale) const
{
    if (algo == 0) {
        check_cuda(launch_c2r_one(dtype, in, out, batch, idist, odist, st, scale), "launch C2R n=1");
    } else if (algo == 1 && !(fold_split && wmode == 2)) {
        check_cuda(launch_c2r_fused(dtype, logn - 1, wmode, in, out, batch, idist, odist, tw, dtw, st, scale),
                   "launch fused C2R");
    } else {
        const long long H = 1LL << (logn - 1);
        // Z' (n/2 complex = the n output reals) into the output buffer, then
        // the unscaled inverse C2C of n/2 points in place
        check_cuda(launch_c2r_pre(dtype, wmode, in, out, H, batch, idist, odist / 2, dtw, st), "launch C2R pre-pass");
        c2c.run(1, out, out, batch, odist / 2, odist / 2, 1, 1, st, scale);
    }
}

}  // namespace gfft
