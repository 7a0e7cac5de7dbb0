// tc.cu -- split-precision tensor-core C2C (fp32 in/out): radix-16 DFT
// blocks computed as dense FP16 or BF16 products on the 5th-generation
// tensor cores (tcgen05.mma, FP32 accumulation in tensor memory).
//
// No counterpart in the reference, whose butterflies are scalar/SIMD FP32
// (fft_impl_generic.h:36-63); results follow its conventions (forward
// exp(-2 pi i jk/n), unscaled inverse) and are checked against an FP64 DFT.
//
// One CTA (256 threads) owns a tile of 4096 points at a time.  Every
// radix-16 stage of the tile is 256 independent 16-point DFTs; thread m owns
// vector m:
//   1. gathers its 16 complex points (fp32) from the tile in shared memory
//      and multiplies them by the stage's twiddles with a compensated
//      product (twiddles stored as fp32 hi + lo pairs made in FP64);
//   2. splits the 32 reals into 16-bit terms: FP16 hi + lo after scaling the
//      vector by a power of two (so its largest component sits in
//      [2^14, 2^15): no overflow, and the lo terms keep 11 more bits), or
//      BF16 hi + mid + lo (FP32 range, 24 bits, no scaling);
//   3. stores each term as row m of an A operand (K = 32: re/im of the 16
//      points) in the canonical no-swizzle K-major layout;
// then one thread issues, per 128-row half, the MMAs of the products
//   FP16: A_hi B_hi + A_lo B_hi + A_hi B_lo             (3 x K=32)
//   BF16: the six products of total order <= 2         (6 x K=32)
// against the split 32 x 32 real form of the DFT-16 matrix, accumulating in
// FP32 in tensor memory (M = 128, N = 32 per half): the hi x hi products in
// one accumulator, the smaller correction products in another, added in FP32
// on the CUDA cores (the tensor core's accumulator truncates; keeping the
// large and small terms apart keeps that error at the corrections' scale).
// Thread m reads its row back with tcgen05.ld, undoes the scale and scatters
// the 16 outputs to the tile (or to global memory after the last stage).
//
// Kinds: K256  - 16 transforms of 256 points per tile (2 stages)
//        K4096 - one transform of 4096 points per tile (3 stages)
//        KCOL / KROW - the column and row passes of n = 65536 = 256 x 256
//        (four-step, W_65536 twiddle after the column pass).
// Every twiddle comes from two 256-entry (hi, lo) tables in shared memory:
// W_N^e = W_256^(e >> s) * W_N^(e mod 2^s), two compensated products.
// Tiles arrive by TMA (bulk copies; a 3D tensor box for KCOL) into a dense
// stage buffer: the copy of the next tile starts as soon as stage 0 of the
// current one has gathered its inputs, and lands while the later stages run.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "internal.h"
#include "plan.h"
#include "stockham.cuh"
#include "tc.cuh"
#include "tiles_registry.h"
#include "twiddle.h"

namespace gfft {
namespace tcf {

constexpr int THREADS = 256;
constexpr int A_TERM = 256 * 64;             // bytes: 256 rows x 32 16-bit values
constexpr int A_HALF = 128 * 64;             // bytes of one 128-row half
constexpr int B_TERM = 32 * 64;              // bytes: 32 rows x 32 16-bit values
constexpr int XELEMS = 4096 + 4096 / 16 + 2; // padded tile (spad<float>), even
constexpr uint32_t LBO = 128, SBO = 512;     // core-matrix strides of both operands
constexpr uint32_t TMEM_COLS = 128;           // 2 halves x (main + correction) x 32 columns

enum Kind { K256 = 0, K4096 = 1, KCOL = 2, KROW = 3 };

// split terms of the data (TA) and of the DFT matrix (TB), and the products
template <bool BF16>
struct Prec {
    static constexpr int TA = 2, TB = 2, NP = 3;
    __device__ static int pa(int i) { return i == 1 ? 1 : 0; }  // (0,0) (1,0) (0,1)
    __device__ static int pb(int i) { return i == 2 ? 1 : 0; }
};
template <>
struct Prec<true> {
    static constexpr int TA = 3, TB = 3, NP = 6;
    // (0,0) (1,0) (0,1) (2,0) (1,1) (0,2)
    __device__ static int pa(int i) { return i == 1 ? 1 : i == 3 ? 2 : i == 4 ? 1 : 0; }
    __device__ static int pb(int i) { return i == 2 ? 1 : i == 4 ? 1 : i == 5 ? 2 : 0; }
};

template <bool BF16>
struct Smem {
    static constexpr int B_OFF = Prec<BF16>::TA * A_TERM;
    static constexpr int STG_OFF = B_OFF + Prec<BF16>::TB * B_TERM;  // incoming tile, dense (TMA)
    static constexpr int X_OFF = STG_OFF + 4096 * 8;                  // inter-stage tile, padded
    static constexpr int T_OFF = X_OFF + XELEMS * 8;     // W_256^e (hi, lo) pairs
    static constexpr int T2_OFF = T_OFF + 512 * 8;       // W_N^e, e < 256 (KCOL) / W_4096^e, e < 16 (K4096)
    static constexpr int BAR_OFF = T2_OFF + 512 * 8;
    static constexpr int BYTES = BAR_OFF + 24;  // MMA barrier, load barrier, TMEM address
    static constexpr int MIN_BLOCKS = (228 * 1024) / (BYTES + 1024);
};

struct TcArgs {
    const float2 *in;
    float2 *out;
    long long ntiles, batch, idist, odist;
    const void *bmat;      // TB split terms of the DFT-16 matrix, canonical layout
    const float2 *tw256;   // W_256^e, (hi, lo) pairs
    const float2 *tw2;     // W_4096^e, e < 16 (K4096) or W_65536^e, e < 256 (KCOL): (hi, lo) pairs
    unsigned *err;
    int tma;      // 1: TMA copies of the tiles (16-byte aligned), 0: thread loads
    float scale;  // applied to every output of the last pass (norm= scaling)
};

__device__ __forceinline__ int xpad(int i) { return i + (i >> 4); }

// v * w with w = h + l (fp32 pair), conjugated for the inverse
template <bool INV>
__device__ __forceinline__ float2 ctw(float2 v, float2 h, float2 l)
{
    if (INV) {
        h.y = -h.y;
        l.y = -l.y;
    }
    const float lr = fmaf(v.x, l.x, -v.y * l.y);
    const float li = fmaf(v.x, l.y, v.y * l.x);
    return make_float2(fmaf(v.x, h.x, fmaf(-v.y, h.y, lr)), fmaf(v.x, h.y, fmaf(v.y, h.x, li)));
}

// scale + split + store row m of every A term; returns the inverse scale
template <bool BF16>
__device__ __forceinline__ float split_store(const float2 (&v)[16], unsigned char *Aop, int m)
{
    float sc = 1.f, isc = 1.f;
    if (!BF16) {
        float mx = 0.f;
#pragma unroll
        for (int r = 0; r < 16; r++) mx = fmaxf(mx, fmaxf(fabsf(v[r].x), fabsf(v[r].y)));
        int e = (__float_as_int(mx) >> 23) & 0xFF;
        e = max(e, 15);
        sc = __int_as_float((268 - e) << 23);   // 2^(141 - e): max component in [2^14, 2^15)
        isc = __int_as_float((e - 14) << 23);   // 2^(e - 141)
    }
    unsigned char *row = Aop + (m >> 7) * A_HALF + ((m & 127) >> 3) * 512 + (m & 7) * 16;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        uint32_t w0[4], w1[4], w2[4];
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const float x = v[4 * j + p].x * sc, y = v[4 * j + p].y * sc;
            if (!BF16) {
                const __half2 h = __floats2half2_rn(x, y);
                const float2 f = __half22float2(h);
                const __half2 l = __floats2half2_rn(x - f.x, y - f.y);
                w0[p] = *reinterpret_cast<const uint32_t *>(&h);
                w1[p] = *reinterpret_cast<const uint32_t *>(&l);
            } else {
                const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
                const float2 f = __bfloat1622float2(h);
                const float rx = x - f.x, ry = y - f.y;
                const __nv_bfloat162 md = __floats2bfloat162_rn(rx, ry);
                const float2 g = __bfloat1622float2(md);
                const __nv_bfloat162 l = __floats2bfloat162_rn(rx - g.x, ry - g.y);
                w0[p] = *reinterpret_cast<const uint32_t *>(&h);
                w1[p] = *reinterpret_cast<const uint32_t *>(&md);
                w2[p] = *reinterpret_cast<const uint32_t *>(&l);
            }
        }
        *reinterpret_cast<uint4 *>(row + j * LBO) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
        *reinterpret_cast<uint4 *>(row + A_TERM + j * LBO) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
        if (BF16) *reinterpret_cast<uint4 *>(row + 2 * A_TERM + j * LBO) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
    }
    return isc;
}

// thread 0: start the copy of tile w into the dense stage buffer (TMA)
template <int KIND>
__device__ __forceinline__ void issue_tile(const CUtensorMap *map, const TcArgs &a, long long w, float2 *stg,
                                           uint64_t *tbar)
{
    if (KIND == K4096) {
        mbar_arrive_expect_tx(tbar, 32768u);
        bulk_load(stg, a.in + w * a.idist, 32768u, tbar);
    } else if (KIND == K256) {
        const long long t0 = w * 16;
        const int valid = (int)(a.batch - t0 < 16 ? a.batch - t0 : 16);
        mbar_arrive_expect_tx(tbar, (uint32_t)valid * 2048u);
        for (int sl = 0; sl < valid; sl++) bulk_load(stg + sl * 256, a.in + (t0 + sl) * a.idist, 2048u, tbar);
    } else if (KIND == KROW) {
        mbar_arrive_expect_tx(tbar, 32768u);
        bulk_load(stg, a.in + (w >> 4) * a.idist + (w & 15) * 16 * 256, 32768u, tbar);
    } else {  // KCOL: 256 rows x 16 columns, one tensor box
        mbar_arrive_expect_tx(tbar, 32768u);
        tensor_load_3d(stg, map, (int)((w & 15) * 16), 0, (int)(w >> 4), tbar);
    }
}

template <bool BF16, int KIND, bool INV>
__global__ void __launch_bounds__(THREADS, Smem<BF16>::MIN_BLOCKS)
    k_tc(const __grid_constant__ CUtensorMap map, const TcArgs a)
{
    using P = Prec<BF16>;
    using L = Smem<BF16>;
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *const Aop = sm;
    unsigned char *const Bop = sm + L::B_OFF;
    float2 *const STG = reinterpret_cast<float2 *>(sm + L::STG_OFF);
    float2 *const X = reinterpret_cast<float2 *>(sm + L::X_OFF);
    float2 *const T = reinterpret_cast<float2 *>(sm + L::T_OFF);
    float2 *const T2 = reinterpret_cast<float2 *>(sm + L::T2_OFF);
    uint64_t *const bar = reinterpret_cast<uint64_t *>(sm + L::BAR_OFF);
    uint64_t *const tbar = bar + 1;
    uint32_t *const s_taddr = reinterpret_cast<uint32_t *>(sm + L::BAR_OFF + 16);
    const int tid = threadIdx.x;

    // ---- set-up: DFT matrix terms and W_256 to shared memory, barrier, TMEM
    {
        const uint4 *src = static_cast<const uint4 *>(a.bmat);
        uint4 *dst = reinterpret_cast<uint4 *>(Bop);
        for (int i = tid; i < P::TB * B_TERM / 16; i += THREADS) dst[i] = src[i];
        for (int i = tid; i < 512; i += THREADS) T[i] = a.tw256[i];
        if (KIND == KCOL)
            for (int i = tid; i < 512; i += THREADS) T2[i] = a.tw2[i];
        if (KIND == K4096)
            for (int i = tid; i < 32; i += THREADS) T2[i] = a.tw2[i];
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init(tbar, 1);
        fence_barrier_init();
    }
    if (tid < 32) tc::tmem_alloc(s_taddr, TMEM_COLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = *s_taddr;
    // this thread's accumulator row: lane 32 (warp % 4) + lane; each 128-row
    // half owns 64 columns: the hi x hi products in the first 32, the
    // correction products in the next 32
    const uint32_t my_tmem = taddr + ((uint32_t)((tid >> 5) & 3) * 32u << 16) + (uint32_t)(tid >> 7) * 64u;
    const uint32_t a_s = smem_u32(Aop), b_s = smem_u32(Bop);
    constexpr uint32_t IDESC = tc::idesc_f16(BF16, 128, 32);
    constexpr int S = KIND == K4096 ? 3 : 2;
    const int m = tid;
    uint32_t phase = 0, tphase = 0;
    bool ok = true;
    if (a.tma && tid == 0 && blockIdx.x < a.ntiles) issue_tile<KIND>(&map, a, blockIdx.x, STG, tbar);

    for (long long w = blockIdx.x; w < a.ntiles; w += gridDim.x) {
        if (a.tma) {
            // the copy of this tile, started during the previous one
            ok = __syncthreads_and(mbar_wait(tbar, tphase));
            tphase ^= 1u;
            if (!ok) break;
        } else {
            // thread loads into the dense stage buffer (all 16 in flight
            // before the first store)
            float2 ld[16];
            if (KIND == K4096) {
                const float2 *src = a.in + w * a.idist;
#pragma unroll
                for (int q = 0; q < 16; q++) ld[q] = __ldcs(src + tid + 256 * q);
            } else if (KIND == K256 || KIND == KROW) {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int i = tid + 256 * q, sl = i >> 8, pos = i & 255;
                    ld[q] = make_float2(0.f, 0.f);
                    if (KIND == K256) {
                        const long long t = w * 16 + sl;
                        if (t < a.batch) ld[q] = __ldcs(a.in + t * a.idist + pos);
                    } else {
                        const long long t = w >> 4;
                        ld[q] = __ldcs(a.in + t * a.idist + ((w & 15) * 16 + sl) * 256 + pos);
                    }
                }
            } else {  // KCOL: X[a * 16 + c] = x[a * 256 + c0 + c]
                const long long t = w >> 4, c0 = (w & 15) * 16;
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int i = tid + 256 * q;
                    ld[q] = __ldcs(a.in + t * a.idist + (i >> 4) * 256 + c0 + (i & 15));
                }
            }
#pragma unroll
            for (int q = 0; q < 16; q++) STG[tid + 256 * q] = ld[q];
            __syncthreads();
        }

#pragma unroll 1
        for (int s = 0; s < S; s++) {
            // ---- gather + stage twiddle
            float2 v[16];
            const int base = (KIND == K256 || KIND == KROW) ? (m >> 4) * 256 + (m & 15) : m;
            const int step = (KIND == K256 || KIND == KROW) ? 16 : 256;
            if (s == 0) {
#pragma unroll
                for (int r = 0; r < 16; r++) v[r] = STG[base + step * r];
            } else {
#pragma unroll
                for (int r = 0; r < 16; r++) v[r] = X[xpad(base + step * r)];
            }
            if (s == 1) {
                const int jj = (KIND == KCOL) ? (m >> 4) : (m & 15);  // W_256^(jj r)
#pragma unroll
                for (int r = 1; r < 16; r++) v[r] = ctw<INV>(v[r], T[2 * (jj * r)], T[2 * (jj * r) + 1]);
            } else if (s == 2) {  // K4096 last pass: W_4096^(m r) = W_256^(e >> 4) W_4096^(e & 15)
#pragma unroll
                for (int r = 1; r < 16; r++) {
                    const int e = m * r;
                    v[r] = ctw<INV>(ctw<INV>(v[r], T[2 * (e >> 4)], T[2 * (e >> 4) + 1]), T2[2 * (e & 15)],
                                    T2[2 * (e & 15) + 1]);
                }
            }
            const float isc = split_store<BF16>(v, Aop, m);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            // ---- one thread: the MMAs of both 128-row halves
            if (tid == 0) {
                tc::fence_after_sync();
#pragma unroll
                for (int g = 0; g < 2; g++) {
#pragma unroll
                    for (int pi = 0; pi < P::NP; pi++) {
#pragma unroll
                        for (int kc = 0; kc < 2; kc++) {
                            const uint64_t ad =
                                tc::smem_desc(a_s + P::pa(pi) * A_TERM + g * A_HALF + kc * 2 * LBO, LBO, SBO);
                            const uint64_t bd = tc::smem_desc(b_s + P::pb(pi) * B_TERM + kc * 2 * LBO, LBO, SBO);
                            // hi x hi into the main accumulator, the rest into
                            // the correction accumulator
                            const uint32_t d = taddr + (uint32_t)g * 64u + (pi > 0 ? 32u : 0u);
                            tc::mma_f16(d, ad, bd, IDESC, pi > 1 || kc > 0);
                        }
                    }
                }
                tc::commit(bar);
                // every thread has gathered this tile: refill the stage buffer
                if (s == 0 && a.tma && w + gridDim.x < a.ntiles) {
                    fence_proxy_async_smem();
                    issue_tile<KIND>(&map, a, w + gridDim.x, STG, tbar);
                }
            }
            ok = __syncthreads_and(mbar_wait(bar, phase));
            phase ^= 1u;
            if (!ok) break;
            tc::fence_after_sync();
            // main + correction, summed in FP32 with round-to-nearest outside
            // the tensor core (its accumulator does not round to nearest)
            float2 o[16];
            {
                float r32[32];
                tc::tmem_ld32(my_tmem, r32);
#pragma unroll
                for (int k = 0; k < 16; k++) o[k] = make_float2(r32[2 * k], r32[2 * k + 1]);
                tc::tmem_ld32(my_tmem + 32u, r32);
#pragma unroll
                for (int k = 0; k < 16; k++)
                    o[k] = make_float2((o[k].x + r32[2 * k]) * isc, (o[k].y + r32[2 * k + 1]) * isc);
            }
            tc::fence_before_sync();

            // ---- scatter (the gathers of this stage are done: every thread
            // passed the MMA barrier)
            if (s < S - 1) {
                if (KIND == K4096) {
                    if (s == 0) {
#pragma unroll
                        for (int k = 0; k < 16; k++) X[xpad(16 * m + k)] = o[k];
                    } else {
#pragma unroll
                        for (int k = 0; k < 16; k++) X[xpad((m >> 4) * 256 + (m & 15) + 16 * k)] = o[k];
                    }
                } else if (KIND == KCOL) {
#pragma unroll
                    for (int k = 0; k < 16; k++) X[xpad(256 * (m >> 4) + 16 * k + (m & 15))] = o[k];
                } else {
#pragma unroll
                    for (int k = 0; k < 16; k++) X[xpad((m >> 4) * 256 + 16 * (m & 15) + k)] = o[k];
                }
            } else {
                if (KIND == K4096) {
                    float2 *dst = a.out + w * a.odist + m;
#pragma unroll
                    for (int k = 0; k < 16; k++) __stcs(dst + 256 * k, make_float2(o[k].x * a.scale, o[k].y * a.scale));
                } else if (KIND == K256) {
                    const long long t = w * 16 + (m >> 4);
                    if (t < a.batch) {
                        float2 *dst = a.out + t * a.odist + (m & 15);
#pragma unroll
                        for (int k = 0; k < 16; k++) __stcs(dst + 16 * k, make_float2(o[k].x * a.scale, o[k].y * a.scale));
                    }
                } else if (KIND == KCOL) {
                    // X[K] of column c, K = j + 16 k, times W_65536^(col K)
                    const long long t = w >> 4;
                    const int col = (int)((w & 15) * 16) + (m & 15), j = m >> 4;
                    float2 *dst = a.out + t * a.odist + col;
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        // W_65536^e = W_256^(e >> 8) W_65536^(e & 255)
                        const int K = j + 16 * k;
                        const int e = (col * K) & 65535;
                        dst[(long long)K * 256] = ctw<INV>(ctw<INV>(o[k], T[2 * (e >> 8)], T[2 * (e >> 8) + 1]),
                                                           T2[2 * (e & 255)], T2[2 * (e & 255) + 1]);
                    }
                } else {  // KROW: transpose through X, then 16-element runs
#pragma unroll
                    for (int k = 0; k < 16; k++) X[xpad(((m & 15) + 16 * k) * 16 + (m >> 4))] = o[k];
                    __syncthreads();
                    const long long t = w >> 4, r0 = (w & 15) * 16;
                    float2 *dst = a.out + t * a.odist + r0;
#pragma unroll 4
                    for (int q = 0; q < 16; q++) {
                        const int i = tid + 256 * q;
                        const float2 z = X[xpad(i)];
                        __stcs(dst + (i & 15) + (long long)(i >> 4) * 256, make_float2(z.x * a.scale, z.y * a.scale));
                    }
                }
            }
            __syncthreads();  // X, the A operand and the accumulator are reused
        }
        if (!ok) break;
    }
    if (!ok) {
        if (tid == 0) atomicOr(a.err, DEV_ERR_TC_TIMEOUT);
        mbar_wait(bar, phase ^ 1u);  // let an MMA still in flight finish (bounded)
        if (a.tma) mbar_wait(tbar, tphase);  // and a tile copy (bounded)
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid < 32) tc::tmem_dealloc(taddr, TMEM_COLS);
}

// ---------------------------------------------------------------------------
// host side

// the 32 x 32 real DFT-16 matrix (D = A B^T, K and N both interleaved re/im),
// split into 16-bit terms in the canonical no-swizzle K-major layout
void fill_bmat(bool bf16, bool inv, unsigned char *out)
{
    const int terms = bf16 ? 3 : 2;
    std::memset(out, 0, (size_t)terms * B_TERM);
    for (int n = 0; n < 32; n++)
        for (int k = 0; k < 32; k++) {
            const int q = n >> 1, r = k >> 1;
            double c, s;
            exact_root((long long)((q * r) & 15), 16, &c, &s);  // cos, sin of 2 pi q r / 16
            const double sg = inv ? 1.0 : -1.0;                   // F = c + sg i s
            double val;
            if ((n & 1) == 0) val = (k & 1) == 0 ? c : -sg * s;   // re: c xr - sg s xi
            else val = (k & 1) == 0 ? sg * s : c;                 // im: sg s xr + c xi
            const size_t off = (size_t)(n >> 3) * 512 + (size_t)(k >> 3) * 128 + (size_t)(n & 7) * 16 + (size_t)(k & 7) * 2;
            double rest = val;
            for (int t = 0; t < terms; t++) {
                uint16_t bits;
                float fv;
                if (!bf16) {
                    const __half h = __float2half_rn((float)rest);
                    fv = __half2float(h);
                    std::memcpy(&bits, &h, 2);
                } else {
                    const __nv_bfloat16 h = __float2bfloat16_rn((float)rest);
                    fv = __bfloat162float(h);
                    std::memcpy(&bits, &h, 2);
                }
                std::memcpy(out + (size_t)t * B_TERM + off, &bits, 2);
                rest -= (double)fv;
            }
        }
}

// W_M^e for e < count as (hi, lo) fp32 pairs
void fill_pairs(long long M, long long count, float *out)
{
    for (long long e = 0; e < count; e++) {
        double c, s;
        exact_root(e, M, &c, &s);
        const double re = c, im = -s;
        const float hr = (float)re, hi = (float)im;
        out[4 * e + 0] = hr;
        out[4 * e + 1] = hi;
        out[4 * e + 2] = (float)(re - (double)hr);
        out[4 * e + 3] = (float)(im - (double)hi);
    }
}

template <bool BF16, int KIND, bool INV>
const void *kfn()
{
    return (const void *)&k_tc<BF16, KIND, INV>;
}

const void *kernel_for(bool bf16, int kind, bool inv)
{
    static const void *tab[2][4][2] = {
        {{kfn<false, 0, false>(), kfn<false, 0, true>()}, {kfn<false, 1, false>(), kfn<false, 1, true>()},
         {kfn<false, 2, false>(), kfn<false, 2, true>()}, {kfn<false, 3, false>(), kfn<false, 3, true>()}},
        {{kfn<true, 0, false>(), kfn<true, 0, true>()}, {kfn<true, 1, false>(), kfn<true, 1, true>()},
         {kfn<true, 2, false>(), kfn<true, 2, true>()}, {kfn<true, 3, false>(), kfn<true, 3, true>()}}};
    return tab[bf16 ? 1 : 0][kind][inv ? 1 : 0];
}

int smem_bytes(bool bf16) { return bf16 ? Smem<true>::BYTES : Smem<false>::BYTES; }

int grid_for(const void *fn, bool bf16, long long ntiles)
{
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> done;
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!done.count({dev, fn})) {
            check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(bf16)),
                       "tensor-core kernel shared memory opt-in");
            check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                            cudaSharedmemCarveoutMaxShared),
                       "tensor-core kernel carveout");
            done.insert({dev, fn});
        }
    }
    int per_sm = 0, sms = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, THREADS, smem_bytes(bf16)), "occupancy");
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    // CTAs only loop over independent tiles, so a grid above what is
    // resident is safe; never plan for fewer than the static residency
    per_sm = std::max(per_sm, bf16 ? Smem<true>::MIN_BLOCKS : Smem<false>::MIN_BLOCKS);
    return (int)std::max<long long>(1, std::min<long long>(ntiles, (long long)per_sm * sms));
}

}  // namespace tcf

// ---------------------------------------------------------------------------

void TCCore::init(int mode_, int logn_, long long batch_hint)
{
    mode = mode_;
    logn = logn_;
    if (logn != 8 && logn != 12 && logn != 16)
        fail(GFFT_ERR_UNSUPPORTED, "the tensor-core path covers n = 256, 4096 and 65536");
    const bool bf16 = mode == GFFT_MODE_TC_BF16;
    const int terms = bf16 ? 3 : 2;
    const size_t bcount = (size_t)terms * tcf::B_TERM / 8;  // in fp32 complex elements
    for (int inv = 0; inv < 2; inv++)
        bmat[inv] = cached_table("tc/bmat/" + std::to_string(bf16) + "/" + std::to_string(inv), GFFT_F32, bcount,
                                 [bf16, inv](void *buf) { tcf::fill_bmat(bf16, inv != 0, (unsigned char *)buf); });
    tw256 = cached_table("tc/w256", GFFT_F32, 512, [](void *buf) { tcf::fill_pairs(256, 256, (float *)buf); });
    if (logn == 12)
        tw2 = cached_table("tc/w4096lo", GFFT_F32, 32, [](void *buf) { tcf::fill_pairs(4096, 16, (float *)buf); });
    if (logn == 16) {
        tw2 = cached_table("tc/w65536lo", GFFT_F32, 512, [](void *buf) { tcf::fill_pairs(65536, 256, (float *)buf); });
        // transforms per column/row launch pair, within the workspace budget
        // of the tile launches (GFFT_WS_BUDGET_MB, 1 GB: 2048 transforms)
        const char *v = std::getenv("GFFT_WS_BUDGET_MB");
        const long long budget_mb = (v && *v) ? std::max(1LL, std::atoll(v)) : 1024;
        const long long cap = std::max<long long>(1, (budget_mb << 20) / (65536 * 8));
        group = std::max<long long>(1, std::min<long long>(std::max<long long>(1, batch_hint), cap));
        ws_bytes = (size_t)group * 65536 * 8;
        check_cuda(cudaMalloc(&ws, ws_bytes), "cudaMalloc(workspace)");
    }
    device_error_word();
}

void TCCore::release()
{
    if (ws) cudaFree(ws);
    ws = nullptr;
}

int TCCore::launches(long long batch) const
{
    if (logn != 16) return 1;
    return 2 * (int)((batch + group - 1) / group);
}

void TCCore::run(int inverse, const void *in, void *out, long long batch, long long idist, long long odist,
                 long long istride, long long ostride, cudaStream_t st, double scale) const
{
    if (istride != 1 || ostride != 1) fail(GFFT_ERR_UNSUPPORTED, "the tensor-core path needs unit element strides");
    const bool bf16 = mode == GFFT_MODE_TC_BF16;
    auto launch = [&](int kind, const void *src, void *dst, long long ntiles, long long nb, long long id,
                      long long od) {
        // TMA copies need 16-byte aligned tiles: aligned base, even distance
        CUtensorMap map;
        std::memset(&map, 0, sizeof map);
        bool tma = ((uintptr_t)src % 16 == 0) && (id % 2 == 0);
        if (tma && kind == tcf::KCOL)
            tma = make_tensor_map_3d(&map, src, 256, 256, (unsigned long long)nb, 256 * 8,
                                     (unsigned long long)((nb > 1 ? id : 65536) * 8), 16, 256);
        tcf::TcArgs a;
        a.in = static_cast<const float2 *>(src);
        a.out = static_cast<float2 *>(dst);
        a.ntiles = ntiles;
        a.batch = nb;
        a.idist = id;
        a.odist = od;
        a.bmat = bmat[inverse ? 1 : 0];
        a.tw256 = static_cast<const float2 *>(tw256);
        a.tw2 = static_cast<const float2 *>(tw2);
        a.err = device_error_word();
        a.tma = tma ? 1 : 0;
        a.scale = kind == tcf::KCOL ? 1.0f : (float)scale;
        const void *fn = tcf::kernel_for(bf16, kind, inverse != 0);
        const int grid = tcf::grid_for(fn, bf16, ntiles);
        void *args[] = {&map, &a};
        check_cuda(cudaLaunchKernel(fn, dim3(grid), dim3(tcf::THREADS), args, tcf::smem_bytes(bf16), st),
                   "launch tensor-core C2C");
    };
    if (logn == 8) {
        launch(tcf::K256, in, out, (batch + 15) / 16, batch, idist, odist);
    } else if (logn == 12) {
        launch(tcf::K4096, in, out, batch, batch, idist, odist);
    } else {
        for (long long b0 = 0; b0 < batch; b0 += group) {
            const long long nb = std::min(group, batch - b0);
            const char *src = static_cast<const char *>(in) + (size_t)(b0 * idist) * 8;
            char *dst = static_cast<char *>(out) + (size_t)(b0 * odist) * 8;
            launch(tcf::KCOL, src, ws, nb * 16, nb, idist, 65536);
            launch(tcf::KROW, ws, dst, nb * 16, nb, 65536, odist);
        }
    }
}

}  // namespace gfft
