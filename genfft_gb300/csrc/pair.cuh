// pair.cuh -- two fp32 transforms per thread in split form, on the packed
// two-lane FP32 instructions of the sm_100 family (add/sub/mul/fma .f32x2).
//
// A "pair point" holds the same point of two independent sub-transforms:
//   re = (re of transform 0, re of transform 1), im = (im0, im1).
// Every operation of a butterfly is then one packed instruction for both
// transforms, and the +-i rotations of the radix-4 steps are free (the real
// and imaginary halves swap roles in the next add or subtract).  The
// codelets below follow the radix structure and the rotation formulas of
// common.cuh lane by lane (dft<R>, rot32<K>), so each lane computes what
// the single-transform kernels compute, in the same order of operations.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"
#include "stockham.cuh"

namespace gfft {

struct __align__(16) pcx {
    float2 re, im;
};

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 f2bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 f2neg(float2 a) { return f2sub(make_float2(0.f, 0.f), a); }

__device__ __forceinline__ pcx operator+(pcx a, pcx b) { return {f2add(a.re, b.re), f2add(a.im, b.im)}; }
__device__ __forceinline__ pcx operator-(pcx a, pcx b) { return {f2sub(a.re, b.re), f2sub(a.im, b.im)}; }

// a * w for a twiddle w = (c, s) shared by both lanes; INV: a * conj(w)
// (cmul / cmulc of common.cuh, lane by lane)
template <bool INV>
__device__ __forceinline__ pcx ptw(pcx a, float2 w)
{
    const float2 c = f2bc(w.x), s = f2bc(w.y);
    if (INV) return {f2fma(a.re, c, f2mul(a.im, s)), f2sub(f2mul(a.im, c), f2mul(a.re, s))};
    return {f2sub(f2mul(a.re, c), f2mul(a.im, s)), f2fma(a.re, s, f2mul(a.im, c))};
}
// a * w with a different twiddle per lane: wc = (c0, c1), ws = (s0, s1)
template <bool INV>
__device__ __forceinline__ pcx ptw2(pcx a, float2 wc, float2 ws)
{
    if (INV) return {f2fma(a.re, wc, f2mul(a.im, ws)), f2sub(f2mul(a.im, wc), f2mul(a.re, ws))};
    return {f2sub(f2mul(a.re, wc), f2mul(a.im, ws)), f2fma(a.re, ws, f2mul(a.im, wc))};
}
__device__ __forceinline__ pcx pscl(pcx a, float s) { return {f2mul(a.re, f2bc(s)), f2mul(a.im, f2bc(s))}; }

// multiplication by the compile-time root W_32^K (forward) or its conjugate
template <int K, bool INV>
__device__ __forceinline__ pcx prot32(pcx a)
{
    constexpr int k = INV ? ((32 - (K % 32)) % 32) : (K % 32);
    constexpr float r2 = (float)cos32d(4);
    if constexpr (k == 0) return a;
    else if constexpr (k == 8) return {a.im, f2neg(a.re)};
    else if constexpr (k == 16) return {f2neg(a.re), f2neg(a.im)};
    else if constexpr (k == 24) return {f2neg(a.im), a.re};
    else if constexpr (k == 4) return {f2mul(f2bc(r2), f2add(a.re, a.im)), f2mul(f2bc(r2), f2sub(a.im, a.re))};
    else if constexpr (k == 12) return {f2mul(f2bc(r2), f2sub(a.im, a.re)), f2mul(f2bc(-r2), f2add(a.re, a.im))};
    else if constexpr (k == 20) return {f2mul(f2bc(-r2), f2add(a.re, a.im)), f2mul(f2bc(r2), f2sub(a.re, a.im))};
    else if constexpr (k == 28) return {f2mul(f2bc(r2), f2sub(a.re, a.im)), f2mul(f2bc(r2), f2add(a.re, a.im))};
    else {
        constexpr float wr = (float)cos32d(k);
        constexpr float wi = (float)(-cos32d(k - 8));
        return {f2sub(f2mul(a.re, f2bc(wr)), f2mul(a.im, f2bc(wi))), f2fma(a.re, f2bc(wi), f2mul(a.im, f2bc(wr)))};
    }
}

// in-register DFT of R pair points (R = 1, 2, 4, 8, 16), the split of dft<R>
template <int R, bool INV>
__device__ __forceinline__ void pdft(pcx *v)
{
    if constexpr (R == 1) {
        return;
    } else if constexpr (R == 2) {
        const pcx a = v[0], b = v[1];
        v[0] = a + b;
        v[1] = a - b;
    } else if constexpr (R == 4) {
        const pcx s02 = v[0] + v[2], d02 = v[0] - v[2];
        const pcx s13 = v[1] + v[3], d13 = v[1] - v[3];
        v[0] = s02 + s13;
        v[2] = s02 - s13;
        // forward: X1 = d02 - i d13, X3 = d02 + i d13 (inverse: the conjugates)
        if (INV) {
            v[1] = {f2sub(d02.re, d13.im), f2add(d02.im, d13.re)};
            v[3] = {f2add(d02.re, d13.im), f2sub(d02.im, d13.re)};
        } else {
            v[1] = {f2add(d02.re, d13.im), f2sub(d02.im, d13.re)};
            v[3] = {f2sub(d02.re, d13.im), f2add(d02.im, d13.re)};
        }
    } else {
        constexpr int A = (R >= 16) ? 4 : 2;
        constexpr int B = R / A;
        pcx y[A][B];
#pragma unroll
        for (int n1 = 0; n1 < A; n1++) {
#pragma unroll
            for (int n2 = 0; n2 < B; n2++) y[n1][n2] = v[n1 + A * n2];
            pdft<B, INV>(y[n1]);
        }
        constexpr int S = 32 / R;
        static_for<0, B>([&](auto k1c) {
            constexpr int k1 = decltype(k1c)::value;
            pcx z[A];
            static_for<0, A>([&](auto n1c) {
                constexpr int n1 = decltype(n1c)::value;
                z[n1] = prot32<n1 * k1 * S, INV>(y[n1][k1]);
            });
            pdft<A, INV>(z);
#pragma unroll
            for (int k2 = 0; k2 < A; k2++) v[k1 + B * k2] = z[k2];
        });
    }
}

// Stockham passes of one pair of 2^LOGN-point transforms held by thread t
// of its group (the schedule of StockhamPlan<float, LOGN, E_>, whose
// twiddle table it reads: E_ pair points a thread).  v[q] = pair point
// t + q G on entry and exit.
// at(i): the pair point i slot of the group's exchange buffer; tw(p): the
// table entry p; SYNC(): the group's barrier.  The first exchange write
// comes before any SYNC: the caller orders it after the group's last reads
// of the buffer.
template <int LOGN, int E_, bool INV, typename At, typename Tw, typename Sync>
__device__ __forceinline__ void pstockham_run(pcx (&v)[StockhamPlan<float, LOGN, E_>::E], int t, At at, Tw tw,
                                              Sync SYNC)
{
    using SP = StockhamPlan<float, LOGN, E_>;
    constexpr int E = SP::E, G = SP::G, P = SP::P, R0 = SP::R0;
#pragma unroll
    for (int m = 0; m < E / R0; m++) {
        pcx u[R0];
#pragma unroll
        for (int r = 0; r < R0; r++) u[r] = v[m + r * (E / R0)];
        pdft<R0, INV>(u);
        if constexpr (P == 1) {
#pragma unroll
            for (int r = 0; r < R0; r++) v[m + r * (E / R0)] = u[r];
        } else {
            const int j = t + m * G;
#pragma unroll
            for (int r = 0; r < R0; r++) at(j * R0 + r) = u[r];
        }
    }
    static_for<1, P>([&](auto pc) {
        constexpr int p = decltype(pc)::value;
        constexpr int Ns = R0 * ipow(E, p - 1);
        constexpr int off = SP::twiddle_offset(p);
        SYNC();
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = at(t + q * G);
        const int jm = t % Ns;
#pragma unroll
        for (int r = 1; r < E; r++) v[r] = ptw<INV>(v[r], tw(off + jm + (r - 1) * Ns));
        pdft<E, INV>(v);
        if constexpr (p < P - 1) {
            SYNC();
            const int base = (t / Ns) * Ns * E + jm;
#pragma unroll
            for (int r = 0; r < E; r++) at(base + r * Ns) = v[r];
        }
    });
}

// padded slot of pair point i: 16 bytes a point, one pad slot per 8 so the
// strided Stockham writes of a quarter warp fall on distinct banks
__device__ __forceinline__ int ppad(int i) { return i + (i >> 3); }
__host__ __device__ constexpr int ppad_size(int n) { return n + n / 8 + 1; }

}  // namespace gfft
