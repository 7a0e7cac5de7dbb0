// stockham.cuh -- block-level Stockham autosort FFT engine.
//
// One transform of N = 2^LOGN points is owned by a group of G = N/E threads;
// each thread holds E points in registers.  The pass schedule is one radix
// R0 pass (R0 <= E, no twiddles) followed by radix-E passes, so no bit
// reversal is ever needed (the reference's scramble, FFTUtil.h:51-83, is
// eliminated).  Pass p with radix R and sub-transform size Ns:
//   butterfly j in [0, N/R):   u[r]  = x[j + r N/R] * W_{Ns R}^((j mod Ns) r)
//                              u     = DFT_R(u)
//                              y[(j/Ns) Ns R + (j mod Ns) + r Ns] = u[r]
// On entry and on exit thread t holds v[q] = x[t + q G] (resp. X[t + q G]):
// the first pass reads and the last pass writes global memory in that
// pattern directly (coalesced across t); only the P-1 intermediate
// exchanges go through shared memory.
#pragma once

#include "common.cuh"

namespace gfft {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// shared-memory slot of element i: one padding slot per 128 bytes keeps the
// strided Stockham stores free of bank conflicts
template <typename T>
__device__ __forceinline__ int spad(int i)
{
    return sizeof(T) == 4 ? i + (i >> 4) : i + (i >> 3);
}

// padded slot count for n elements laid out through spad<T>
template <typename T>
__host__ __device__ constexpr int spad_size(int n)
{
    return n <= 1 ? 1 : n + (sizeof(T) == 4 ? n / 16 : n / 8) + 1;
}

template <typename T, int LOGN, int E_>
struct StockhamPlan {
    static constexpr int N = 1 << LOGN;
    static constexpr int E = (N < E_) ? N : E_;        // points per thread
    static constexpr int G = N / E;                    // threads per transform
    static constexpr int LOGE = ilog2c(E);
    static constexpr int P = (LOGE == 0) ? 1 : (LOGN + LOGE - 1) / LOGE;  // passes
    static constexpr int R0 = N >> (LOGE * (P - 1));   // first-pass radix
    // shared-memory elements per transform (0 when a single pass suffices)
    static constexpr int SMEM = (P > 1) ? (N + (sizeof(T) == 4 ? N / 16 : N / 8)) : 0;
    // twiddle elements: pass p >= 1 with Ns = R0 E^(p-1) uses (E-1) Ns entries
    __host__ __device__ static constexpr int twiddle_offset(int p)
    {
        int off = 0, ns = R0;
        for (int q = 1; q < p; q++) {
            off += (E - 1) * ns;
            ns *= E;
        }
        return off;
    }
    static constexpr int TW = twiddle_offset(P);
};

// Runs all passes of one transform held by thread t of its group.
//   v   : E points per thread, v[q] = x[t + q G] on entry, X[t + q G] on exit
//   at  : at(i) is the shared-memory slot of element i of this transform
//         (only touched when P > 1)
//   tw  : the plan's twiddle table (StockhamPlan::TW elements)
// SYNC() must synchronise every thread that shares the shared memory (the
// whole CTA, or the group).
// twiddle loads through the read-only cache (tables in global memory)
struct TwGlobal {
    template <typename T>
    __device__ __forceinline__ cpx<T> operator()(const cpx<T> *p) const { return ldg_c(p); }
};
// plain loads (tables staged in shared memory)
struct TwShared {
    template <typename T>
    __device__ __forceinline__ cpx<T> operator()(const cpx<T> *p) const { return *p; }
};

template <typename T, int LOGN, int E_, bool INV, typename TwLoad = TwGlobal, typename At, typename Sync>
__device__ __forceinline__ void stockham_run(cpx<T> (&v)[StockhamPlan<T, LOGN, E_>::E], int t,
                                             At at, const cpx<T> *__restrict__ tw, Sync SYNC)
{
    using SP = StockhamPlan<T, LOGN, E_>;
    constexpr int E = SP::E, G = SP::G, P = SP::P, R0 = SP::R0;

    // ---- pass 0: radix R0, Ns = 1, no twiddles
#pragma unroll
    for (int m = 0; m < E / R0; m++) {
        cpx<T> u[R0];
#pragma unroll
        for (int r = 0; r < R0; r++) u[r] = v[m + r * (E / R0)];
        dft<R0, INV, T>(u);
        if constexpr (P == 1) {
#pragma unroll
            for (int r = 0; r < R0; r++) v[m + r * (E / R0)] = u[r];
        } else {
            const int j = t + m * G;
#pragma unroll
            for (int r = 0; r < R0; r++) at(j * R0 + r) = u[r];
        }
    }

    // ---- passes 1 .. P-1: radix E
    static_for<1, P>([&](auto pc) {
        constexpr int p = decltype(pc)::value;
        constexpr int Ns = R0 * ipow(E, p - 1);
        constexpr int off = SP::twiddle_offset(p);
        SYNC();
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = at(t + q * G);
        const int jm = t % Ns;  // Ns <= G, so j = t
        const cpx<T> *twp = tw + off + jm;
#pragma unroll
        for (int r = 1; r < E; r++) v[r] = twmul<INV>(v[r], TwLoad{}(twp + (r - 1) * Ns));
        dft<E, INV, T>(v);
        if constexpr (p < P - 1) {
            SYNC();
            const int base = (t / Ns) * Ns * E + jm;
#pragma unroll
            for (int r = 0; r < E; r++) at(base + r * Ns) = v[r];
        }
    });
}

// host-side fill of a StockhamPlan twiddle table (TW complex elements)
template <typename T, int LOGN, int E_, typename Root>
void stockham_fill_twiddles(cpx<T> *o, Root root)
{
    using SP = StockhamPlan<T, LOGN, E_>;
    int ns = SP::R0;
    for (int p = 1; p < SP::P; p++) {
        const int off = SP::twiddle_offset(p);
        for (int r = 1; r < SP::E; r++)
            for (int m = 0; m < ns; m++)
                root((long long)m * r, (long long)ns * SP::E, &o[off + (r - 1) * ns + m]);
        ns *= SP::E;
    }
}

// bit reversal of the low `bits` bits
__device__ __forceinline__ int bitrev(int i, int bits) { return bits ? (int)(__brev((unsigned)i) >> (32 - bits)) : 0; }

}  // namespace gfft
