// common.cuh -- complex arithmetic and in-register DFT codelets for the
// sm_103a transform kernels.
//
// Conventions (same as the reference genFFT, fft.h:80-85, FFTTwiddle.h:44-51):
//   forward  X[k] = sum_n x[n] * exp(-2*pi*i*n*k/N)
//   inverse  x[n] = sum_k X[k] * exp(+2*pi*i*n*k/N)   (unscaled)
// Complex values are interleaved {re, im} pairs (float2 / double2 layout).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace gfft {

template <typename T>
struct alignas(2 * sizeof(T)) cpx {
    T x, y;
};

template <typename T>
__device__ __forceinline__ cpx<T> mk(T a, T b) { return cpx<T>{a, b}; }
template <typename T>
__device__ __forceinline__ cpx<T> operator+(cpx<T> a, cpx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T>
__device__ __forceinline__ cpx<T> operator-(cpx<T> a, cpx<T> b) { return {a.x - b.x, a.y - b.y}; }

#ifndef GFFT_PACKED_F32
#define GFFT_PACKED_F32 1
#endif
#if GFFT_PACKED_F32
// fp32 complex add / subtract as one packed two-lane instruction
// (add/sub.rn.f32x2, sm_100 family): both lanes of a butterfly at once
template <>
__device__ __forceinline__ cpx<float> operator+(cpx<float> a, cpx<float> b)
{
    cpx<float> d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
template <>
__device__ __forceinline__ cpx<float> operator-(cpx<float> a, cpx<float> b)
{
    cpx<float> d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
#endif
template <typename T>
__device__ __forceinline__ cpx<T> operator-(cpx<T> a) { return {-a.x, -a.y}; }

// complex product a*b
template <typename T>
__device__ __forceinline__ cpx<T> cmul(cpx<T> a, cpx<T> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <typename T>
__device__ __forceinline__ cpx<T> cmulc(cpx<T> a, cpx<T> b)
{
    return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
// twiddle product in the transform's direction: forward multiplies by w,
// inverse by conj(w) (tables hold the forward twiddles exp(-2 pi i k/N)).
template <bool INV, typename T>
__device__ __forceinline__ cpx<T> twmul(cpx<T> a, cpx<T> w)
{
    return INV ? cmulc(a, w) : cmul(a, w);
}
template <typename T>
__device__ __forceinline__ cpx<T> conj(cpx<T> a) { return {a.x, -a.y}; }
// a * s for a real scale (the norm= factor of a transform's last store)
template <typename T>
__device__ __forceinline__ cpx<T> scl(cpx<T> a, T s) { return {a.x * s, a.y * s}; }

__host__ __device__ constexpr int ipow(int b, int e) { return e <= 0 ? 1 : b * ipow(b, e - 1); }

// vector loads/stores of one complex value (8 or 16 bytes, naturally aligned)
template <typename T>
struct vec2;
template <>
struct vec2<float> { using type = float2; };
template <>
struct vec2<double> { using type = double2; };

// read-only path (twiddle tables)
template <typename T>
__device__ __forceinline__ cpx<T> ldg_c(const cpx<T> *p)
{
    auto v = __ldg(reinterpret_cast<const typename vec2<T>::type *>(p));
    return {v.x, v.y};
}
// plain global load
template <typename T>
__device__ __forceinline__ cpx<T> ld_c(const cpx<T> *p)
{
    auto v = *reinterpret_cast<const typename vec2<T>::type *>(p);
    return {v.x, v.y};
}
// streaming (evict-first) global load / store for data touched once
// Entry of a kernel launched as a programmatic dependent of the previous
// kernel on the stream (launch_pdl; a no-op in an ordinary launch): let the
// next kernel's CTAs be scheduled once every CTA of this grid has started,
// then wait for the previous kernel's completion, and its writes, before
// touching global memory.
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <typename T>
__device__ __forceinline__ cpx<T> ldcs_c(const cpx<T> *p)
{
    auto v = __ldcs(reinterpret_cast<const typename vec2<T>::type *>(p));
    return {v.x, v.y};
}
template <typename T>
__device__ __forceinline__ void stcs_c(cpx<T> *p, cpx<T> a)
{
    typename vec2<T>::type v;
    v.x = a.x;
    v.y = a.y;
    __stcs(reinterpret_cast<typename vec2<T>::type *>(p), v);
}
template <typename T>
__device__ __forceinline__ void st_c(cpx<T> *p, cpx<T> a)
{
    typename vec2<T>::type v;
    v.x = a.x;
    v.y = a.y;
    *reinterpret_cast<typename vec2<T>::type *>(p) = v;
}

// ---------------------------------------------------------------------------
// Multiplication by the compile-time root W_32^k = exp(-2 pi i k / 32)
// (forward) or its conjugate (inverse).  Trivial roots cost no multiply,
// the 45-degree roots two.  Constants are the correctly rounded values of
// cos(pi m / 16), m = 0..8.

// cos(2 pi k / 32) for any integer k
__host__ __device__ constexpr double cos32d(int k)
{
    k = ((k % 32) + 32) % 32;
    if (k > 16) k = 32 - k;
    if (k > 8) return -cos32d(16 - k);
    return k == 0 ? 1.0
         : k == 1 ? 0.98078528040323044913
         : k == 2 ? 0.92387953251128675613
         : k == 3 ? 0.83146961230254523708
         : k == 4 ? 0.70710678118654752440
         : k == 5 ? 0.55557023301960222474
         : k == 6 ? 0.38268343236508977173
         : k == 7 ? 0.19509032201612826785
                  : 0.0;
}

// compile-time loop: f(std::integral_constant<int, I>) for I in [B, E)
template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F &&f)
{
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

template <int K, bool INV, typename T>
__device__ __forceinline__ cpx<T> rot32(cpx<T> a)
{
    // exponent of the effective forward root after folding direction
    constexpr int k = INV ? ((32 - (K % 32)) % 32) : (K % 32);
    constexpr T r2 = (T)cos32d(4);
    if constexpr (k == 0) return a;
    else if constexpr (k == 8) return {a.y, -a.x};     // * (-i)
    else if constexpr (k == 16) return {-a.x, -a.y};   // * (-1)
    else if constexpr (k == 24) return {-a.y, a.x};    // * (+i)
    else if constexpr (k == 4) return {r2 * (a.x + a.y), r2 * (a.y - a.x)};      // (r2, -r2)
    else if constexpr (k == 12) return {r2 * (a.y - a.x), -r2 * (a.x + a.y)};    // (-r2, -r2)
    else if constexpr (k == 20) return {-r2 * (a.x + a.y), r2 * (a.x - a.y)};    // (-r2, r2)
    else if constexpr (k == 28) return {r2 * (a.x - a.y), r2 * (a.x + a.y)};     // (r2, r2)
    else {
        // general root: cos(2 pi k/32), -sin(2 pi k/32); sin(t) = cos(t - pi/2)
        constexpr T wr = (T)cos32d(k);
        constexpr T wi = (T)(-cos32d(k - 8));
        return {a.x * wr - a.y * wi, a.x * wi + a.y * wr};
    }
}

// ---------------------------------------------------------------------------
// In-register DFT of R points (R = 1, 2, 4, 8, 16, 32), natural order in
// and out, stride-1 over the array v.  R >= 8 is split as A x B
// (A = 2 for R = 8, else 4): n = n1 + A*n2, k = k1 + B*k2,
//   X[k1 + B k2] = sum_n1 W_A^(n1 k2) W_R^(n1 k1) sum_n2 x[n1 + A n2] W_B^(n2 k1)
template <int R, bool INV, typename T>
__device__ __forceinline__ void dft(cpx<T> *v)
{
    if constexpr (R == 1) {
        return;
    } else if constexpr (R == 2) {
        cpx<T> a = v[0], b = v[1];
        v[0] = a + b;
        v[1] = a - b;
    } else if constexpr (R == 4) {
        cpx<T> s02 = v[0] + v[2], d02 = v[0] - v[2];
        cpx<T> s13 = v[1] + v[3], d13 = v[1] - v[3];
        // forward: X1 = d02 - i d13, X3 = d02 + i d13
        cpx<T> jd13 = INV ? cpx<T>{-d13.y, d13.x} : cpx<T>{d13.y, -d13.x};  // (-+i) * d13
        v[0] = s02 + s13;
        v[2] = s02 - s13;
        v[1] = d02 + jd13;
        v[3] = d02 - jd13;
    } else {
        constexpr int A = (R >= 16) ? 4 : 2;
        constexpr int B = R / A;
        cpx<T> y[A][B];
#pragma unroll
        for (int n1 = 0; n1 < A; n1++) {
#pragma unroll
            for (int n2 = 0; n2 < B; n2++) y[n1][n2] = v[n1 + A * n2];
            dft<B, INV, T>(y[n1]);
        }
        // inner twiddles W_R^(n1 k1) = W_32^(n1 k1 32/R)
        constexpr int S = 32 / R;
        static_for<0, B>([&](auto k1c) {
            constexpr int k1 = decltype(k1c)::value;
            cpx<T> z[A];
            static_for<0, A>([&](auto n1c) {
                constexpr int n1 = decltype(n1c)::value;
                z[n1] = rot32<n1 * k1 * S, INV, T>(y[n1][k1]);
            });
            dft<A, INV, T>(z);
#pragma unroll
            for (int k2 = 0; k2 < A; k2++) v[k1 + B * k2] = z[k2];
        });
    }
}

}  // namespace gfft
