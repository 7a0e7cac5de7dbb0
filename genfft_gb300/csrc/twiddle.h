// twiddle.h -- host-side generation of twiddle factors in FP64.
//
// The reference computes its tables in double and rounds to T
// (FFTTwiddle.h:44-51, 116-127).  Here every root is computed from an exact
// integer phase k/M with an octant reduction, so each cos/sin argument lies
// in [0, pi/4] and the FP64 value is within about one ulp before it is
// rounded to the table type.
#pragma once

#include <cmath>

namespace gfft {

// c = cos(2 pi k / M), s = sin(2 pi k / M) for any integer k, M > 0
inline void exact_root(long long k, long long M, double *c, double *s)
{
    const double PI = 3.14159265358979323846;
    k %= M;
    if (k < 0) k += M;
    const long long t8 = 8 * k;
    const int o = (int)(t8 / M);
    const long long r = t8 - (long long)o * M;              // [0, M)
    const double phi = PI * (double)r / (4.0 * (double)M);  // [0, pi/4)
    const double psi = PI * (double)(M - r) / (4.0 * (double)M);
    double cf = std::cos(phi), sf = std::sin(phi), cp = std::cos(psi), sp = std::sin(psi);
    switch (o) {
    case 0: *c = cf; *s = sf; break;
    case 1: *c = sp; *s = cp; break;
    case 2: *c = -sf; *s = cf; break;
    case 3: *c = -cp; *s = sp; break;
    case 4: *c = -cf; *s = -sf; break;
    case 5: *c = -sp; *s = -cp; break;
    case 6: *c = sf; *s = -cf; break;
    default: *c = cp; *s = -sp; break;
    }
}

// forward twiddle W_M^k = exp(-2 pi i k / M) as {re, im}
template <typename T>
inline void forward_root(long long k, long long M, T *re, T *im)
{
    double c, s;
    exact_root(k, M, &c, &s);
    *re = (T)c;
    *im = (T)(-s);
}

}  // namespace gfft
