// threepass.h -- host-side registry and launcher of the three-pass C2C
// (threepass.cu): n = 2^a * 2^b * 2^c with short tiles in every pass.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace gfft {

struct ThreePass {
    int la = 0, lb = 0, lc = 0;   // n = 2^la * 2^lb * 2^lc
    int c1 = 0, c2 = 0, r3 = 0;   // columns (passes 1, 2) / rows (pass 3) per tile
    const void *fwd[3] = {}, *inv[3] = {};
    int threads[3] = {};
    size_t smem[3] = {};
    size_t tw_count[3] = {};      // Stockham tables of the 2^la-, 2^lb- and 2^lc-point FFTs
    void (*tw_fill[3])(void *) = {};
};

struct ThreePassArgs {
    const void *in;
    void *out;
    void *ws;                      // nb * n elements
    long long batch, idist, odist;
    const void *tw[3];             // Stockham tables
    const void *lo1, *hi1;         // W_n^e = hi1[e >> bits1] * lo1[e & (2^bits1 - 1)]
    int bits1;
    const void *lo2, *hi2;         // W_m^e, m = 2^(lb + lc), split the same way
    int bits2;
    double scale;
};

// the registered three-pass layout of fp32 n = 2^logn, or nullptr
const ThreePass *threepass_find(int dtype, int logn);
// one group of a.batch transforms: in -> ws (pass 1), ws in place (pass 2),
// ws -> out (pass 3), each a programmatic dependent launch
cudaError_t launch_threepass(const ThreePass &k, int inverse, const ThreePassArgs &a, cudaStream_t st);

}  // namespace gfft
