// fourstep.h -- host-side registry and launcher of the persistent four-step
// C2C kernels (fourstep.cuh).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace gfft {

// kernel arguments (one struct, passed by value)
struct FourStepArgs {
    const void *in;
    void *out;
    void *ws;                 // slots * N elements
    long long batch, idist, odist;
    int *ctr;                 // [0] next item, [1] abort, [2, 2+S) col_done, [2+S, 2+2S) row_done
    unsigned *err;
    const void *tw_a, *tw_b;  // Stockham tables of the A- and B-point tile FFTs
    const void *tw_lo, *tw_hi;  // W_N^e = hi[e >> lo_bits] * lo[e & (2^lo_bits - 1)]
    int lo_bits;
    int slots, lag;
    int nitems;
    double scale;             // applied to every output (norm= scaling)
    const void *dtw;          // real-input mode: the DIT twiddles t_k, k = 0 .. N
};

struct FourStepKernel {
    const void *fwd = nullptr, *inv = nullptr;
    const void *dit = nullptr;  // real-input (forward, DIT fused) version, or null
    int threads = 0;
    size_t smem = 0;
    int la = 0, lb = 0;      // N = 2^la * 2^lb: column length A, row length B
    int cc = 0, cr = 0;      // columns per COL tile, rows per ROW tile
    int nc = 0, nr = 0;      // tiles per transform
    int nrp = 0;             // row items per transform in real-input mode (A / cr + 1)
    int boxr = 0;            // rows per tensor box of a COL tile
    int ns = 0;              // shared-memory stages
    size_t twa = 0, twb = 0; // Stockham table sizes (complex elements)
    void (*fill_a)(void *) = nullptr;
    void (*fill_b)(void *) = nullptr;
    // pair-packed kernel (fourstep2.cuh): also needs a 16-byte aligned
    // output and even output distances (two-row stores)
    bool pair = false;
};

void fourstep_register(int dtype, int logn, const FourStepKernel &k);
// every registered variant of (dtype, logn), widest tile first; count in *n
const FourStepKernel *const *fourstep_variants(int dtype, int logn, int *n);

// ring slots and lag for a transform of `bytes` bytes: slots * bytes within
// the L2 budget where possible (at least lag + 1 slots)
void fourstep_schedule(size_t bytes, long long batch, int grid, int depth, int items_per_transform, int *slots,
                       int *lag);

// `map` is the 3D tensor map of the input (8-byte units x rows x batch)
// (dit: the real-input version, k.dit)
cudaError_t launch_fourstep(const FourStepKernel &k, int inverse, const CUtensorMap &map, const FourStepArgs &a,
                            int grid, cudaStream_t st, bool dit = false);
// CTAs of kernel k (or of its real-input version) that run at once on the
// current device
int fourstep_grid(const FourStepKernel &k, bool dit = false);

}  // namespace gfft
