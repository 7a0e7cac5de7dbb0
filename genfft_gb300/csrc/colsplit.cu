// colsplit.cu -- the passes around the split column FFTs (ColCore::run) for
// columns longer than one tile (2^13 .. 2^24 points):
//   k_rows_bitrev : rows in bit-reversed order -> natural order, whole rows
//                   at a time (FFTVert<T>::transform_no_scramble reads its
//                   input in that order, fft.h:132-136); in place it swaps
//                   row pairs, out of place it copies;
//   k_herm_fill   : the full-width real 2D layout (RealFFT2D::forward,
//                   FFTReal.h:90-103): columns W/2+1 .. W-1 of every row k
//                   are conj X[(H - k) mod H][W - col].
// Both are HBM-bound element passes: one read and one write per element.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"
#include "plan.h"
#include "stockham.cuh"

namespace gfft {

template <typename T>
__global__ void k_rows_bitrev(const cpx<T> *in, cpx<T> *out, int logh, long long ncols, long long ld_in,
                              long long ld_out, long long batch, long long idist, long long odist)
{
    const long long H = 1LL << logh;
    const long long total = batch * H * ncols;
    const bool inplace = in == out;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long c = idx % ncols;
        const long long rest = idx / ncols;
        const long long i = rest & (H - 1), b = rest >> logh;
        const long long r = logh ? (long long)(__brevll((unsigned long long)i) >> (64 - logh)) : 0;
        if (inplace) {
            if (r > i) {
                cpx<T> *p = out + b * odist + c;
                const cpx<T> u = ld_c(p + i * ld_out), w = ld_c(p + r * ld_out);
                st_c(p + i * ld_out, w);
                st_c(p + r * ld_out, u);
            }
        } else {
            st_c(out + b * odist + r * ld_out + c, ld_c(in + b * idist + i * ld_in + c));
        }
    }
}

template <typename T>
__global__ void k_herm_fill(cpx<T> *out, long long H, long long W, long long ld, long long batch, long long odist)
{
    const long long m = W / 2 - 1;  // columns W/2+1 .. W-1
    const long long total = batch * H * m;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long col = W / 2 + 1 + idx % m;
        const long long rest = idx / m;
        const long long k = rest % H, b = rest / H;
        cpx<T> *p = out + b * odist;
        st_c(p + k * ld + col, conj(ld_c(p + ((H - k) & (H - 1)) * ld + (W - col))));
    }
}

static unsigned elem_grid(long long total)
{
    return (unsigned)std::max<long long>(1, std::min<long long>((total + 255) / 256, 152LL * 64));
}

cudaError_t launch_rows_bitrev(int dtype, const void *in, void *out, int logh, long long ncols, long long ld_in,
                               long long ld_out, long long batch, long long idist, long long odist, cudaStream_t st)
{
    const long long total = batch * (1LL << logh) * ncols;
    if (total <= 0) return cudaSuccess;
    const unsigned g = elem_grid(total);
    if (dtype == GFFT_F32)
        k_rows_bitrev<float><<<g, 256, 0, st>>>((const cpx<float> *)in, (cpx<float> *)out, logh, ncols, ld_in, ld_out,
                                                 batch, idist, odist);
    else
        k_rows_bitrev<double><<<g, 256, 0, st>>>((const cpx<double> *)in, (cpx<double> *)out, logh, ncols, ld_in,
                                                  ld_out, batch, idist, odist);
    return cudaGetLastError();
}

cudaError_t launch_herm_fill(int dtype, void *out, long long H, long long W, long long ld, long long batch,
                             long long odist, cudaStream_t st)
{
    const long long total = batch * H * (W / 2 - 1);
    if (W < 4 || total <= 0) return cudaSuccess;
    const unsigned g = elem_grid(total);
    if (dtype == GFFT_F32) k_herm_fill<float><<<g, 256, 0, st>>>((cpx<float> *)out, H, W, ld, batch, odist);
    else k_herm_fill<double><<<g, 256, 0, st>>>((cpx<double> *)out, H, W, ld, batch, odist);
    return cudaGetLastError();
}

}  // namespace gfft
