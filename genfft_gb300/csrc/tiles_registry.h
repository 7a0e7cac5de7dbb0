// tiles_registry.h -- host-side registry of the tile-kernel instantiations
// (column pass, row pass) so the planner can pick one by (dtype, variant,
// log2 length, columns per tile).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace gfft {

enum TileVariant {
    TILE_COL_TW4 = 0,     // column pass of the four-step split (with W_N twiddle)
    TILE_COL_PLAIN = 1,   // column FFT, natural-order input
    TILE_COL_BITREV = 2,  // column FFT, bit-reversed row order on input
    TILE_ROW_XPOSE = 3,   // row pass with transposed store
    TILE_COL_HERM = 4,    // column FFT + Hermitian mirror store (real 2D)
    TILE_COL_TWB = 5      // column pass with the W_N^(batch * row) twiddle (split column FFTs)
};

struct TileKernel {
    const void *fwd = nullptr, *inv = nullptr;
    int threads = 0;
    size_t smem = 0;
    size_t twcount = 0;
    void (*fill)(void *) = nullptr;  // Stockham twiddles for the L-point sub-FFT
    int elem_bytes = 8;              // sizeof one complex element
    // persistent TMA-pipelined version (nullptr when not instantiated or
    // when its two stage buffers do not fit shared memory)
    const void *tma_fwd = nullptr, *tma_inv = nullptr;
    int tma_threads = 0;
    size_t tma_smem = 0;
    int tma_boxr = 0;  // column pass: rows per tensor box
    int tma_rows = 0;  // column pass: column length (tensor rows)
    int tma_c = 0;     // columns per tile
    int tma_stages = 0;  // 2 double-buffered, 1 single buffer
    bool tma_row = false;  // a row-pass kernel (for the GFFT_TMA1 knob)
};

// register / look up (returns nullptr when not instantiated)
void tile_register(int dtype, int variant, int logl, int c, const TileKernel &k);
const TileKernel *tile_find(int dtype, int variant, int logl, int c);
// widest registered column count <= max_c (0 if none)
int tile_widest(int dtype, int variant, int logl, int max_c);

// Launch over tiles x nbatch CTAs (the batch is split into launches of at
// most 65535 items).  Strides and distances are in complex elements.
cudaError_t launch_colpass(const TileKernel &k, int inverse, long long tiles, long long nbatch,
                           const void *in, void *out, long long ncols, long long ld_in, long long ld_out,
                           long long idist, long long odist, const void *tw, const void *tw_lo,
                           const void *tw_hi, int lo_bits, unsigned nmask, cudaStream_t st, double scale = 1.0);
cudaError_t launch_rowpass(const TileKernel &k, int inverse, long long tiles, long long nbatch,
                           const void *in, void *out, long long nrows, long long ld_in, long long ostride,
                           long long idist, long long odist, const void *tw, cudaStream_t st, double scale = 1.0);

// 3D tiled tensor map over 8-byte units (dims x, y, z; byte strides of y
// and z; box bx x by x 1); false if the driver entry point is missing or
// the base / strides are not 16-byte aligned
bool make_tensor_map_3d(CUtensorMap *map, const void *base, unsigned long long dx, unsigned long long dy,
                        unsigned long long dz, unsigned long long sy_bytes, unsigned long long sz_bytes, unsigned bx,
                        unsigned by);

// the device error word the persistent kernels report timeouts into
unsigned *device_error_word();

}  // namespace gfft
