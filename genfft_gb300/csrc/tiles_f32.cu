// tiles_f32.cu -- fp32 instantiations of the tile kernels (tiles.cuh).
// A tile holds C columns of 2^LOGL points, E = 16 points per thread, so a
// tile has 2^LOGL * C / 16 threads and C * 2^LOGL * 8 B of shared memory.
// Two column counts per length: the wider tile gives longer contiguous runs
// in HBM, the narrower one half the threads (no register cap of 64).
#include "tiles_impl.cuh"

namespace gfft {
#define R(V, L, C, E) static TileReg<float, V, L, C, E> reg_f32_##V##_##L##_##C;
#define ALLV(L, C, E) R(TILE_COL_TW4, L, C, E) R(TILE_ROW_XPOSE, L, C, E) \
                      R(TILE_COL_PLAIN, L, C, E) R(TILE_COL_BITREV, L, C, E)
ALLV(6, 16, 16) ALLV(7, 16, 16) ALLV(8, 16, 16) ALLV(9, 16, 16)
ALLV(10, 16, 16) ALLV(10, 8, 16) ALLV(11, 8, 16) ALLV(11, 4, 16) ALLV(12, 4, 16) ALLV(12, 2, 16)
// short columns (2D / FFTVert with few rows)
#define SHORT(L) R(TILE_COL_PLAIN, L, 16, 16) R(TILE_COL_BITREV, L, 16, 16)
SHORT(0) SHORT(1) SHORT(2) SHORT(3) SHORT(4) SHORT(5)
#undef SHORT
#undef ALLV
#undef R
}  // namespace gfft
