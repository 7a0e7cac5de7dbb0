// tiles_f64.cu -- fp64 instantiations of the tile kernels (tiles.cuh).
// E = 8 points per thread; C * 2^LOGL * 16 B of shared memory per tile.
#include "tiles_impl.cuh"

namespace gfft {
#define R(V, L, C, E) static TileReg<double, V, L, C, E> reg_f64_##V##_##L##_##C;
#define ALLV(L, C, E) R(TILE_COL_TW4, L, C, E) R(TILE_ROW_XPOSE, L, C, E) \
                      R(TILE_COL_PLAIN, L, C, E) R(TILE_COL_BITREV, L, C, E)
ALLV(6, 8, 8) ALLV(7, 8, 8) ALLV(8, 8, 8) ALLV(9, 8, 8) ALLV(9, 4, 8)
ALLV(10, 4, 8) ALLV(10, 2, 8) ALLV(11, 2, 8) ALLV(12, 2, 8)
#define SHORT(L) R(TILE_COL_PLAIN, L, 8, 8) R(TILE_COL_BITREV, L, 8, 8)
SHORT(0) SHORT(1) SHORT(2) SHORT(3) SHORT(4) SHORT(5)
#undef SHORT
#undef ALLV
#undef R
}  // namespace gfft
