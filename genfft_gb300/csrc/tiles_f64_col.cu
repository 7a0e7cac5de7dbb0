// tiles_f64_col.cu -- double column-FFT tile kernels (2D column pass,
// FFTVert, real-2D Hermitian fill), see tiles.cuh.
#include "tiles_impl.cuh"

namespace gfft {
#define R(V, L, C, E) static TileReg<double, V, L, C, E> reg_f64_##V##_##L##_##C;
#define V3(L, C, E) R(TILE_COL_PLAIN, L, C, E) R(TILE_COL_BITREV, L, C, E) R(TILE_COL_HERM, L, C, E)
V3(0, 8, 8) V3(1, 8, 8) V3(2, 8, 8) V3(3, 8, 8) V3(4, 8, 8) V3(5, 8, 8)
V3(6, 8, 8) V3(7, 8, 8) V3(8, 8, 8) V3(9, 8, 8) V3(10, 4, 8) V3(11, 2, 8) V3(12, 2, 8)
#undef V3
#undef R
}  // namespace gfft
