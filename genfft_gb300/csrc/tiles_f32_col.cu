// tiles_f32_col.cu -- float column-FFT tile kernels (2D column pass,
// FFTVert, real-2D Hermitian fill), see tiles.cuh.
#include "tiles_impl.cuh"

namespace gfft {
#define R(V, L, C, E) static TileReg<float, V, L, C, E> reg_f32_##V##_##L##_##C;
#define V3(L, C, E) R(TILE_COL_PLAIN, L, C, E) R(TILE_COL_BITREV, L, C, E) R(TILE_COL_HERM, L, C, E)
V3(0, 16, 16) V3(1, 16, 16) V3(2, 16, 16) V3(3, 16, 16) V3(4, 16, 16) V3(5, 16, 16)
V3(6, 16, 16) V3(7, 16, 16) V3(8, 16, 16) V3(9, 16, 16) V3(10, 16, 16) V3(10, 8, 16)
V3(11, 8, 16) V3(11, 4, 16) V3(12, 4, 16)
// split column FFTs of 2^10 .. 2^14 points (2D column passes): the twiddled
// first step and the plain second step over 32-, 64- and 128-point columns
#define S2(L, C, E) R(TILE_COL_TWB, L, C, E) static TileReg<float, TILE_COL_PLAIN, L, C, E> reg_f32_split_##L##_##C;
S2(5, 64, 16) S2(6, 64, 16) S2(7, 32, 16)
#undef S2
#undef V3
#undef R
}  // namespace gfft
