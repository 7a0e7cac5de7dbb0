// tiles_f64_split.cu -- double split column FFTs for columns of 2^13 ..
// 2^24 points: the twiddled first steps (TILE_COL_TWB, H1 = 2^6 .. 2^12),
// see ColCore::run.  The second steps are the plain column tiles.
#include "tiles_impl.cuh"

namespace gfft {
#define R(L, C, E) static TileReg<double, TILE_COL_TWB, L, C, E> reg_f64_twb_##L##_##C;
R(6, 8, 8) R(7, 8, 8) R(8, 8, 8) R(9, 8, 8) R(10, 4, 8) R(11, 2, 8) R(12, 2, 8)
#undef R
}  // namespace gfft
