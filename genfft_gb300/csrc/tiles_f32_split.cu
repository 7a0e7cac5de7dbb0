// tiles_f32_split.cu -- float first steps of the split column FFTs for
// columns of 2^13 .. 2^24 points (H = H1 * H2, H1 = 2^8 .. 2^12): the
// H1-point column FFTs with the W_H^(batch * row) twiddle (TILE_COL_TWB),
// see ColCore::run.  The second steps are the plain column tiles.
#include "tiles_impl.cuh"

namespace gfft {
#define R(L, C, E) static TileReg<float, TILE_COL_TWB, L, C, E> reg_f32_twb_##L##_##C;
R(8, 16, 16) R(9, 16, 16) R(10, 8, 16) R(11, 8, 16) R(12, 4, 16)
#undef R
}  // namespace gfft
