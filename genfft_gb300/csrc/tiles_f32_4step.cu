// tiles_f32_4step.cu -- float four-step column (with inter-pass twiddle) and
// row (transposed store) tile kernels, see tiles.cuh.  A tile holds C
// columns of 2^LOGL points; several C per length trade HBM run length
// (C * sizeof complex) against CTAs per SM.
#include "tiles_impl.cuh"

namespace gfft {
#define R(V, L, C, E) static TileReg<float, V, L, C, E> reg_f32_##V##_##L##_##C;
#define V2(L, C, E) R(TILE_COL_TW4, L, C, E) R(TILE_ROW_XPOSE, L, C, E)
V2(6, 16, 16) V2(7, 16, 16) V2(8, 16, 16) V2(8, 8, 16) V2(9, 16, 16) V2(9, 8, 16)
V2(10, 16, 16) V2(10, 8, 16) V2(10, 4, 16) V2(11, 8, 16) V2(11, 4, 16) V2(12, 4, 16) V2(12, 2, 16)
#undef V2
#undef R
}  // namespace gfft
