// tiles_f64_4step.cu -- double four-step column (with inter-pass twiddle) and
// row (transposed store) tile kernels, see tiles.cuh.  A tile holds C
// columns of 2^LOGL points; several C per length trade HBM run length
// (C * sizeof complex) against CTAs per SM.
#include "tiles_impl.cuh"

namespace gfft {
#define R(V, L, C, E) static TileReg<double, V, L, C, E> reg_f64_##V##_##L##_##C;
#define V2(L, C, E) R(TILE_COL_TW4, L, C, E) R(TILE_ROW_XPOSE, L, C, E)
V2(6, 8, 8) V2(7, 8, 8) V2(8, 8, 8) V2(8, 4, 8) V2(9, 8, 8) V2(9, 4, 8)
V2(10, 4, 8) V2(10, 2, 8) V2(11, 2, 8) V2(12, 2, 8)
#undef V2
#undef R
}  // namespace gfft
