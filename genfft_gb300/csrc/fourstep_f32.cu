// fourstep_f32.cu -- float persistent four-step kernels, n = 2^15 .. 2^24
// (see fourstep.cuh).  R(logn, CC, NS): tiles of CC columns of
// 2^(logn/2) points, NS shared-memory stages.  Tiles are capped at 512
// compute threads: 1024-thread tiles spill at the register count that
// keeps a CTA resident.
#include "fourstep_impl.cuh"

namespace gfft {
#define R(L, C, S) static FourStepReg<float, L, C, 16, S> fs_f32_##L##_##C##_##S;
R(15, 32, 2) R(16, 16, 2) R(16, 32, 2) R(17, 16, 2) R(17, 32, 2) R(18, 8, 2) R(18, 16, 2) R(19, 8, 2) R(19, 16, 2)
R(20, 4, 2) R(20, 8, 2) R(21, 8, 2) R(22, 4, 2) R(22, 4, 3) R(23, 4, 2) R(24, 2, 2)
#undef R
}  // namespace gfft
