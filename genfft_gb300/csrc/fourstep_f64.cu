// fourstep_f64.cu -- double persistent four-step kernels, n = 2^14 .. 2^24
// (see fourstep.cuh), tiles capped at 512 compute threads.
#include "fourstep_impl.cuh"

namespace gfft {
#define R(L, C, S) static FourStepReg<double, L, C, 8, S> fs_f64_##L##_##C##_##S;
R(14, 16, 2) R(15, 16, 2) R(16, 8, 2) R(17, 16, 2) R(18, 8, 2) R(19, 8, 2) R(20, 4, 2) R(21, 4, 2) R(22, 2, 2)
R(23, 2, 2) R(24, 1, 2)
#undef R
}  // namespace gfft
