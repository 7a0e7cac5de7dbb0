// fourstep2_f32.cu -- registrations of the pair-packed persistent four-step
// kernel (fourstep2.cuh), fp32 n = 2^16 .. 2^23.  R(logn, E, CT, NS): E
// pair points a thread, CT compute threads, NS shared-memory stages.
#include "fourstep2.cuh"
#include "fourstep_impl.cuh"

namespace gfft {

template <int LOGN, int E, int CT, int NS>
struct Fs2Reg {
    static constexpr int LA = LOGN / 2, LB = LOGN - LA;
    using Cfg = Fs2Cfg<LA, LB, E, CT, NS>;
    Fs2Reg()
    {
        if constexpr (Cfg::FITS) {
            FourStepKernel k;
            k.fwd = (const void *)&k_fs2<LA, LB, E, CT, NS, false>;
            k.inv = (const void *)&k_fs2<LA, LB, E, CT, NS, true>;
            k.threads = Cfg::THREADS;
            k.smem = Cfg::SMEM;
            k.la = LA;
            k.lb = LB;
            k.cc = Cfg::CC;
            k.cr = Cfg::CR;
            k.nc = Cfg::NC;
            k.nr = Cfg::NR;
            k.nrp = 0;
            k.boxr = Cfg::BOXR;
            k.ns = NS;
            k.twa = (size_t)StockhamPlan<float, LA, E>::TW;
            k.twb = (size_t)StockhamPlan<float, LB, E>::TW;
            k.fill_a = &fs_fill_tw<float, LA, E>;
            k.fill_b = &fs_fill_tw<float, LB, E>;
            k.pair = true;
            fourstep_register(GFFT_F32, LOGN, k);
        }
    }
};

#ifndef FS2_SET
#define FS2_SET 0
#endif
#define R(L, E, C, S) static Fs2Reg<L, E, C, S> fs2_f32_##L##_##E##_##C##_##S;
#if FS2_SET == 0
R(22, 16, 256, 2) R(22, 16, 256, 1) R(22, 8, 512, 1) R(23, 16, 256, 1) R(16, 8, 256, 2) R(17, 8, 256, 2)
#else
R(18, 16, 256, 2) R(18, 8, 256, 2) R(19, 16, 256, 2) R(19, 8, 256, 2) R(20, 16, 256, 2) R(20, 8, 512, 1)
R(20, 8, 256, 2) R(21, 16, 256, 2)
#endif
#undef R
}  // namespace gfft
