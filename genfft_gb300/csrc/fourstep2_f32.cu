// fourstep2_f32.cu -- registrations of the pair-packed persistent four-step
// kernel (fourstep2.cuh), fp32 n = 2^18 .. 2^22.  R(logn, CT, NS): CT
// compute threads, NS shared-memory stages.
#include "fourstep2.cuh"
#include "fourstep_impl.cuh"

namespace gfft {

template <int LOGN, int CT, int NS>
struct Fs2Reg {
    static constexpr int LA = LOGN / 2, LB = LOGN - LA;
    using Cfg = Fs2Cfg<LA, LB, CT, NS>;
    Fs2Reg()
    {
        if constexpr (Cfg::FITS) {
            FourStepKernel k;
            k.fwd = (const void *)&k_fs2<LA, LB, CT, NS, false>;
            k.inv = (const void *)&k_fs2<LA, LB, CT, NS, true>;
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
            k.twa = (size_t)StockhamPlan<float, LA, 16>::TW;
            k.twb = (size_t)StockhamPlan<float, LB, 16>::TW;
            k.fill_a = &fs_fill_tw<float, LA, 16>;
            k.fill_b = &fs_fill_tw<float, LB, 16>;
            k.pair = true;
            fourstep_register(GFFT_F32, LOGN, k);
        }
    }
};

#define R(L, C, S) static Fs2Reg<L, C, S> fs2_f32_##L##_##C##_##S;
R(18, 256, 2) R(19, 256, 2) R(20, 256, 2) R(21, 256, 2) R(22, 256, 2) R(22, 256, 1)
#undef R
}  // namespace gfft
