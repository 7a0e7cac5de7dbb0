// fourstep_impl.cuh -- registration helper for the persistent four-step
// kernels; included by the per-type translation units.
#pragma once

#include "fourstep.cuh"
#include "fourstep.h"
#include "twiddle.h"
#include "../../include/genfft_gb300.h"

namespace gfft {

template <typename T, int L, int E>
void fs_fill_tw(void *buf)
{
    stockham_fill_twiddles<T, L, E>(static_cast<cpx<T> *>(buf),
                                    [](long long k, long long M, cpx<T> *w) { forward_root<T>(k, M, &w->x, &w->y); });
}

template <typename T, int LOGN, int CC, int E, int NS>
struct FourStepReg {
    FourStepReg()
    {
        constexpr int LA = LOGN / 2, LB = LOGN - LA;
        using Cfg = FourStepCfg<T, LA, LB, CC, E, NS>;
        if constexpr (Cfg::FITS) reg();
    }
    void reg()
    {
        constexpr int LA = LOGN / 2, LB = LOGN - LA;
        using Cfg = FourStepCfg<T, LA, LB, CC, E, NS>;
        FourStepKernel k;
        k.fwd = (const void *)&k_fourstep<T, LA, LB, CC, E, NS, false>;
        k.inv = (const void *)&k_fourstep<T, LA, LB, CC, E, NS, true>;
        if constexpr (sizeof(T) == 4 && Cfg::CR >= 2 && Cfg::SPB::P > 1)
            k.dit = (const void *)&k_fourstep<T, LA, LB, CC, E, NS, false, true>;
        k.threads = Cfg::THREADS;
        k.smem = Cfg::SMEM;
        k.la = LA;
        k.lb = LB;
        k.cc = CC;
        k.cr = Cfg::CR;
        k.nc = Cfg::NC;
        k.nr = Cfg::NR;
        k.nrp = Cfg::NRP;
        k.boxr = Cfg::BOXR;
        k.ns = NS;
        k.twa = (size_t)StockhamPlan<T, LA, E>::TW;
        k.twb = (size_t)StockhamPlan<T, LB, E>::TW;
        k.fill_a = &fs_fill_tw<T, LA, E>;
        k.fill_b = &fs_fill_tw<T, LB, E>;
        fourstep_register(sizeof(T) == 4 ? GFFT_F32 : GFFT_F64, LOGN, k);
    }
};

}  // namespace gfft
