// tiles_impl.cuh -- instantiation helper for the tile kernels; included by
// the per-type translation units (tiles_f32.cu, tiles_f64.cu).
#pragma once

#include "tiles.cuh"
#include "tiles_tma.cuh"
#include "tiles_registry.h"
#include "twiddle.h"
#include "../../include/genfft_gb300.h"

namespace gfft {

template <typename T, int LOGL, int E>
void tile_fill_tw(void *buf)
{
    stockham_fill_twiddles<T, LOGL, E>(
        static_cast<cpx<T> *>(buf), [](long long k, long long M, cpx<T> *w) { forward_root<T>(k, M, &w->x, &w->y); });
}

template <typename T, int V, int LOGL, int C, int E>
struct TileReg {
    TileReg()
    {
        TileKernel k;
        using SP = StockhamPlan<T, LOGL, E>;
        if constexpr (V == TILE_ROW_XPOSE) {
            using Cfg = RowCfg<T, LOGL, C, E>;
            k.fwd = (const void *)&k_rowpass<T, LOGL, C, E, false>;
            k.inv = (const void *)&k_rowpass<T, LOGL, C, E, true>;
            k.threads = Cfg::THREADS;
            k.smem = Cfg::SMEM;
            using TCfg = RowTmaCfg<T, LOGL, C, E>;
            if constexpr (TCfg::SMEM <= 220 * 1024 && SP::N * sizeof(cpx<T>) % 16 == 0) {
                k.tma_fwd = (const void *)&k_rowpass_tma<T, LOGL, C, E, false>;
                k.tma_inv = (const void *)&k_rowpass_tma<T, LOGL, C, E, true>;
                k.tma_threads = TCfg::THREADS;
                k.tma_smem = TCfg::SMEM;
            }
        } else {
            using Cfg = ColCfg<T, LOGL, C, E>;
            constexpr bool tw4 = V == TILE_COL_TW4, br = V == TILE_COL_BITREV, herm = V == TILE_COL_HERM;
            k.fwd = (const void *)&k_colpass<T, LOGL, C, E, false, tw4, br, herm>;
            k.inv = (const void *)&k_colpass<T, LOGL, C, E, true, tw4, br, herm>;
            k.threads = Cfg::THREADS;
            k.smem = Cfg::SMEM;
            using TCfg = ColTmaCfg<T, LOGL, C, E>;
            if constexpr (!br && TCfg::SMEM <= 220 * 1024 && C * sizeof(cpx<T>) % 16 == 0) {
                k.tma_fwd = (const void *)&k_colpass_tma<T, LOGL, C, E, false, tw4, herm>;
                k.tma_inv = (const void *)&k_colpass_tma<T, LOGL, C, E, true, tw4, herm>;
                k.tma_threads = TCfg::THREADS;
                k.tma_smem = TCfg::SMEM;
                k.tma_boxr = TCfg::BOXR;
                k.tma_rows = TCfg::N;
                k.tma_c = C;
            }
        }
        k.twcount = (size_t)SP::TW;
        k.fill = &tile_fill_tw<T, LOGL, E>;
        k.elem_bytes = (int)sizeof(cpx<T>);
        tile_register(sizeof(T) == 4 ? GFFT_F32 : GFFT_F64, V, LOGL, C, k);
    }
};

}  // namespace gfft
