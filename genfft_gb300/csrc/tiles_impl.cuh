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
            using TCfg1 = RowTmaCfg<T, LOGL, C, E, 1>;
            if constexpr (TCfg::SMEM <= 220 * 1024 && SP::N * sizeof(cpx<T>) % 16 == 0) {
                k.tma_fwd = (const void *)&k_rowpass_tma<T, LOGL, C, E, false>;
                k.tma_inv = (const void *)&k_rowpass_tma<T, LOGL, C, E, true>;
                k.tma_threads = TCfg::THREADS;
                k.tma_smem = TCfg::SMEM;
                k.tma_stages = 2;
            } else if constexpr (LOGL >= 12 && TCfg1::SMEM <= 220 * 1024 && SP::N * sizeof(cpx<T>) % 16 == 0) {
                // single-buffered rows only where the double-buffered tile
                // is two rows (16-byte store runs): measured on GB300 at
                // n = 2^23 / 2^24 +18 % / +19 %; against four- or eight-row
                // double-buffered tiles (n = 2^20 .. 2^22) it is slower
                k.tma_fwd = (const void *)&k_rowpass_tma<T, LOGL, C, E, false, 1>;
                k.tma_inv = (const void *)&k_rowpass_tma<T, LOGL, C, E, true, 1>;
                k.tma_threads = TCfg1::THREADS;
                k.tma_smem = TCfg1::SMEM;
                k.tma_stages = 1;
                k.tma_row = true;
            }
        } else {
            using Cfg = ColCfg<T, LOGL, C, E>;
            constexpr bool tw4 = V == TILE_COL_TW4, br = V == TILE_COL_BITREV, herm = V == TILE_COL_HERM;
            constexpr int twm = tw4 ? 1 : V == TILE_COL_TWB ? 2 : 0;
            k.fwd = (const void *)&k_colpass<T, LOGL, C, E, false, twm, br, herm>;
            k.inv = (const void *)&k_colpass<T, LOGL, C, E, true, twm, br, herm>;
            k.threads = Cfg::THREADS;
            k.smem = Cfg::SMEM;
            using TCfg = ColTmaCfg<T, LOGL, C, E>;
            using TCfg1 = ColTmaCfg<T, LOGL, C, E, 1>;
            if constexpr (!br && TCfg::SMEM <= 220 * 1024 && C * sizeof(cpx<T>) % 16 == 0) {
                k.tma_fwd = (const void *)&k_colpass_tma<T, LOGL, C, E, false, twm, herm>;
                k.tma_inv = (const void *)&k_colpass_tma<T, LOGL, C, E, true, twm, herm>;
                k.tma_threads = TCfg::THREADS;
                k.tma_smem = TCfg::SMEM;
                k.tma_boxr = TCfg::BOXR;
                k.tma_rows = TCfg::N;
                k.tma_c = C;
                k.tma_stages = 2;
            } else if constexpr (tw4 && TCfg1::SMEM <= 220 * 1024 && C * sizeof(cpx<T>) % 16 == 0) {
                // four-step column pass only: measured on GB300, the wider
                // single-buffered tile beats the narrower double-buffered one
                // (n = 2^20 .. 2^24: 7-42 %); for 2D columns it does not
                k.tma_fwd = (const void *)&k_colpass_tma<T, LOGL, C, E, false, twm, herm, 1>;
                k.tma_inv = (const void *)&k_colpass_tma<T, LOGL, C, E, true, twm, herm, 1>;
                k.tma_threads = TCfg1::THREADS;
                k.tma_smem = TCfg1::SMEM;
                k.tma_boxr = TCfg1::BOXR;
                k.tma_rows = TCfg1::N;
                k.tma_c = C;
                k.tma_stages = 1;
            }
        }
        k.twcount = (size_t)SP::TW;
        k.fill = &tile_fill_tw<T, LOGL, E>;
        k.elem_bytes = (int)sizeof(cpx<T>);
        tile_register(sizeof(T) == 4 ? GFFT_F32 : GFFT_F64, V, LOGL, C, k);
    }
};

}  // namespace gfft
