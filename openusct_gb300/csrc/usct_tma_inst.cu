// usct_tma_inst.cu -- the TMA-ring kernels and their launchers for one
// shot-channel count C, given at compile time as -DUSCT_TMA_C=C.  The build
// compiles this file once per C in {1, 2, 4, 8, 16, 32, 64} (in parallel);
// usct_engine.cu dispatches on the plan's C.
#include <cuda_runtime.h>

#include "usct_tma.cuh"
#include "usct_tma2.cuh"

#ifndef USCT_TMA_C
#error "compile with -DUSCT_TMA_C=<shot channels>"
#endif

namespace usct {

namespace {
template <int kC, int TX, int TY_, bool D3>
int fwd_tile(const TmaLaunch& t, const FwdArgs& a, const FwdMaps& mp, bool born, bool pcs) {
    if constexpr (tma_tile_ok(TX, kC, D3)) {
        if (pcs) {
            if constexpr (kC >= 4) {
                k_forward_tma<TX, TY_, D3, false, kC, true>
                    <<<t.grid, dim3(TX, TY_), t.smem, t.stream>>>(a, mp, t.R, t.err);
                return 0;
            } else {
                return -1;
            }
        }
        if (born)
            k_forward_tma<TX, TY_, D3, true, kC>
                <<<t.grid, dim3(TX, TY_), t.smem, t.stream>>>(a, mp, t.R, t.err);
        else
            k_forward_tma<TX, TY_, D3, false, kC>
                <<<t.grid, dim3(TX, TY_), t.smem, t.stream>>>(a, mp, t.R, t.err);
        return 0;
    } else {
        return -1;
    }
}

template <int kC, int TX, int TY_, bool D3>
int adj_tile(const TmaLaunch& t, const AdjArgs& a, const AdjMaps& mp) {
    if constexpr (tma_tile_ok(TX, kC, D3)) {
        k_adjoint_tma<TX, TY_, D3, kC><<<t.grid, dim3(TX, TY_), t.smem, t.stream>>>(a, mp, t.R,
                                                                                 t.err);
        return 0;
    } else {
        return -1;
    }
}

constexpr int kFwd2Threads = 256;

template <int kC, int W, int H>
int fwd2_tile(const TmaLaunch2& t, const Fwd2Args& a, const Fwd2Maps& mp) {
    if constexpr (kC >= 8) {
        k_forward2_tma<W, H, kC, kFwd2Threads>
            <<<t.grid, kFwd2Threads, t.smem, t.stream>>>(a, mp, t.RA, t.RB, t.err);
        return 0;
    } else {
        return -1;
    }
}

template <int kC, int W, int H>
void allow_tile2(int bytes) {
    if constexpr (kC >= 8) {
        cudaFuncSetAttribute(k_forward2_tma<W, H, kC, kFwd2Threads>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    }
}

template <int kC, int TX, int TY_, bool D3>
void allow_tile(int bytes) {
    if constexpr (tma_tile_ok(TX, kC, D3)) {
        cudaFuncSetAttribute(k_forward_tma<TX, TY_, D3, false, kC>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaFuncSetAttribute(k_forward_tma<TX, TY_, D3, true, kC>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if constexpr (kC >= 4)
            cudaFuncSetAttribute(k_forward_tma<TX, TY_, D3, false, kC, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaFuncSetAttribute(k_adjoint_tma<TX, TY_, D3, kC>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    }
}
}  // namespace

// the tiles: 3D 32x4, 32x8, 64x2, 64x4; 2D 64x1, 128x1 (key = tile_x * 1000 + tile_y)
template <int kC>
int tma_forward(const TmaLaunch& t, const FwdArgs& a, const FwdMaps& mp, bool born, bool pcs) {
    const int key = t.txv * 1000 + t.ty;
    if (t.is3d) {
        switch (key) {
            case 32004: return fwd_tile<kC, 32, 4, true>(t, a, mp, born, pcs);
            case 32008: return fwd_tile<kC, 32, 8, true>(t, a, mp, born, pcs);
            case 64002: return fwd_tile<kC, 64, 2, true>(t, a, mp, born, pcs);
            case 64004: return fwd_tile<kC, 64, 4, true>(t, a, mp, born, pcs);
            default: return -1;
        }
    }
    switch (key) {
        case 64001: return fwd_tile<kC, 64, 1, false>(t, a, mp, born, pcs);
        case 128001: return fwd_tile<kC, 128, 1, false>(t, a, mp, born, pcs);
        default: return -1;
    }
}

template <int kC>
int tma_adjoint(const TmaLaunch& t, const AdjArgs& a, const AdjMaps& mp) {
    const int key = t.txv * 1000 + t.ty;
    if (t.is3d) {
        switch (key) {
            case 32004: return adj_tile<kC, 32, 4, true>(t, a, mp);
            case 32008: return adj_tile<kC, 32, 8, true>(t, a, mp);
            case 64002: return adj_tile<kC, 64, 2, true>(t, a, mp);
            case 64004: return adj_tile<kC, 64, 4, true>(t, a, mp);
            default: return -1;
        }
    }
    switch (key) {
        case 64001: return adj_tile<kC, 64, 1, false>(t, a, mp);
        case 128001: return adj_tile<kC, 128, 1, false>(t, a, mp);
        default: return -1;
    }
}

// the two-step tiles (key = W * 100 + H): 4x8, 8x4, 8x8, 16x4, 16x8
template <int kC>
int tma_forward2(const TmaLaunch2& t, const Fwd2Args& a, const Fwd2Maps& mp) {
    switch (t.w * 100 + t.h) {
        case 408: return fwd2_tile<kC, 4, 8>(t, a, mp);
        case 804: return fwd2_tile<kC, 8, 4>(t, a, mp);
        case 808: return fwd2_tile<kC, 8, 8>(t, a, mp);
        case 1604: return fwd2_tile<kC, 16, 4>(t, a, mp);
        case 1608: return fwd2_tile<kC, 16, 8>(t, a, mp);
        default: return -1;
    }
}

template <int kC>
void tma_allow_smem(int bytes) {
    allow_tile2<kC, 4, 8>(bytes);
    allow_tile2<kC, 8, 4>(bytes);
    allow_tile2<kC, 8, 8>(bytes);
    allow_tile2<kC, 16, 4>(bytes);
    allow_tile2<kC, 16, 8>(bytes);
    allow_tile<kC, 32, 4, true>(bytes);
    allow_tile<kC, 32, 8, true>(bytes);
    allow_tile<kC, 64, 2, true>(bytes);
    allow_tile<kC, 64, 4, true>(bytes);
    allow_tile<kC, 64, 1, false>(bytes);
    allow_tile<kC, 128, 1, false>(bytes);
}

template int tma_forward<USCT_TMA_C>(const TmaLaunch&, const FwdArgs&, const FwdMaps&, bool, bool);
template int tma_adjoint<USCT_TMA_C>(const TmaLaunch&, const AdjArgs&, const AdjMaps&);
template void tma_allow_smem<USCT_TMA_C>(int);
template int tma_forward2<USCT_TMA_C>(const TmaLaunch2&, const Fwd2Args&, const Fwd2Maps&);

}  // namespace usct
