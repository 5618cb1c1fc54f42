// usct_tma.cuh -- TMA-fed pipelined variants of the forward and adjoint stencils.
//
// Same arithmetic, same op order, same outputs as k_forward / k_adjoint
// (usct_kernels.cuh); only the way planes reach shared memory differs.  Each
// CTA keeps a ring of R plane stages in shared memory.  One elected thread
// issues cp.async.bulk.tensor copies (one per field per plane: the halo tile
// of p^{n-1} -- TY+2 rows of (cells+2)*C floats --, the own tile of p^{n-2},
// the model cells) for plane z+R-1 while every warp computes plane z from the
// stages of z-1, z and z+1; completion is tracked by one mbarrier per stage
// (expect_tx byte counts).  Bytes in flight per SM no longer cost registers,
// which is what limited the register-queue kernels (long-scoreboard stalls at
// 25 % occupancy).  Out-of-range planes, rows and cells are zero-filled by the
// tensor copy itself.
//
// Waits are bounded: a stage that does not complete within kWaitNs sets *err,
// the CTA drains (again bounded) the copies it issued and returns; once *err is
// set every later launch returns before issuing anything, and the host reports
// the flag (usct_plan_check).
#pragma once

#include <cuda.h>

#include "usct_kernels.cuh"

namespace usct {

constexpr unsigned long long kWaitNs = 250000000ull;   // 250 ms per stage wait
constexpr int kSpinCap = 1 << 26;                      // backstop on the poll count
constexpr uint32_t kSuspendNs = 1000000u;              // longest single suspension (1 ms)

// The kernels take the shot-channel count C as a template parameter: every
// row length, halo width and cell shift is then a constant and the shared
// memory addresses fold into immediate offsets (a fifth fewer instructions than
// with C read from the arguments).  A (tile, C) pair has a TMA kernel when a
// thread's 4 floats never straddle a tile row end: C >= 4 with whole cells per
// 4-float group, or C < 4 on the 3D 32-wide tiles.
__host__ __device__ constexpr int ilog2c(int c) { return c >= 64 ? 6 : c >= 32 ? 5 : c >= 16 ? 4 : c >= 8 ? 3 : c >= 4 ? 2 : c >= 2 ? 1 : 0; }
__host__ __device__ constexpr bool tma_tile_ok(int txv, int c, bool is3d) {
    return c >= 4 ? (((4 * txv) >> ilog2c(c)) % 4 == 0) : (is3d && txv == 32);
}

struct FwdMaps {
    CUtensorMap pc, pp, S, sp, dc, dpp, vm;
};
struct AdjMaps {
    CUtensorMap l1, S, l2, d2, sp, g;
};

__host__ __device__ constexpr int al32(int x) { return (x + 31) & ~31; }

// Stage layout in floats, shared by host (smem sizing) and device.
struct FwdStage {
    int o_pp, o_S, o_sp, o_dc, o_dpp, o_vm, floats;
};
// pcs: the model S per group of four shot channels (one value per lane)
__host__ __device__ inline FwdStage fwd_stage(int TXV, int TY, bool is3d, bool born, int C, int logC,
                                              bool has_sp, bool pcs = false) {
    const int HF = C < 4 ? 4 : C;
    const int TXF = 4 * TXV;
    const int rows = TY + (is3d ? 2 : 0);
    const int SR = TXF + 2 * HF;
    const int cells = TXF >> logC;
    FwdStage s{};
    s.o_pp = al32(rows * SR);
    s.o_S = s.o_pp + al32(TY * TXF);
    s.o_sp = s.o_S + al32(TY * (pcs ? TXF / 4 : cells));
    int end = s.o_sp + (has_sp ? al32(TY * cells) : 0);
    s.o_dc = end;
    if (born) {
        s.o_dpp = s.o_dc + al32(rows * SR);
        s.o_vm = s.o_dpp + al32(TY * TXF);
        end = s.o_vm + al32(TY * cells);
    }
    s.floats = end;
    return s;
}

struct AdjStage {
    int o_S, o_l2, o_d2, o_sp, o_g, floats;
};
__host__ __device__ inline AdjStage adj_stage(int TXV, int TY, bool is3d, int C, int logC, bool has_sp,
                                              bool has_g) {
    const int HF = C < 4 ? 4 : C;
    const int TXF = 4 * TXV;
    const int rows = TY + (is3d ? 2 : 0);
    const int SR = TXF + 2 * HF;
    const int cells = TXF >> logC;
    AdjStage s{};
    s.o_S = al32(rows * SR);
    s.o_l2 = s.o_S + al32(rows * (cells + 8));
    s.o_d2 = s.o_l2 + al32(TY * TXF);
    s.o_sp = s.o_d2 + al32(TY * TXF);
    s.o_g = s.o_sp + (has_sp ? al32(TY * cells) : 0);
    s.floats = s.o_g + (has_g ? al32(2 * TY * cells) : 0);
    return s;
}

// ---- PTX wrappers ----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// test the phase of the given parity; a warp whose phase has not completed is
// suspended by the hardware until it completes (or kSuspendNs passes) instead
// of spinning on issue slots the computing warps need
__device__ __forceinline__ bool mbar_wait_suspend(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// bounded wait for the stage barrier b to complete the phase of the given parity
__device__ __forceinline__ bool wait_bar(uint64_t* b, uint32_t parity) {
    if (mbar_wait_suspend(b, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (int it = 1; it < kSpinCap; ++it) {
        if (mbar_wait_suspend(b, parity)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}
// local plane i of a ring of R stages (used on the rare drain path only)
__device__ __forceinline__ bool wait_stage(uint64_t* bars, int i, int R) {
    return wait_bar(bars + (i % R), (uint32_t)((i / R) & 1));
}
// every thread of the CTA learns whether an earlier wait already gave up
// (flag word in shared memory right after the R stage barriers)
__device__ __forceinline__ bool aborted(const int* err, int* s_abort) {
    if (threadIdx.x == 0 && threadIdx.y == 0) *s_abort = *reinterpret_cast<const volatile int*>(err);
    __syncthreads();
    return *s_abort != 0;
}
__device__ __forceinline__ void tma3(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                     int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}
__device__ __forceinline__ void tma4(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                     int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2),
        "r"(c3)
        : "memory");
}

// cell-layout row (smem) expanded to the 4 floats starting at float lf
__device__ __forceinline__ float4 cell4s(const float* row, int lf, int logC) {
    if (logC == 0) return ld4(row + lf);
    if (logC == 1) {
        const float2 s = *reinterpret_cast<const float2*>(row + (lf >> 1));
        return make_float4(s.x, s.x, s.y, s.y);
    }
    const float s = row[lf >> logC];
    return make_float4(s, s, s, s);
}

// Paired FP32 arithmetic on float4 (two lanes per instruction on sm_100+).
// Every lane is rounded exactly as the scalar operation would be, so results
// stay bit-identical to the scalar op order of the oracle.
__device__ __forceinline__ float2 lo2(const float4& a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ float2 hi2(const float4& a) { return make_float2(a.z, a.w); }
__device__ __forceinline__ float4 cat4(const float2& l, const float2& h) {
    return make_float4(l.x, l.y, h.x, h.y);
}
__device__ __forceinline__ float4 add4(const float4& a, const float4& b) {
    return cat4(__fadd2_rn(lo2(a), lo2(b)), __fadd2_rn(hi2(a), hi2(b)));
}
__device__ __forceinline__ float4 mul4(const float4& a, const float4& b) {
    return cat4(__fmul2_rn(lo2(a), lo2(b)), __fmul2_rn(hi2(a), hi2(b)));
}
__device__ __forceinline__ float4 fma4(const float4& a, const float4& b, const float4& c) {
    return cat4(__ffma2_rn(lo2(a), lo2(b), lo2(c)), __ffma2_rn(hi2(a), hi2(b), hi2(c)));
}
__device__ __forceinline__ float4 neg4(const float4& a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
__device__ __forceinline__ float4 splat4(float v) { return make_float4(v, v, v, v); }
__device__ __forceinline__ float4 sel4(const bool in[4], const float4& a) {
    return make_float4(in[0] ? a.x : 0.f, in[1] ? a.y : 0.f, in[2] ? a.z : 0.f, in[3] ? a.w : 0.f);
}
// The stencil of usct_kernels.cuh's stencil(), four lanes at once:
// lap = fma(cen, c, ((x- + x+) [+ (y- + y+)]) + (z- + z+)) * inv_h2, 0 off the interior.
// Border lanes (x, y or z on the grid's outer layer) get 0.  The forward
// kernel tests whether all four lanes are interior -- true on all but the
// outermost tiles -- and only otherwise builds the per-lane mask (fewer
// instructions: 2D sweeps 5 % faster); the adjoint keeps the always-masked form
// below (stencil4m), measured faster there.
__device__ __forceinline__ float4 stencil4(bool all_in, bool zy_in, const bool x_in[4], float cen,
                                           const float4& c, const float4& xm, const float4& xp,
                                           const float4& ym, const float4& yp, const float4& zm,
                                           const float4& zp, bool is3d, float inv_h2) {
    float4 t = add4(xm, xp);
    if (is3d) t = add4(t, add4(ym, yp));
    t = add4(t, add4(zm, zp));
    float4 l = mul4(fma4(splat4(cen), c, t), splat4(inv_h2));
    if (__builtin_expect(!all_in, 0)) {
        bool in[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) in[q] = zy_in && x_in[q];
        l = sel4(in, l);
    }
    return l;
}
// the same with the mask always applied (the adjoint's form: measured faster
// there than testing for an interior group first)
__device__ __forceinline__ float4 stencil4m(const bool in[4], float cen, const float4& c,
                                            const float4& xm, const float4& xp, const float4& ym,
                                            const float4& yp, const float4& zm, const float4& zp,
                                            bool is3d, float inv_h2) {
    float4 t = add4(xm, xp);
    if (is3d) t = add4(t, add4(ym, yp));
    t = add4(t, add4(zm, zp));
    return sel4(in, mul4(fma4(splat4(cen), c, t), splat4(inv_h2)));
}
__device__ __forceinline__ void put4(float* d, const float4& v) {
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
}

// Source injection and receiver sampling for the planes that have entries,
// out of line: kept as calls, their bodies cannot be predicated into every
// plane's instruction stream (they run on a few planes of a few tiles).
struct SrcStep {
    float4 lap;
    int si, snz;
};
static __device__ __noinline__ SrcStep add_sources(float4 lap4, const SrcEnt* __restrict__ ent, int si,
                                            int se, int z, int ty, int tx, float wv) {
    float lap[4] = {lap4.x, lap4.y, lap4.z, lap4.w};
    while (si < se) {
        const SrcEnt e = ent[si];
        if (e.z != z) break;
        if (e.ly == ty) {
            const int d = e.f - 4 * tx;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (d == q) lap[q] = lap[q] + e.w * wv;
        }
        ++si;
    }
    return SrcStep{make_float4(lap[0], lap[1], lap[2], lap[3]), si,
                   si < se ? ent[si].z : 0x7fffffff};
}
struct RxStep {
    int ri, rnz;
};
static __device__ __noinline__ RxStep record_receivers(float4 out4, const RxEnt* __restrict__ ent, int ri,
                                                int re, int z, int ty, int tx, int C,
                                                float* __restrict__ rs) {
    const float out[4] = {out4.x, out4.y, out4.z, out4.w};
    while (ri < re) {
        const RxEnt e = ent[ri];
        if (e.z != z) break;
        if (e.ly == ty) {
            const int base = e.lcell * C - 4 * tx;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = q - base;
                if (c >= 0 && c < C) rs[(long long)e.slot * C + c] = e.w * out[q];
            }
        }
        ++ri;
    }
    return RxStep{ri, ri < re ? ent[ri].z : 0x7fffffff};
}

// adjoint injection lam^k[rx] -= r^k * w for the planes with receivers
struct InjStep {
    float4 lk;
    int ri, rnz;
};
static __device__ __noinline__ InjStep inject_residuals(float4 lk4, const RxEnt* __restrict__ ent,
                                                       int ri, int re, int z, int ty, int tx, int C,
                                                       const float* __restrict__ res) {
    float lk[4] = {lk4.x, lk4.y, lk4.z, lk4.w};
    while (ri < re) {
        const RxEnt e = ent[ri];
        if (e.z != z) break;
        if (e.ly == ty) {
            const int base = e.lcell * C - 4 * tx;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = q - base;
                if (c >= 0 && c < C) lk[q] = lk[q] - res[(long long)e.j * C + c] * e.w;
            }
        }
        ++ri;
    }
    return InjStep{make_float4(lk[0], lk[1], lk[2], lk[3]), ri, ri < re ? ent[ri].z : 0x7fffffff};
}

// ---------------------------------------------------------------------------
// forward step, TMA ring
// ---------------------------------------------------------------------------
// PCS: the shot channels carry their own models -- the shots of co-admitted
// requests on different models advancing in one launch; forward sweeps only,
// C >= 4.  S is stored per group of four channels, [z][y][x][C/4]: a lane's
// float4 holds four channels of one cell, so lane tx reads quad tx of the
// tile row (C/4 floats per cell, where the wavefields hold C).
template <int TXV, int TY, bool IS3D, bool BORN, int C, bool PCS = false>
__global__ void __launch_bounds__(TXV* TY, BORN ? ((TXV * TY >= 256) ? 2 : 4) : ((TXV * TY >= 256) ? 4 : 8)) k_forward_tma(const FwdArgs a, const __grid_constant__ FwdMaps mp,
                                                         const int R, int* err) {
    extern __shared__ __align__(128) float smf[];
    const Geo& g = a.g;
    constexpr int logC = ilog2c(C);
    constexpr int HF = C < 4 ? 4 : C;
    constexpr int HR = IS3D ? 1 : 0;
    constexpr int TXF = 4 * TXV;
    constexpr int ROWS = TY + 2 * HR;
    constexpr int SR = TXF + 2 * HF;
    constexpr int cells = TXF >> logC;
    const bool has_sp = a.sp != nullptr;
    static_assert(!PCS || (!BORN && C >= 4), "per-channel models: forward sweeps with C >= 4");
    const FwdStage L = fwd_stage(TXV, TY, IS3D, BORN, C, logC, has_sp, PCS);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smf + (size_t)R * L.floats);

    const int tx = threadIdx.x;
    const int ty = (TY > 1) ? (int)threadIdx.y : 0;
    const int tid = tx + TXV * ty;
    const int fx0 = blockIdx.x * TXF;
    const int x0c = fx0 >> logC;
    const int y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * g.zc;
    const int z1 = min(z0 + g.zc, g.nz);
    const int nloc = z1 - z0 + 2;   // local planes z0-1 .. z1
    const int f = fx0 + 4 * tx;
    const int y = y0 + ty;
    const bool own = (f < g.RP) && (y < g.ny);
    const int col = HF + 4 * tx;
    const int r = ty + HR;
    const long long ro = (long long)y * g.RP + f;
    const bool y_in = !IS3D || (y >= 1 && y <= g.ny - 2);
    bool x_in[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int xq = (f + q) >> logC;
        x_in[q] = xq >= 1 && xq <= g.nx - 2;
    }
    const bool x_all = x_in[0] && x_in[1] && x_in[2] && x_in[3];
    const float cen = IS3D ? -6.f : -4.f;
    const float inv_h2 = g.inv_h2;
    const float wv = a.wav[a.n - 1];

    const uint32_t b_halo = (uint32_t)(ROWS * SR * 4), b_own = (uint32_t)(TY * TXF * 4),
                   b_cell = (uint32_t)(TY * cells * 4), b_quad = (uint32_t)(TY * TXV * 4);
    auto issue = [&](int i, int slot) {
        const int p = z0 - 1 + i;
        float* st = smf + (size_t)slot * L.floats;
        uint64_t* bar = bars + slot;
        const bool inner = i >= 1 && i <= nloc - 2;
        uint32_t bytes = b_halo * (BORN ? 2u : 1u);
        if (inner)
            bytes += b_own * (BORN ? 2u : 1u) + (PCS ? b_quad : b_cell) +
                     b_cell * ((has_sp ? 1u : 0u) + (BORN ? 1u : 0u));
        if (a.wait_test && i == 0) bytes += 16u;   // never delivered: exercises the bounded wait
        mbar_expect_tx(bar, bytes);
        if (C >= 4) tma4(st, &mp.pc, bar, 0, x0c - 1, y0 - HR, p);
        else tma3(st, &mp.pc, bar, fx0 - 4, y0 - HR, p);
        if (BORN) {
            if (C >= 4) tma4(st + L.o_dc, &mp.dc, bar, 0, x0c - 1, y0 - HR, p);
            else tma3(st + L.o_dc, &mp.dc, bar, fx0 - 4, y0 - HR, p);
        }
        if (inner) {
            if (C >= 4) tma4(st + L.o_pp, &mp.pp, bar, 0, x0c, y0, p);
            else tma3(st + L.o_pp, &mp.pp, bar, fx0, y0, p);
            if (PCS) tma3(st + L.o_S, &mp.S, bar, fx0 >> 2, y0, p);   // quads: TXV a row
            else tma3(st + L.o_S, &mp.S, bar, x0c, y0, p);
            if (has_sp) tma3(st + L.o_sp, &mp.sp, bar, x0c, y0, p);
            if (BORN) {
                if (C >= 4) tma4(st + L.o_dpp, &mp.dpp, bar, 0, x0c, y0, p);
                else tma3(st + L.o_dpp, &mp.dpp, bar, fx0, y0, p);
                tma3(st + L.o_vm, &mp.vm, bar, x0c, y0, p);
            }
        }
    };

    if (aborted(err, reinterpret_cast<int*>(bars + R))) return;
    if (tid == 0) {
        for (int s = 0; s < R; ++s) mbar_init(bars + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int npro = min(R, nloc);
    if (tid == 0)
        for (int i = 0; i < npro; ++i) issue(i, i);
    int issued = npro;

    // per-tile entry cursors
    const int tile = blockIdx.x + g.ntiles_x * blockIdx.y;
    int si = a.s_ptr ? a.s_ptr[tile] : 0;
    const int se = a.s_ptr ? a.s_ptr[tile + 1] : 0;
    while (si < se && a.s_ent[si].z < z0) ++si;
    int snz = si < se ? a.s_ent[si].z : 0x7fffffff;
    int ri = 0, re = 0;
    if (a.rs) {
        ri = a.r_ptr[tile];
        re = a.r_ptr[tile + 1];
        while (ri < re && a.r_ent[ri].z < z0) ++ri;
    }
    int rnz = ri < re ? a.r_ent[ri].z : 0x7fffffff;

    // ring bookkeeping without divisions: slots of local planes im, im+1, im+2
    // and the phase parity of the stage being waited for
    int s_m = 0, s_c = 1, s_p = 2 % R;
    uint32_t ph_p = (R == 2) ? 1u : 0u;
    bool ok = wait_bar(bars + 0, 0u);
    ok = wait_bar(bars + 1, 0u) && ok;
    float* pn_ptr = a.pn + (long long)z0 * g.PP + ro;
    float* ck_ptr = a.ck ? a.ck + (long long)z0 * g.PP + ro : nullptr;
    float* d2_ptr = a.d2 ? a.d2 + (long long)z0 * g.PP + ro : nullptr;
    float* dn_ptr = BORN ? a.dn + (long long)z0 * g.PP + ro : nullptr;
    for (int z = z0; z < z1; ++z) {
        const int im = z - z0;
        ok = wait_bar(bars + s_p, ph_p) && ok;
        const float* sm_m = smf + (size_t)s_m * L.floats;
        const float* sm_c = smf + (size_t)s_c * L.floats;
        const float* sm_p = smf + (size_t)s_p * L.floats;

        const float4 cc = ld4(sm_c + r * SR + col);
        float4 xm, xp;
        xnb(sm_c + r * SR, col, C, cc, xm, xp);
        float4 ym = f4zero(), yp = f4zero();
        if (IS3D) {
            ym = ld4(sm_c + (r - 1) * SR + col);
            yp = ld4(sm_c + (r + 1) * SR + col);
        }
        const float4 cm = ld4(sm_m + r * SR + col);
        const float4 cp = ld4(sm_p + r * SR + col);
        const float4 ppv = ld4(sm_c + L.o_pp + ty * TXF + 4 * tx);
        const float4 Sv = PCS ? splat4(sm_c[L.o_S + ty * TXV + tx])
                              : cell4s(sm_c + L.o_S + ty * cells, 4 * tx, logC);
        const float4 spv = has_sp ? cell4s(sm_c + L.o_sp + ty * cells, 4 * tx, logC) : f4zero();
        const bool zy_in = y_in && z >= 1 && z <= g.nz - 2;
        const bool all_in = zy_in && x_all;
        float lap[4];
        put4(lap, stencil4(all_in, zy_in, x_in, cen, cc, xm, xp, ym, yp, cm, cp, IS3D, inv_h2));
        if (__builtin_expect(z == snz, 0)) {
            const SrcStep st = add_sources(make_float4(lap[0], lap[1], lap[2], lap[3]), a.s_ent,
                                           si, se, z, ty, tx, wv);
            put4(lap, st.lap);
            si = st.si;
            snz = st.snz;
        }
        // p^n = fma(S, lap, 2c - p^{n-2}) with 2c - p computed as fma(2, c, -p) (2c is exact)
        float4 v4 = fma4(Sv, make_float4(lap[0], lap[1], lap[2], lap[3]),
                         fma4(splat4(2.f), cc, neg4(ppv)));
        if (has_sp) v4 = mul4(v4, spv);
        float pn[4], d2v[4], out[4];
        put4(pn, v4);
        put4(out, v4);
        if (BORN || d2_ptr) put4(d2v, add4(fma4(splat4(-2.f), cc, v4), ppv));   // (p^n - 2c) + p
        if (BORN) {
            const float* dcs = sm_c + L.o_dc;
            const float4 dcc = ld4(dcs + r * SR + col);
            float4 dxm, dxp;
            xnb(dcs + r * SR, col, C, dcc, dxm, dxp);
            float4 dym = f4zero(), dyp = f4zero();
            if (IS3D) {
                dym = ld4(dcs + (r - 1) * SR + col);
                dyp = ld4(dcs + (r + 1) * SR + col);
            }
            const float4 dm = ld4(sm_m + L.o_dc + r * SR + col);
            const float4 dp = ld4(sm_p + L.o_dc + r * SR + col);
            const float4 dppv = ld4(sm_c + L.o_dpp + ty * TXF + 4 * tx);
            const float4 vmv = cell4s(sm_c + L.o_vm + ty * cells, 4 * tx, logC);
            const float4 dl = stencil4(all_in, zy_in, x_in, cen, dcc, dxm, dxp, dym, dyp, dm, dp, IS3D, inv_h2);
            float4 dv = fma4(Sv, dl, fma4(splat4(2.f), dcc, neg4(dppv)));
            dv = fma4(neg4(vmv), make_float4(d2v[0], d2v[1], d2v[2], d2v[3]), dv);
            if (has_sp) dv = mul4(dv, spv);
            put4(out, dv);
            if (own) st4(dn_ptr, dv);
        }
        if (own) {
            const float4 v = make_float4(pn[0], pn[1], pn[2], pn[3]);
            st4(pn_ptr, v);
            if (ck_ptr) st4(ck_ptr, v);
            if (d2_ptr) st4(d2_ptr, make_float4(d2v[0], d2v[1], d2v[2], d2v[3]));
        }
        pn_ptr += g.PP;
        if (ck_ptr) ck_ptr += g.PP;
        if (d2_ptr) d2_ptr += g.PP;
        if (BORN) dn_ptr += g.PP;
        if (__builtin_expect(z == rnz, 0)) {
            const RxStep st = record_receivers(make_float4(out[0], out[1], out[2], out[3]), a.r_ent,
                                               ri, re, z, ty, tx, C, a.rs);
            ri = st.ri;
            rnz = st.rnz;
        }

        // everyone is done with the stage of plane z-1: refill it with plane z-1+R
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        if (tid == 0 && im + R < nloc) {
            fence_proxy_async();
            issue(im + R, s_m);
        }
        if (im + R < nloc) issued = im + R + 1;
        s_m = s_c;
        s_c = s_p;
        if (++s_p == R) { s_p = 0; ph_p ^= 1u; }
    }
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // drain what was issued so no copy lands in a retired CTA's memory
        for (int i = (issued > R ? issued - R : 0); i < issued; ++i) (void)wait_stage(bars, i, R);
    }
}

// ---------------------------------------------------------------------------
// adjoint step, TMA ring
// ---------------------------------------------------------------------------
template <int TXV, int TY, bool IS3D, int C>
__global__ void __launch_bounds__(TXV* TY, (TXV * TY >= 256) ? 3 : 4) k_adjoint_tma(const AdjArgs a, const __grid_constant__ AdjMaps mp,
                                                         const int R, int* err) {
    extern __shared__ __align__(128) float smf[];
    const Geo& g = a.g;
    constexpr int logC = ilog2c(C);
    constexpr int HF = C < 4 ? 4 : C;
    constexpr int HR = IS3D ? 1 : 0;
    constexpr int TXF = 4 * TXV;
    constexpr int ROWS = TY + 2 * HR;
    constexpr int SR = TXF + 2 * HF;
    constexpr int cells = TXF >> logC;
    constexpr int SH = cells + 8;   // S halo row length (cells)
    const bool has_sp = a.sp != nullptr;
    const bool has_g = a.gacc != nullptr;
    const AdjStage L = adj_stage(TXV, TY, IS3D, C, logC, has_sp, has_g);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smf + (size_t)R * L.floats);

    const int tx = threadIdx.x;
    const int ty = (TY > 1) ? (int)threadIdx.y : 0;
    const int tid = tx + TXV * ty;
    const int fx0 = blockIdx.x * TXF;
    const int x0c = fx0 >> logC;
    const int y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * g.zc;
    const int z1 = min(z0 + g.zc, g.nz);
    const int nloc = z1 - z0 + 2;
    const int f = fx0 + 4 * tx;
    const int y = y0 + ty;
    const bool own = (f < g.RP) && (y < g.ny);
    const int r = ty + HR;
    const long long ro = (long long)y * g.RP + f;
    const bool y_in = !IS3D || (y >= 1 && y <= g.ny - 2);
    bool x_in[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int xq = (f + q) >> logC;
        x_in[q] = xq >= 1 && xq <= g.nx - 2;
    }
    const float cen = IS3D ? -6.f : -4.f;
    const float inv_h2 = g.inv_h2;

    const uint32_t b_halo = (uint32_t)(ROWS * SR * 4), b_sh = (uint32_t)(ROWS * SH * 4),
                   b_own = (uint32_t)(TY * TXF * 4), b_cell = (uint32_t)(TY * cells * 4);
    auto issue = [&](int i, int slot) {
        const int p = z0 - 1 + i;
        float* st = smf + (size_t)slot * L.floats;
        uint64_t* bar = bars + slot;
        const bool inner = i >= 1 && i <= nloc - 2;
        uint32_t bytes = b_halo + b_sh;
        if (inner) bytes += 2 * b_own + (has_sp ? b_cell : 0u) + (has_g ? 2 * b_cell : 0u);
        if (a.wait_test && i == 0) bytes += 16u;   // never delivered: exercises the bounded wait
        mbar_expect_tx(bar, bytes);
        if (C >= 4) tma4(st, &mp.l1, bar, 0, x0c - 1, y0 - HR, p);
        else tma3(st, &mp.l1, bar, fx0 - 4, y0 - HR, p);
        tma3(st + L.o_S, &mp.S, bar, x0c - 4, y0 - HR, p);
        if (inner) {
            if (C >= 4) {
                tma4(st + L.o_l2, &mp.l2, bar, 0, x0c, y0, p);
                tma4(st + L.o_d2, &mp.d2, bar, 0, x0c, y0, p);
            } else {
                tma3(st + L.o_l2, &mp.l2, bar, fx0, y0, p);
                tma3(st + L.o_d2, &mp.d2, bar, fx0, y0, p);
            }
            if (has_sp) tma3(st + L.o_sp, &mp.sp, bar, x0c, y0, p);
            if (has_g) tma3(st + L.o_g, &mp.g, bar, x0c, y0, p);
        }
    };

    if (aborted(err, reinterpret_cast<int*>(bars + R))) return;
    if (tid == 0) {
        for (int s = 0; s < R; ++s) mbar_init(bars + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int npro = min(R, nloc);
    if (tid == 0)
        for (int i = 0; i < npro; ++i) issue(i, i);
    int issued = npro;

    const int tile = blockIdx.x + g.ntiles_x * blockIdx.y;
    int ri = a.r_ptr[tile];
    const int re = a.r_ptr[tile + 1];
    while (ri < re && a.r_ent[ri].z < z0) ++ri;
    int rnz = ri < re ? a.r_ent[ri].z : 0x7fffffff;

    // q = S * lam^{k+1} at float lf (multiple of 4) / scalar, of a stage row
    auto qv4 = [&](const float* st, int row, int lf) -> float4 {
        const float4 l = ld4(st + row * SR + HF + lf);
        const float4 s = cell4s(st + L.o_S + row * SH + 4, lf, logC);
        return mul4(s, l);
    };
    auto qs = [&](const float* st, int row, int lf) -> float {
        return st[L.o_S + row * SH + 4 + (lf >> logC)] * st[row * SR + HF + lf];
    };

    int s_m = 0, s_c = 1, s_p = 2 % R;
    uint32_t ph_p = (R == 2) ? 1u : 0u;
    bool ok = wait_bar(bars + 0, 0u);
    ok = wait_bar(bars + 1, 0u) && ok;
    float* lk_ptr = a.lk + (long long)z0 * g.PP + ro;
    double* g_row = has_g ? a.gacc + (long long)z0 * g.CPP + (long long)y * g.nxs + x0c : nullptr;
    // C >= 4: a plane's per-lane shot sum is reduced across the cell's lanes
    // and added to the gradient one iteration later, while that plane's stage
    // is still resident (it is refilled only after the next plane's barrier),
    // so the shuffle chain and the FP64 update overlap the next plane's
    // stencil instead of holding up this plane's barrier; same arithmetic.
    float s_def = 0.f;
    double* g_def = nullptr;
    const double* gs_def = nullptr;
    auto flush = [&]() {
        float s = s_def;
        constexpr int G = C >= 4 ? C >> 2 : 1;
        for (int o = 1; o < G; o <<= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
        const int c0 = (4 * tx) >> logC;
        if (own && (tx & (G - 1)) == 0) g_def[c0] = gs_def[c0] + (double)s;
    };
    for (int z = z0; z < z1; ++z) {
        const int im = z - z0;
        ok = wait_bar(bars + s_p, ph_p) && ok;
        if (C >= 4 && has_g && im > 0) flush();
        const float* sm_m = smf + (size_t)s_m * L.floats;
        const float* sm_c = smf + (size_t)s_c * L.floats;
        const float* sm_p = smf + (size_t)s_p * L.floats;
        const int lf = 4 * tx;
        const float4 qc = qv4(sm_c, r, lf);
        float4 xm, xp;
        if (C >= 4) {
            xm = qv4(sm_c, r, lf - C);
            xp = qv4(sm_c, r, lf + C);
        } else if (C == 2) {
            xm = make_float4(qs(sm_c, r, lf - 2), qs(sm_c, r, lf - 1), qc.x, qc.y);
            xp = make_float4(qc.z, qc.w, qs(sm_c, r, lf + 4), qs(sm_c, r, lf + 5));
        } else {
            xm = make_float4(qs(sm_c, r, lf - 1), qc.x, qc.y, qc.z);
            xp = make_float4(qc.y, qc.z, qc.w, qs(sm_c, r, lf + 4));
        }
        float4 ym = f4zero(), yp = f4zero();
        if (IS3D) {
            ym = qv4(sm_c, r - 1, lf);
            yp = qv4(sm_c, r + 1, lf);
        }
        const float4 qm = qv4(sm_m, r, lf);
        const float4 qp = qv4(sm_p, r, lf);
        const float4 l1c = ld4(sm_c + r * SR + HF + lf);
        const float4 l2v = ld4(sm_c + L.o_l2 + ty * TXF + lf);
        const float4 d2v = ld4(sm_c + L.o_d2 + ty * TXF + lf);
        const float4 spv = has_sp ? cell4s(sm_c + L.o_sp + ty * cells, lf, logC) : f4zero();
        const bool zy_in = y_in && z >= 1 && z <= g.nz - 2;
        bool in[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) in[q] = zy_in && x_in[q];
        // lam^k = (2 lam^{k+1} - lam^{k+2}) + L q, with 2l - l2 as fma(2, l, -l2)
        const float4 lq = stencil4m(in, cen, qc, xm, xp, ym, yp, qm, qp, IS3D, inv_h2);
        float4 lk4 = add4(fma4(splat4(2.f), l1c, neg4(l2v)), lq);
        if (has_sp) lk4 = mul4(lk4, spv);
        float lk[4];
        put4(lk, lk4);
        if (z == rnz) {
            const InjStep st = inject_residuals(make_float4(lk[0], lk[1], lk[2], lk[3]), a.r_ent,
                                                ri, re, z, ty, tx, C, a.res);
            put4(lk, st.lk);
            ri = st.ri;
            rnz = st.rnz;
        }
        if (own) st4(lk_ptr, make_float4(lk[0], lk[1], lk[2], lk[3]));
        lk_ptr += g.PP;
        if (has_g) {
            float pr[4];
            put4(pr, own ? mul4(make_float4(lk[0], lk[1], lk[2], lk[3]), d2v) : f4zero());
            const double* gs = reinterpret_cast<const double*>(sm_c + L.o_g) + ty * cells;
            double* grow = g_row;
            g_row += g.CPP;
            if (logC == 0) {
                if (own) {
                    const int c0 = lf;
                    double2* gp = reinterpret_cast<double2*>(grow + c0);
                    gp[0] = make_double2(gs[c0] + (double)pr[0], gs[c0 + 1] + (double)pr[1]);
                    gp[1] = make_double2(gs[c0 + 2] + (double)pr[2], gs[c0 + 3] + (double)pr[3]);
                }
            } else if (logC == 1) {
                if (own) {
                    const int c0 = lf >> 1;
                    *reinterpret_cast<double2*>(grow + c0) =
                        make_double2(gs[c0] + (double)(pr[0] + pr[1]), gs[c0 + 1] + (double)(pr[2] + pr[3]));
                }
            } else {
                s_def = (pr[0] + pr[1]) + (pr[2] + pr[3]);
                g_def = grow;
                gs_def = gs;
            }
        }

        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        if (tid == 0 && im + R < nloc) {
            fence_proxy_async();
            issue(im + R, s_m);
        }
        if (im + R < nloc) issued = im + R + 1;
        s_m = s_c;
        s_c = s_p;
        if (++s_p == R) { s_p = 0; ph_p ^= 1u; }
    }
    // the last plane's update: its stage is never refilled (no plane is
    // issued after the last one's barrier)
    if (ok && C >= 4 && has_g && z1 > z0) flush();
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        for (int i = (issued > R ? issued - R : 0); i < issued; ++i) (void)wait_stage(bars, i, R);
    }
}

// ---------------------------------------------------------------------------
// launchers, one translation unit per C (usct_tma_inst.cu built with
// -DUSCT_TMA_C=C): 0 = launched, -1 = no kernel for this tile and C
// ---------------------------------------------------------------------------
struct TmaLaunch {
    dim3 grid;
    size_t smem;
    int R;
    cudaStream_t stream;
    int* err;
    int txv, ty;
    bool is3d;
};
template <int C>
int tma_forward(const TmaLaunch& t, const FwdArgs& a, const FwdMaps& mp, bool born,
                bool pcs = false);
template <int C>
int tma_adjoint(const TmaLaunch& t, const AdjArgs& a, const AdjMaps& mp);
template <int C>
void tma_allow_smem(int bytes);

// the two-step forward (usct_tma2.cuh): tile W x H cells, RA / RB ring stages
struct Fwd2Args;
struct Fwd2Maps;
struct TmaLaunch2 {
    dim3 grid;
    size_t smem;
    int RA, RB;
    cudaStream_t stream;
    int* err;
    int w, h;
};
template <int C>
int tma_forward2(const TmaLaunch2& t, const Fwd2Args& a, const Fwd2Maps& mp);


}  // namespace usct
