// usct_kernels.cuh -- sm_103a kernels of the batched acoustic FWI engine.
//
// Layout.  A batch of C shots (C a power of two <= 64) shares one model.  Its
// wavefields are stored shot-innermost: level[z][y][x][c], rows padded to nxs
// cells (a multiple of 4), so a row is RP = nxs*C contiguous floats and every
// thread moves 16-byte float4s.  In 2D the grid rows play the role of z (the
// marching axis) and there is a single "y" row per plane.  Model-sized fields
// (S = dt^2/m, sponge, v/m, the FP64 gradient) use the cell layout
// [z][y][nxs] and are read once per cell for all C shots.
//
// Stencil engine ("2.5D" z-marching).  A CTA owns a tile of TXF = 4*TXV
// floats x TY rows of a plane and marches over a chunk of planes.  Each thread
// keeps its column's values at z-1, z, z+1 in registers (the register queue);
// the plane z is staged in shared memory with its x/y halo so in-plane
// neighbours come from shared memory; the next plane's loads are issued right
// after the barrier so they overlap the current plane's arithmetic.  The
// x-neighbour of a value is C floats away, so one code path serves every batch
// width.
//
// Numerics follow the reference scheme (simulation/ringfwi/fwi.py:34-81,
// 306-331, 350-379; software/core/libuap.hpp:29-224) in FP32 with a fixed op
// order (this file is compiled with -fmad=false; every fused multiply-add is an
// explicit __fmaf_rn):
//   forward  lap = fma(-2*ndim, c, t) * inv_h2 (0 on the one-cell border),
//            t = (x- + x+) [+ (y- + y+)] + (z- + z+);  lap += w*wavelet[n-1]
//            at source cells;  p^n = fma(S, lap, 2c - p^{n-2});  p^n *= sponge
//            d2p = (p^n - 2c) + p^{n-2}   (stashed for the imaging condition)
//   adjoint  q = S*lam^{k+1};  lam^k = (2 lam^{k+1} - lam^{k+2}) + L q;
//            lam^k *= sponge;  lam^k -= r_j^k * w at receiver cells (j order)
//            g[cell] += (double) sum_c lam^k_c * d2p^k_c   (fixed shot tree)
//   Born     dp^n = fma(-v/m, d2U^n, fma(S, L dp^{n-1}, 2dp^{n-1} - dp^{n-2}))
// The CPU restatement in oracle/usct_oracle.c (o32_*) uses the same order and
// reproduces these kernels bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace usct {

// Per-tile source entry: plane z, tile row ly, float offset f = lcell*C + c
// inside the tile row, weight w (applied as lap += w * wavelet[n-1]).
struct SrcEnt {
    int z, ly, f;
    float w;
};

// Per-tile receiver entry: cell (z, ly, lcell) of receiver j; slot is the
// entry's index in the receiver CSR (footprint order).
struct RxEnt {
    int z, ly, lcell, slot, j;
    float w;
    int pad0, pad1;
};

struct Geo {
    int nx, ny, nz;   // 2D: ny = 1, nz = grid rows
    int nxs;          // padded cells per row (multiple of 4)
    int C, logC;      // shot channels
    int RP;           // floats per wavefield row (nxs*C)
    long long PP;     // floats per wavefield plane (RP*ny)
    long long CPP;    // cells per model plane (nxs*ny)
    float inv_h2;
    int zc;           // planes per z-chunk
    int ntiles_x;     // tiles along the row (for the tile id)
};

struct FwdArgs {
    Geo g;
    const float* pc;    // p^{n-1}
    const float* pp;    // p^{n-2}
    float* pn;          // p^n (may alias pp)
    const float* S;
    const float* sp;    // sponge (cell layout) or null
    const float* wav;   // FP32 wavelet [nt]
    int n;              // level produced
    float* ck;          // optional copy of p^n (checkpoint)
    float* d2;          // optional d2p output (stash)
    const int* s_ptr;   // [ntiles+1] for this batch
    const SrcEnt* s_ent;
    const int* r_ptr;   // [ntiles+1]
    const RxEnt* r_ent;
    float* rs;          // receiver slot samples of level n ([nslot][C]) or null
    // Born (fused lockstep linearisation)
    const float* dc;    // dp^{n-1}
    const float* dpp;   // dp^{n-2}
    float* dn;          // dp^n (may alias dpp)
    const float* vm;    // v/m (cell layout)
    int wait_test;      // test hook: nonzero makes the first ring stage unreachable
};

struct AdjArgs {
    Geo g;
    const float* l1;    // lam^{k+1}
    const float* l2;    // lam^{k+2}
    float* lk;          // lam^k (may alias l2)
    const float* S;
    const float* sp;
    const float* d2;    // stash level d2p^k
    double* gacc;       // FP64 gradient accumulator (cell layout) or null
    const int* r_ptr;
    const RxEnt* r_ent;
    const float* res;   // adjoint source of step k: [n_rx][C]
    int wait_test;      // test hook: nonzero makes the first ring stage unreachable
};

__device__ __forceinline__ float4 f4zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }

__device__ __forceinline__ float4 ld4(const float* p) {
    return *reinterpret_cast<const float4*>(p);
}
__device__ __forceinline__ float4 ldg4(const float* p) {
    return __ldg(reinterpret_cast<const float4*>(p));
}
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// Cell-layout field expanded to the 4 floats starting at flat row offset f.
__device__ __forceinline__ float4 ld_cell4(const float* row, int f, int logC) {
    if (logC == 0) return __ldg(reinterpret_cast<const float4*>(row + f));
    if (logC == 1) {
        const float2 s = __ldg(reinterpret_cast<const float2*>(row + (f >> 1)));
        return make_float4(s.x, s.x, s.y, s.y);
    }
    const float s = __ldg(row + (f >> logC));
    return make_float4(s, s, s, s);
}

__device__ __forceinline__ float comp(const float4& v, int q) {
    return q == 0 ? v.x : (q == 1 ? v.y : (q == 2 ? v.z : v.w));
}

// In-plane x-neighbours (x-, x+) of the float4 at shared-memory column col of
// row r (c = the thread's own centre values, also stored at col).
__device__ __forceinline__ void xnb(const float* r, int col, int C, const float4& c, float4& m,
                                    float4& p) {
    if (C >= 4) {
        m = ld4(r + col - C);
        p = ld4(r + col + C);
    } else if (C == 2) {
        m = make_float4(r[col - 2], r[col - 1], c.x, c.y);
        p = make_float4(c.z, c.w, r[col + 4], r[col + 5]);
    } else {
        m = make_float4(r[col - 1], c.x, c.y, c.z);
        p = make_float4(c.y, c.z, c.w, r[col + 4]);
    }
}

// Stencil value for component q: fma(cen, c, t) * inv_h2 or 0 off the interior.
__device__ __forceinline__ float stencil(bool in, float cen, float c, float xm, float xp, float ym,
                                        float yp, float zm, float zp, bool is3d, float inv_h2) {
    float t = xm + xp;
    if (is3d) t = t + (ym + yp);
    t = t + (zm + zp);
    return in ? __fmul_rn(__fmaf_rn(cen, c, t), inv_h2) : 0.f;
}

// ---------------------------------------------------------------------------
// Forward step (optionally fused with the Born linearisation).
// ---------------------------------------------------------------------------
template <int TXV, int TY, bool IS3D, bool BORN>
__global__ void __launch_bounds__(TXV* TY) k_forward(const FwdArgs a) {
    extern __shared__ __align__(16) float sm[];
    const Geo& g = a.g;
    const int C = g.C, logC = g.logC;
    const int HF = C < 4 ? 4 : C;
    const int HV = HF >> 2;
    constexpr int TXF = 4 * TXV;
    const int SR = TXF + 2 * HF;
    const int SPL = (TY + 2) * SR;
    const int NF = BORN ? 2 : 1;
    const int tx = threadIdx.x;
    const int ty = (TY > 1) ? (int)threadIdx.y : 0;
    const int fx0 = blockIdx.x * TXF;
    const int y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * g.zc;
    const int z1 = min(z0 + g.zc, g.nz);
    const int f = fx0 + 4 * tx;
    const int y = y0 + ty;
    const bool own = (f < g.RP) && (y < g.ny);
    const int col = HF + 4 * tx;
    const long long ro = (long long)y * g.RP + f;
    const bool hl = tx < HV;
    const int fl = fx0 - HF + 4 * tx;
    const bool hl_ok = hl && fl >= 0 && y < g.ny;
    const int ir = tx - (TXV - HV);
    const bool hr = ir >= 0;
    const int fr = fx0 + TXF + 4 * ir;
    const bool hr_ok = hr && fr < g.RP && y < g.ny;
    const bool hyl = IS3D && ty == 0;
    const bool hyl_ok = hyl && y0 >= 1 && f < g.RP;
    const bool hyh = IS3D && ty == TY - 1;
    const bool hyh_ok = hyh && (y0 + TY) < g.ny && f < g.RP;
    const long long rol = (long long)y * g.RP + fl;
    const long long ror = (long long)y * g.RP + fr;
    const long long royl = (long long)(y0 - 1) * g.RP + f;
    const long long royh = (long long)(y0 + TY) * g.RP + f;
    const long long cro = (long long)y * g.nxs;   // model row offset inside a plane
    const bool y_in = !IS3D || (y >= 1 && y <= g.ny - 2);
    bool x_in[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int xq = (f + q) >> logC;
        x_in[q] = xq >= 1 && xq <= g.nx - 2;
    }
    const float cen = IS3D ? -6.f : -4.f;
    const float inv_h2 = g.inv_h2;
    const float wv = a.wav[a.n - 1];
    const bool has_sp = a.sp != nullptr;

    // per-tile entry cursors (entries sorted by z)
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

    // prologue: plane z0
    const float* pc = a.pc;
    float4 cm = (own && z0 >= 1) ? ldg4(pc + (z0 - 1) * g.PP + ro) : f4zero();
    float4 cc = own ? ldg4(pc + z0 * g.PP + ro) : f4zero();
    float4 cp = (own && z0 + 1 < g.nz) ? ldg4(pc + (z0 + 1) * g.PP + ro) : f4zero();
    float4 h_l = hl_ok ? ldg4(pc + z0 * g.PP + rol) : f4zero();
    float4 h_r = hr_ok ? ldg4(pc + z0 * g.PP + ror) : f4zero();
    float4 h_yl = hyl_ok ? ldg4(pc + z0 * g.PP + royl) : f4zero();
    float4 h_yh = hyh_ok ? ldg4(pc + z0 * g.PP + royh) : f4zero();
    float4 ppv = own ? ld4(a.pp + z0 * g.PP + ro) : f4zero();
    float4 Sv = own ? ld_cell4(a.S + z0 * g.CPP + cro, f, logC) : f4zero();
    float4 spv = (own && has_sp) ? ld_cell4(a.sp + z0 * g.CPP + cro, f, logC) : f4zero();
    // Born state
    float4 dm = f4zero(), dcc = f4zero(), dcp = f4zero(), d_l = f4zero(), d_r = f4zero(),
           d_yl = f4zero(), d_yh = f4zero(), dppv = f4zero(), vmv = f4zero();
    if (BORN) {
        const float* dc = a.dc;
        dm = (own && z0 >= 1) ? ldg4(dc + (z0 - 1) * g.PP + ro) : f4zero();
        dcc = own ? ldg4(dc + z0 * g.PP + ro) : f4zero();
        dcp = (own && z0 + 1 < g.nz) ? ldg4(dc + (z0 + 1) * g.PP + ro) : f4zero();
        d_l = hl_ok ? ldg4(dc + z0 * g.PP + rol) : f4zero();
        d_r = hr_ok ? ldg4(dc + z0 * g.PP + ror) : f4zero();
        d_yl = hyl_ok ? ldg4(dc + z0 * g.PP + royl) : f4zero();
        d_yh = hyh_ok ? ldg4(dc + z0 * g.PP + royh) : f4zero();
        dppv = own ? ld4(a.dpp + z0 * g.PP + ro) : f4zero();
        vmv = own ? ld_cell4(a.vm + z0 * g.CPP + cro, f, logC) : f4zero();
    }

    for (int z = z0; z < z1; ++z) {
        float* buf = sm + (z & 1) * (NF * SPL);
        st4(buf + (ty + 1) * SR + col, cc);
        if (hl) st4(buf + (ty + 1) * SR + 4 * tx, h_l);
        if (hr) st4(buf + (ty + 1) * SR + HF + TXF + 4 * ir, h_r);
        if (hyl) st4(buf + col, h_yl);
        if (hyh) st4(buf + (TY + 1) * SR + col, h_yh);
        if (BORN) {
            float* db = buf + SPL;
            st4(db + (ty + 1) * SR + col, dcc);
            if (hl) st4(db + (ty + 1) * SR + 4 * tx, d_l);
            if (hr) st4(db + (ty + 1) * SR + HF + TXF + 4 * ir, d_r);
            if (hyl) st4(db + col, d_yl);
            if (hyh) st4(db + (TY + 1) * SR + col, d_yh);
        }
        __syncthreads();

        // prefetch plane z+1 (consumed next iteration)
        float4 ncp = f4zero(), nh_l = f4zero(), nh_r = f4zero(), nh_yl = f4zero(),
               nh_yh = f4zero(), nppv = f4zero(), nSv = f4zero(), nspv = f4zero();
        float4 ndcp = f4zero(), nd_l = f4zero(), nd_r = f4zero(), nd_yl = f4zero(),
               nd_yh = f4zero(), ndppv = f4zero(), nvmv = f4zero();
        if (z + 1 < z1) {
            const long long zn = z + 1;
            if (own && zn + 1 < g.nz) ncp = ldg4(pc + (zn + 1) * g.PP + ro);
            if (hl_ok) nh_l = ldg4(pc + zn * g.PP + rol);
            if (hr_ok) nh_r = ldg4(pc + zn * g.PP + ror);
            if (hyl_ok) nh_yl = ldg4(pc + zn * g.PP + royl);
            if (hyh_ok) nh_yh = ldg4(pc + zn * g.PP + royh);
            if (own) {
                nppv = ld4(a.pp + zn * g.PP + ro);
                nSv = ld_cell4(a.S + zn * g.CPP + cro, f, logC);
                if (has_sp) nspv = ld_cell4(a.sp + zn * g.CPP + cro, f, logC);
            }
            if (BORN) {
                const float* dc = a.dc;
                if (own && zn + 1 < g.nz) ndcp = ldg4(dc + (zn + 1) * g.PP + ro);
                if (hl_ok) nd_l = ldg4(dc + zn * g.PP + rol);
                if (hr_ok) nd_r = ldg4(dc + zn * g.PP + ror);
                if (hyl_ok) nd_yl = ldg4(dc + zn * g.PP + royl);
                if (hyh_ok) nd_yh = ldg4(dc + zn * g.PP + royh);
                if (own) {
                    ndppv = ld4(a.dpp + zn * g.PP + ro);
                    nvmv = ld_cell4(a.vm + zn * g.CPP + cro, f, logC);
                }
            }
        }

        // Laplacian of p^{n-1}
        const float* row = buf + (ty + 1) * SR;
        float4 xm, xp;
        xnb(row, col, C, cc, xm, xp);
        float4 ym = f4zero(), yp = f4zero();
        if (IS3D) {
            ym = ld4(buf + ty * SR + col);
            yp = ld4(buf + (ty + 2) * SR + col);
        }
        const bool zy_in = y_in && z >= 1 && z <= g.nz - 2;
        float lap[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            lap[q] = stencil(zy_in && x_in[q], cen, comp(cc, q), comp(xm, q), comp(xp, q),
                             comp(ym, q), comp(yp, q), comp(cm, q), comp(cp, q), IS3D, inv_h2);

        // source injection (before the S multiply, fwi.py:65-66)
        if (z == snz) {
            while (si < se) {
                const SrcEnt e = a.s_ent[si];
                if (e.z != z) break;
                if (e.ly == ty) {
                    const int d = e.f - 4 * tx;
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (d == q) lap[q] = lap[q] + e.w * wv;
                }
                ++si;
            }
            snz = si < se ? a.s_ent[si].z : 0x7fffffff;
        }

        float pn[4], d2v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float c = comp(cc, q);
            float v = __fmaf_rn(comp(Sv, q), lap[q], 2.f * c - comp(ppv, q));
            if (has_sp) v = v * comp(spv, q);
            d2v[q] = (v - 2.f * c) + comp(ppv, q);
            pn[q] = v;
        }
        float out[4];   // the field the receivers sample
        if (BORN) {
            const float* drow = buf + SPL + (ty + 1) * SR;
            float4 dxm, dxp;
            xnb(drow, col, C, dcc, dxm, dxp);
            float4 dym = f4zero(), dyp = f4zero();
            if (IS3D) {
                dym = ld4(buf + SPL + ty * SR + col);
                dyp = ld4(buf + SPL + (ty + 2) * SR + col);
            }
            float dv[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float dl = stencil(zy_in && x_in[q], cen, comp(dcc, q), comp(dxm, q),
                                         comp(dxp, q), comp(dym, q), comp(dyp, q), comp(dm, q),
                                         comp(dcp, q), IS3D, inv_h2);
                float v = __fmaf_rn(comp(Sv, q), dl, 2.f * comp(dcc, q) - comp(dppv, q));
                v = __fmaf_rn(-comp(vmv, q), d2v[q], v);
                if (has_sp) v = v * comp(spv, q);
                dv[q] = v;
                out[q] = v;
            }
            if (own) st4(a.dn + z * g.PP + ro, make_float4(dv[0], dv[1], dv[2], dv[3]));
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) out[q] = pn[q];
        }
        if (own) {
            const float4 v = make_float4(pn[0], pn[1], pn[2], pn[3]);
            st4(a.pn + z * g.PP + ro, v);
            if (a.ck) st4(a.ck + z * g.PP + ro, v);
            if (a.d2) st4(a.d2 + z * g.PP + ro, make_float4(d2v[0], d2v[1], d2v[2], d2v[3]));
        }

        // receiver sampling of level n (fwi.py:73-79)
        if (z == rnz) {
            while (ri < re) {
                const RxEnt e = a.r_ent[ri];
                if (e.z != z) break;
                if (e.ly == ty) {
                    const int base = e.lcell * C - 4 * tx;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int c = q - base;
                        if (c >= 0 && c < C) a.rs[(long long)e.slot * C + c] = e.w * out[q];
                    }
                }
                ++ri;
            }
            rnz = ri < re ? a.r_ent[ri].z : 0x7fffffff;
        }

        cm = cc; cc = cp; cp = ncp;
        h_l = nh_l; h_r = nh_r; h_yl = nh_yl; h_yh = nh_yh;
        ppv = nppv; Sv = nSv; spv = nspv;
        if (BORN) {
            dm = dcc; dcc = dcp; dcp = ndcp;
            d_l = nd_l; d_r = nd_r; d_yl = nd_yl; d_yh = nd_yh;
            dppv = ndppv; vmv = nvmv;
        }
    }
}

// ---------------------------------------------------------------------------
// Adjoint step with fused adjoint-source injection and imaging condition.
// ---------------------------------------------------------------------------
template <int TXV, int TY, bool IS3D>
__global__ void __launch_bounds__(TXV* TY) k_adjoint(const AdjArgs a) {
    extern __shared__ __align__(16) float sm[];
    const Geo& g = a.g;
    const int C = g.C, logC = g.logC;
    const int HF = C < 4 ? 4 : C;
    const int HV = HF >> 2;
    constexpr int TXF = 4 * TXV;
    const int SR = TXF + 2 * HF;
    const int SPL = (TY + 2) * SR;
    const int tx = threadIdx.x;
    const int ty = (TY > 1) ? (int)threadIdx.y : 0;
    const int fx0 = blockIdx.x * TXF;
    const int y0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * g.zc;
    const int z1 = min(z0 + g.zc, g.nz);
    const int f = fx0 + 4 * tx;
    const int y = y0 + ty;
    const bool own = (f < g.RP) && (y < g.ny);
    const int col = HF + 4 * tx;
    const long long ro = (long long)y * g.RP + f;
    const bool hl = tx < HV;
    const int fl = fx0 - HF + 4 * tx;
    const bool hl_ok = hl && fl >= 0 && y < g.ny;
    const int ir = tx - (TXV - HV);
    const bool hr = ir >= 0;
    const int fr = fx0 + TXF + 4 * ir;
    const bool hr_ok = hr && fr < g.RP && y < g.ny;
    const bool hyl = IS3D && ty == 0;
    const bool hyl_ok = hyl && y0 >= 1 && f < g.RP;
    const bool hyh = IS3D && ty == TY - 1;
    const bool hyh_ok = hyh && (y0 + TY) < g.ny && f < g.RP;
    const long long rol = (long long)y * g.RP + fl;
    const long long ror = (long long)y * g.RP + fr;
    const long long royl = (long long)(y0 - 1) * g.RP + f;
    const long long royh = (long long)(y0 + TY) * g.RP + f;
    const long long cro = (long long)y * g.nxs;
    const long long crol = cro;
    const long long croyl = (long long)(y0 - 1) * g.nxs;
    const long long croyh = (long long)(y0 + TY) * g.nxs;
    const bool y_in = !IS3D || (y >= 1 && y <= g.ny - 2);
    bool x_in[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int xq = (f + q) >> logC;
        x_in[q] = xq >= 1 && xq <= g.nx - 2;
    }
    const float cen = IS3D ? -6.f : -4.f;
    const float inv_h2 = g.inv_h2;
    const bool has_sp = a.sp != nullptr;

    const int tile = blockIdx.x + g.ntiles_x * blockIdx.y;
    int ri = a.r_ptr[tile];
    const int re = a.r_ptr[tile + 1];
    while (ri < re && a.r_ent[ri].z < z0) ++ri;
    int rnz = ri < re ? a.r_ent[ri].z : 0x7fffffff;

    const float* l1 = a.l1;
    const float* S = a.S;
    auto qload = [&](long long zz, long long off, long long coff, int ff, bool ok) -> float4 {
        if (!ok) return f4zero();
        const float4 l = ldg4(l1 + zz * g.PP + off);
        const float4 s = ld_cell4(S + zz * g.CPP + coff, ff, logC);
        return make_float4(s.x * l.x, s.y * l.y, s.z * l.z, s.w * l.w);
    };

    float4 qm = qload(z0 - 1, ro, cro, f, own && z0 >= 1);
    float4 l1c = own ? ldg4(l1 + z0 * g.PP + ro) : f4zero();
    float4 qc = qload(z0, ro, cro, f, own);
    float4 l1p = (own && z0 + 1 < g.nz) ? ldg4(l1 + (z0 + 1) * g.PP + ro) : f4zero();
    float4 qp = qload(z0 + 1, ro, cro, f, own && z0 + 1 < g.nz);
    float4 h_l = qload(z0, rol, crol, fl, hl_ok);
    float4 h_r = qload(z0, ror, crol, fr, hr_ok);
    float4 h_yl = qload(z0, royl, croyl, f, hyl_ok);
    float4 h_yh = qload(z0, royh, croyh, f, hyh_ok);
    float4 l2v = own ? ld4(a.l2 + z0 * g.PP + ro) : f4zero();
    float4 d2v = own ? ldg4(a.d2 + z0 * g.PP + ro) : f4zero();
    float4 spv = (own && has_sp) ? ld_cell4(a.sp + z0 * g.CPP + cro, f, logC) : f4zero();

    for (int z = z0; z < z1; ++z) {
        float* buf = sm + (z & 1) * SPL;
        st4(buf + (ty + 1) * SR + col, qc);
        if (hl) st4(buf + (ty + 1) * SR + 4 * tx, h_l);
        if (hr) st4(buf + (ty + 1) * SR + HF + TXF + 4 * ir, h_r);
        if (hyl) st4(buf + col, h_yl);
        if (hyh) st4(buf + (TY + 1) * SR + col, h_yh);
        __syncthreads();

        float4 nl1p = f4zero(), nqp = f4zero(), nh_l = f4zero(), nh_r = f4zero(),
               nh_yl = f4zero(), nh_yh = f4zero(), nl2v = f4zero(), nd2v = f4zero(),
               nspv = f4zero();
        if (z + 1 < z1) {
            const long long zn = z + 1;
            const bool okp = own && zn + 1 < g.nz;
            if (okp) nl1p = ldg4(l1 + (zn + 1) * g.PP + ro);
            nqp = okp ? [&] {
                const float4 s = ld_cell4(S + (zn + 1) * g.CPP + cro, f, logC);
                return make_float4(s.x * nl1p.x, s.y * nl1p.y, s.z * nl1p.z, s.w * nl1p.w);
            }() : f4zero();
            nh_l = qload(zn, rol, crol, fl, hl_ok);
            nh_r = qload(zn, ror, crol, fr, hr_ok);
            nh_yl = qload(zn, royl, croyl, f, hyl_ok);
            nh_yh = qload(zn, royh, croyh, f, hyh_ok);
            if (own) {
                nl2v = ld4(a.l2 + zn * g.PP + ro);
                nd2v = ldg4(a.d2 + zn * g.PP + ro);
                if (has_sp) nspv = ld_cell4(a.sp + zn * g.CPP + cro, f, logC);
            }
        }

        const float* row = buf + (ty + 1) * SR;
        float4 xm, xp;
        xnb(row, col, C, qc, xm, xp);
        float4 ym = f4zero(), yp = f4zero();
        if (IS3D) {
            ym = ld4(buf + ty * SR + col);
            yp = ld4(buf + (ty + 2) * SR + col);
        }
        const bool zy_in = y_in && z >= 1 && z <= g.nz - 2;
        float lk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float lq = stencil(zy_in && x_in[q], cen, comp(qc, q), comp(xm, q), comp(xp, q),
                                     comp(ym, q), comp(yp, q), comp(qm, q), comp(qp, q), IS3D,
                                     inv_h2);
            float v = (2.f * comp(l1c, q) - comp(l2v, q)) + lq;
            if (has_sp) v = v * comp(spv, q);
            lk[q] = v;
        }
        // adjoint source: lam^k -= r_j^k * w at receiver cells (fwi.py:316-322)
        if (z == rnz) {
            while (ri < re) {
                const RxEnt e = a.r_ent[ri];
                if (e.z != z) break;
                if (e.ly == ty) {
                    const int base = e.lcell * C - 4 * tx;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int c = q - base;
                        if (c >= 0 && c < C) lk[q] = lk[q] - a.res[(long long)e.j * C + c] * e.w;
                    }
                }
                ++ri;
            }
            rnz = ri < re ? a.r_ent[ri].z : 0x7fffffff;
        }
        if (own) st4(a.lk + z * g.PP + ro, make_float4(lk[0], lk[1], lk[2], lk[3]));

        // imaging condition g += sum_c lam^k_c * d2p^k_c (fwi.py:324-326)
        if (a.gacc) {
            float pr[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) pr[q] = own ? lk[q] * comp(d2v, q) : 0.f;
            double* grow = a.gacc + z * g.CPP + cro;
            if (logC == 0) {
                if (own) {
                    double2* gp = reinterpret_cast<double2*>(grow + f);
                    double2 a0 = gp[0], a1 = gp[1];
                    a0.x += (double)pr[0]; a0.y += (double)pr[1];
                    a1.x += (double)pr[2]; a1.y += (double)pr[3];
                    gp[0] = a0; gp[1] = a1;
                }
            } else if (logC == 1) {
                if (own) {
                    double2* gp = reinterpret_cast<double2*>(grow + (f >> 1));
                    double2 a0 = gp[0];
                    a0.x += (double)(pr[0] + pr[1]);
                    a0.y += (double)(pr[2] + pr[3]);
                    gp[0] = a0;
                }
            } else {
                float s = (pr[0] + pr[1]) + (pr[2] + pr[3]);
                const int G = C >> 2;   // lanes holding one cell's channels
                for (int o = 1; o < G; o <<= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
                if (own && (tx & (G - 1)) == 0) grow[f >> logC] += (double)s;
            }
        }

        qm = qc; qc = qp; qp = nqp;
        l1c = l1p; l1p = nl1p;
        h_l = nh_l; h_r = nh_r; h_yl = nh_yl; h_yh = nh_yh;
        l2v = nl2v; d2v = nd2v; spv = nspv;
    }
}

}  // namespace usct
