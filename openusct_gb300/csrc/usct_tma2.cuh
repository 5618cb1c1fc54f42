// usct_tma2.cuh -- two time levels per launch (temporal blocking) for the 3D
// forward stencil.
//
// One launch advances every shot of a batch from (p^{n-2}, p^{n-1}) to
// (p^n, p^{n+1}).  A CTA owns W x H cells of a plane (all C shot channels) and
// marches over a z-chunk.  For each plane z it first computes p^n on its tile
// grown by one cell and one row on every side -- the halo the second step
// needs -- from a tile of p^{n-1} grown by two, then p^{n+1} on its own cells
// of plane z-1 from the three p^n planes it keeps in shared memory.  p^{n-1}
// and p^{n-2} are each read once (their halos are shared with the
// neighbouring CTAs through L2) and both new levels are written once:
// 16 C + 4 bytes of DRAM traffic per cell for two steps instead of
// 2 (12 C + 4).  The price is the first step's extra work on the grown tile,
// (W+2)(H+2)/(W H) of it.
//
// Arithmetic and op order are those of k_forward_tma (the stencil sum, the
// source injection, p = fma(S, lap, fma(2, c, -p^{n-2})), the sponge product,
// d2p = fma(-2, c, p) + p^{n-2}), so both levels are bit-identical to two
// single-step launches; cells of the grown tile outside the grid read zeros
// from the tensor copies and stay 0.
//
// Pipelining as in k_forward_tma: one elected thread issues the tensor copies
// of plane z+RA-3 of p^{n-1} (ring of RA stages) and of plane z+RB-2 of
// p^{n-2}, S and the sponge (ring of RB stages) while all warps compute; every
// stage wait is bounded and a timeout sets *err, drains the CTA's copies and
// returns.
#pragma once

#include "usct_tma.cuh"

namespace usct {

struct Fwd2Args {
    Geo g;              // with the two-step tiling's ntiles_x and zc
    const float* pc;    // p^{n-1}
    const float* pp;    // p^{n-2}
    float* pn1;         // p^n      (neither pc nor pp: both are read with halos)
    float* pn2;         // p^{n+1}  (likewise)
    const float* S;
    const float* sp;    // sponge (cell layout) or null
    const float* wav;   // FP32 wavelet [nt]
    int n;              // first level produced (n + 1 <= nt - 1)
    float* ck1;         // optional copy of p^n
    float* ck2;         // optional copy of p^{n+1}
    float* d21;         // optional d2p of level n
    float* d22;         // optional d2p of level n + 1
    const int* s_ptr;   // [ntiles+1]: source entries of each tile grown by one cell/row
    const SrcEnt* s_ent;
    const int* r_ptr;   // [ntiles+1]: receiver entries of each tile
    const RxEnt* r_ent;
    float* rs1;         // receiver slot samples of level n ([nslot][C]) or null
    float* rs2;         // the same for level n + 1
    int wait_test;      // test hook: nonzero makes the first ring stage unreachable
};

struct Fwd2Maps {
    CUtensorMap A, B, S, sp;
};

// Shared-memory layout in floats (host: sizing; device: carving).
struct Fwd2Layout {
    int a_stage, b_tile, s_tile, b_stage, p1_plane, floats;
};
__host__ __device__ inline Fwd2Layout fwd2_layout(int W, int H, int C, bool has_sp, int RA, int RB) {
    Fwd2Layout L{};
    L.a_stage = al32((H + 4) * (W + 4) * C);
    L.b_tile = al32((H + 2) * (W + 2) * C);
    L.s_tile = al32((H + 2) * (W + 8));
    L.b_stage = L.b_tile + L.s_tile * (has_sp ? 2 : 1);
    L.p1_plane = L.b_tile;
    L.floats = RA * L.a_stage + RB * L.b_stage + 3 * L.p1_plane;
    return L;
}

// first entry at or above plane z0 of a z-sorted per-tile list
template <class Ent>
__device__ __forceinline__ int first_at(const Ent* __restrict__ ent, int i, int e, int z0) {
    while (i < e && ent[i].z < z0) ++i;
    return i;
}

template <int W, int H, int C, int NT>
__global__ void __launch_bounds__(NT, 1)
    k_forward2_tma(const Fwd2Args a, const __grid_constant__ Fwd2Maps mp, const int RA,
                   const int RB, int* err) {
    static_assert(C >= 4 && W % 4 == 0, "whole cells per float4, 16-byte aligned S boxes");
    extern __shared__ __align__(128) float smf[];
    constexpr int logC = ilog2c(C);
    constexpr int AW = (W + 4) * C;         // floats per row of the p^{n-1} tile (two-cell halo)
    constexpr int BW = (W + 2) * C;         // floats per row of the grown tile
    constexpr int BH = H + 2;
    constexpr int SW = W + 8;               // cells per row of the S / sponge tile (16-byte aligned)
    constexpr int F1 = BW / 4, I1 = BH * F1;
    constexpr int F2 = W * C / 4, I2 = H * F2;
    constexpr int N1 = (I1 + NT - 1) / NT, N2 = (I2 + NT - 1) / NT;
    const bool has_sp = a.sp != nullptr;
    const Fwd2Layout L = fwd2_layout(W, H, C, has_sp, RA, RB);
    float* sA = smf;
    float* sB = smf + (size_t)RA * L.a_stage;
    float* sP = sB + (size_t)RB * L.b_stage;
    uint64_t* barA = reinterpret_cast<uint64_t*>(sP + 3 * L.p1_plane);
    uint64_t* barB = barA + RA;
    int* s_abort = reinterpret_cast<int*>(barB + RB);

    const Geo& g = a.g;
    const int tid = threadIdx.x;
    const int x0c = blockIdx.x * W, y0 = blockIdx.y * H;
    const int z0 = blockIdx.z * g.zc;
    const int z1 = min(z0 + g.zc, g.nz);
    const int nB = z1 - z0 + 2;   // planes z0-1 .. z1 of p^{n-2}, S, sponge (and of the first step)
    const int nA = nB + 2;        // planes z0-2 .. z1+1 of p^{n-1}
    const float inv_h2 = g.inv_h2;
    const float wv1 = a.wav[a.n - 1], wv2 = a.wav[a.n];

    const uint32_t bytesA = (uint32_t)((H + 4) * AW * 4);
    const uint32_t bytesB = (uint32_t)(BH * BW * 4 + BH * SW * 4 * (has_sp ? 2 : 1));
    auto issueA = [&](int i, int slot) {   // plane z0-2+i of p^{n-1}
        uint64_t* bar = barA + slot;
        mbar_expect_tx(bar, bytesA + ((a.wait_test && i == 0) ? 16u : 0u));
        tma4(sA + (size_t)slot * L.a_stage, &mp.A, bar, 0, x0c - 2, y0 - 2, z0 - 2 + i);
    };
    auto issueB = [&](int i, int slot) {   // plane z0-1+i of p^{n-2}, S and the sponge
        uint64_t* bar = barB + slot;
        float* st = sB + (size_t)slot * L.b_stage;
        mbar_expect_tx(bar, bytesB);
        tma4(st, &mp.B, bar, 0, x0c - 1, y0 - 1, z0 - 1 + i);
        tma3(st + L.b_tile, &mp.S, bar, x0c - 4, y0 - 1, z0 - 1 + i);
        if (has_sp) tma3(st + L.b_tile + L.s_tile, &mp.sp, bar, x0c - 4, y0 - 1, z0 - 1 + i);
    };

    if (aborted(err, s_abort)) return;
    if (tid == 0) {
        for (int s = 0; s < RA; ++s) mbar_init(barA + s, 1);
        for (int s = 0; s < RB; ++s) mbar_init(barB + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const int proA = min(RA, nA), proB = min(RB, nB);
    if (tid == 0) {
        for (int i = 0; i < proA; ++i) issueA(i, i);
        for (int i = 0; i < proB; ++i) issueB(i, i);
    }
    int issuedA = proA, issuedB = proB;

    // entry cursors: sources of the first step from plane z0-1, of the second
    // from z0; receivers of both levels from z0
    const int tile = blockIdx.x + g.ntiles_x * blockIdx.y;
    const int se = a.s_ptr[tile + 1];
    int si1 = first_at(a.s_ent, a.s_ptr[tile], se, z0 - 1);
    int si2 = first_at(a.s_ent, si1, se, z0);
    int snz1 = si1 < se ? a.s_ent[si1].z : 0x7fffffff;
    int snz2 = si2 < se ? a.s_ent[si2].z : 0x7fffffff;
    int ri1 = 0, re = 0;
    if (a.rs1) {
        re = a.r_ptr[tile + 1];
        ri1 = first_at(a.r_ent, a.r_ptr[tile], re, z0);
    }
    int ri2 = ri1;
    int rnz1 = ri1 < re ? a.r_ent[ri1].z : 0x7fffffff;
    int rnz2 = rnz1;

    // ring positions (incremental, no divisions): A slots of planes z-1, z, z+1;
    // the next A / B stage to wait for and its phase parity
    int sAm = 0, sAc = 1 % RA, sAp = 2 % RA;
    int wA = 0, wB = 0;
    uint32_t phA = 0u, phB = 0u;
    auto waitA = [&]() {
        const bool r = wait_bar(barA + wA, phA);
        if (++wA == RA) { wA = 0; phA ^= 1u; }
        return r;
    };
    auto waitB = [&]() {
        const bool r = wait_bar(barB + wB, phB);
        if (++wB == RB) { wB = 0; phB ^= 1u; }
        return r;
    };
    int sBc = 0, sBm = RB - 1;   // B slots of planes z and z-1
    int pc3 = 0;                 // p^n plane slot of plane z (z-1: pc3+2, z-2: pc3+1, mod 3)
    bool ok = waitA();
    ok = waitA() && ok;

    for (int i = 0; i < nB; ++i) {
        const int z = z0 - 1 + i;
        ok = waitA() && ok;   // plane z+1 of p^{n-1}
        ok = waitB() && ok;   // plane z of p^{n-2}, S, sponge
        // ---- first step: p^n on the grown tile of plane z ----
        {
            const float* Am = sA + (size_t)sAm * L.a_stage;
            const float* Ac = sA + (size_t)sAc * L.a_stage;
            const float* Ap = sA + (size_t)sAp * L.a_stage;
            const float* Bc = sB + (size_t)sBc * L.b_stage;
            const float* Sc = Bc + L.b_tile;
            const float* SPc = Sc + L.s_tile;
            float* P1 = sP + (size_t)pc3 * L.p1_plane;
            const bool zin = z >= 1 && z <= g.nz - 2;
            const bool zown = z >= z0 && z < z1;
            const bool src = z == snz1, rec = zown && z == rnz1;
#pragma unroll
            for (int u = 0; u < N1; ++u) {
                const int it = tid + u * NT;
                if (N1 * NT == I1 || it < I1) {
                    const int r = it / F1;
                    const int fo = 4 * (it - r * F1);
                    const int ci = fo >> logC;
                    const int ao = (r + 1) * AW + C + fo;
                    const float4 cc = ld4(Ac + ao);
                    const float4 xm = ld4(Ac + ao - C), xp = ld4(Ac + ao + C);
                    const float4 ym = ld4(Ac + ao - AW), yp = ld4(Ac + ao + AW);
                    const float4 zm = ld4(Am + ao), zp = ld4(Ap + ao);
                    const float4 ppv = ld4(Bc + r * BW + fo);
                    const float Sv = Sc[r * SW + ci + 3];
                    const int x = x0c - 1 + ci, y = y0 - 1 + r;
                    const bool in = zin && x >= 1 && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2;
                    float4 t = add4(add4(xm, xp), add4(ym, yp));
                    t = add4(t, add4(zm, zp));
                    float4 lap = mul4(fma4(splat4(-6.f), cc, t), splat4(inv_h2));
                    if (!in) lap = f4zero();
                    if (__builtin_expect(src, 0))
                        lap = add_sources(lap, a.s_ent, si1, se, z, r, fo >> 2, wv1).lap;
                    float4 v = fma4(splat4(Sv), lap, fma4(splat4(2.f), cc, neg4(ppv)));
                    if (has_sp) v = mul4(v, splat4(SPc[r * SW + ci + 3]));
                    st4(P1 + r * BW + fo, v);
                    if (zown && r >= 1 && r <= H && ci >= 1 && ci <= W) {
                        const int yo = y, xo = x;
                        if (yo < g.ny && xo < g.nxs) {
                            const long long go = (long long)z * g.PP + (long long)yo * g.RP +
                                                 (long long)xo * C + (fo & (C - 1));
                            st4(a.pn1 + go, v);
                            if (a.ck1) st4(a.ck1 + go, v);
                            if (a.d21) st4(a.d21 + go, add4(fma4(splat4(-2.f), cc, v), ppv));
                        }
                        if (__builtin_expect(rec, 0))
                            (void)record_receivers(v, a.r_ent, ri1, re, z, r - 1, (fo - C) >> 2, C,
                                                   a.rs1);
                    }
                }
            }
            if (src) {
                while (si1 < se && a.s_ent[si1].z == z) ++si1;
                snz1 = si1 < se ? a.s_ent[si1].z : 0x7fffffff;
            }
            if (rec) {
                while (ri1 < re && a.r_ent[ri1].z == z) ++ri1;
                rnz1 = ri1 < re ? a.r_ent[ri1].z : 0x7fffffff;
            }
        }
        __syncthreads();   // p^n of plane z is complete
        // ---- second step: p^{n+1} on the own cells of plane zz = z-1 ----
        if (i >= 2) {
            const int zz = z - 1;
            const float* Pm = sP + (size_t)(pc3 == 2 ? 0 : pc3 + 1) * L.p1_plane;   // plane zz-1
            const float* Pc = sP + (size_t)(pc3 == 0 ? 2 : pc3 - 1) * L.p1_plane;   // plane zz
            const float* Pp = sP + (size_t)pc3 * L.p1_plane;                        // plane zz+1
            const float* Aw = sA + (size_t)sAm * L.a_stage;                          // p^{n-1}, plane zz
            const float* Sm = sB + (size_t)sBm * L.b_stage + L.b_tile;
            const float* SPm = Sm + L.s_tile;
            const bool zin = zz >= 1 && zz <= g.nz - 2;
            const bool src = zz == snz2, rec = zz == rnz2;
#pragma unroll
            for (int u = 0; u < N2; ++u) {
                const int it = tid + u * NT;
                if (N2 * NT == I2 || it < I2) {
                    const int r = it / F2;
                    const int fo = 4 * (it - r * F2);
                    const int ci = fo >> logC;
                    const int po = (r + 1) * BW + C + fo;
                    const float4 cc = ld4(Pc + po);
                    const float4 xm = ld4(Pc + po - C), xp = ld4(Pc + po + C);
                    const float4 ym = ld4(Pc + po - BW), yp = ld4(Pc + po + BW);
                    const float4 zm = ld4(Pm + po), zp = ld4(Pp + po);
                    const float4 pw = ld4(Aw + (r + 2) * AW + 2 * C + fo);
                    const float Sv = Sm[(r + 1) * SW + ci + 4];
                    const int x = x0c + ci, y = y0 + r;
                    const bool in = zin && x >= 1 && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2;
                    float4 t = add4(add4(xm, xp), add4(ym, yp));
                    t = add4(t, add4(zm, zp));
                    float4 lap = mul4(fma4(splat4(-6.f), cc, t), splat4(inv_h2));
                    if (!in) lap = f4zero();
                    if (__builtin_expect(src, 0))
                        lap = add_sources(lap, a.s_ent, si2, se, zz, r + 1, (fo + C) >> 2, wv2).lap;
                    float4 v = fma4(splat4(Sv), lap, fma4(splat4(2.f), cc, neg4(pw)));
                    if (has_sp) v = mul4(v, splat4(SPm[(r + 1) * SW + ci + 4]));
                    if (y < g.ny && x < g.nxs) {
                        const long long go = (long long)zz * g.PP + (long long)y * g.RP +
                                             (long long)x * C + (fo & (C - 1));
                        st4(a.pn2 + go, v);
                        if (a.ck2) st4(a.ck2 + go, v);
                        if (a.d22) st4(a.d22 + go, add4(fma4(splat4(-2.f), cc, v), pw));
                    }
                    if (__builtin_expect(rec, 0))
                        (void)record_receivers(v, a.r_ent, ri2, re, zz, r, fo >> 2, C, a.rs2);
                }
            }
            if (src) {
                while (si2 < se && a.s_ent[si2].z == zz) ++si2;
                snz2 = si2 < se ? a.s_ent[si2].z : 0x7fffffff;
            }
            if (rec) {
                while (ri2 < re && a.r_ent[ri2].z == zz) ++ri2;
                rnz2 = ri2 < re ? a.r_ent[ri2].z : 0x7fffffff;
            }
        }
        // everyone is done with plane z-1 of p^{n-1} and of S: refill both stages
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        if (tid == 0) {
            fence_proxy_async();
            if (i + RA < nA) issueA(i + RA, sAm);
            if (i >= 1 && i - 1 + RB < nB) issueB(i - 1 + RB, sBm);
        }
        if (i + RA < nA) issuedA = i + RA + 1;
        if (i >= 1 && i - 1 + RB < nB) issuedB = i - 1 + RB + 1;
        sAm = sAc;
        sAc = sAp;
        if (++sAp == RA) sAp = 0;
        sBm = sBc;
        if (++sBc == RB) sBc = 0;
        if (++pc3 == 3) pc3 = 0;
    }
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // drain what was issued so no copy lands in a retired CTA's memory
        for (int i = (issuedA > RA ? issuedA - RA : 0); i < issuedA; ++i)
            (void)wait_stage(barA, i, RA);
        for (int i = (issuedB > RB ? issuedB - RB : 0); i < issuedB; ++i)
            (void)wait_stage(barB, i, RB);
    }
}

}  // namespace usct
