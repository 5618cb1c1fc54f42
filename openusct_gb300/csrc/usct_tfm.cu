// usct_tfm.cu -- total focusing method (delay-and-sum) imaging of an FMC.
//
// Restates simulation/ringfwi/imaging.py:27-74 on the device:
//   I(r) = sum_{tx i, rx j} A_{i,j}[ round((|r - p_tx(i)| + |r - p_j|) / c * fs) ]
// with A the analytic signal of each trace (scipy.signal.hilbert along time)
// and samples outside [0, nt) skipped; the envelope image is |I|.
//
// Kernels, in launch order k_real, k_analytic, k_tfm (and k_pwindow):
//  * k_analytic -- A = x + i (x (*) g): the FFT-based analytic signal written
//    as a circular convolution of each trace with the imaginary part g of the
//    inverse DFT of scipy's spectral multiplier (computed on the host, FP64,
//    handed over as FP32 taps).  FP32 multiply-adds, one lane per trace and
//    a register ring of taps, traces and taps staged in shared memory.  The
//    result is trace-major [tx][rx][n] (float2 re/im), so the gathers of
//    neighbouring pixels hit neighbouring samples of one trace.
//  * k_real -- the transpose to trace-major (real parts), each FP64 sample
//    converted once; k_analytic then fills in the imaginary parts.
//  * k_tfm -- eight threads per pixel, each summing a share of the
//    transmits: FP32 distances (receivers' kept in shared memory); the sample
//    index equals NumPy's np.round((d_tx + d_rx) / c * fs) (an FP32 product
//    decides it except near a half-integer, where the FP64 distances and
//    expression are formed in the reference's order); the complex samples of
//    one transmit are summed in FP32 over the receivers (in the reference's
//    order), the transmits in FP64.
#include <cuda_runtime.h>

#include <cstdint>

#include "usct_convert.cuh"
#include "usct_gb300.h"

int usct_internal_error(int code, const char* msg);   // usct_engine.cu

namespace {

constexpr int kAW = 8;              // warps per block
constexpr int kAB = 16;             // outputs per thread (a power of two)
constexpr int kAM = 64;             // input samples per stage
constexpr int kAN = kAW * kAB;      // outputs per block
constexpr int kAT = 64;             // traces per block: two per lane
constexpr int kAG = kAN + kAM - 1;  // taps per stage
constexpr int kAQ = kAT * kAM / (kAW * 32);   // staged samples per thread

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return USCT_OK;
    return usct_internal_error(e == cudaErrorMemoryAllocation ? USCT_ERR_NOMEM : USCT_ERR_CUDA,
                               cudaGetErrorString(e));
}

// Block (32 * kAW): lane l owns traces tb + l and tb + l + 32, warp w owns the
// outputs nb + S*b, b < kAB, where S = 2 for even nt (the taps vanish at even
// offsets, so an output only meets inputs of the other parity, and the warp
// pair (2v, 2v+1) covers 2*kAB consecutive outputs) and S = 1 for odd nt.
// Output b at input step k needs the tap G[b - k]; G[q] = T[cw + q], T the
// stage's taps g[(n0 - m0 - (kAM-1) + S*i) mod nt].  The outputs are taken in
// pairs (2j, 2j+1), so step k multiplies each trace's sample by the tap pairs
// (T[cw - k + 2j], T[cw - k + 2j + 1]), j < kAB/2, in paired multiply-adds
// (fma.rn.f32x2, two IEEE fmaf per lane).  Those pairs start at indices of one
// parity on even steps and of the other on odd steps, so shared memory holds
// the taps pre-paired in both alignments (tp[a][e] = (T[2e+a], T[2e+a+1])) and
// a thread keeps a register ring of kAB/2 pairs for each: every step loads one
// new pair, two samples and issues kAB paired multiply-adds.  The stages are
// double-buffered: the next stage's samples and taps are loaded into
// registers before this stage's multiply-adds and stored after them, one
// barrier per stage.  Every output sums its inputs in increasing m, one fmaf
// each.  The samples come from the real parts k_real wrote
// (out[2*(t*nt + m)]); only the imaginary parts are written here.
template <int S>
__global__ void __launch_bounds__(kAW * 32, 2) k_analytic(float* __restrict__ out, long long ntr,
                                                          int nt, const float* __restrict__ g) {
    constexpr int kL = (S == 1) ? kAG : (kAG + 1) / 2;   // taps T of one stage
    constexpr int kP = kL / 2 + 1;                      // pairs per alignment
    constexpr int kH = kAB / 2;                         // output pairs per thread
    __shared__ float xs[2][kAT][kAM + 1];   // odd pitch: the lanes' rows fall in distinct banks
    __shared__ float2 tp[2][2][kP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n0 = blockIdx.y * kAN;
    const int nb = (S == 1) ? n0 + kAB * w : n0 + 2 * kAB * (w >> 1) + (w & 1);
    const int par = (S == 1) ? 0 : 1 - (w & 1);   // parity of the inputs this warp meets
    const int cw = (nb - n0 - par + kAM - 1) / S;  // T index of G[0] (exact: even for S = 2)
    const long long tb = (long long)blockIdx.x * kAT;
    // staging: thread x stages sample (x & 63) of traces (x >> 6) + 4q, q < kAQ
    // (a warp reads 32 consecutive samples of one trace), and threads below
    // 2*kP the tap pair tp[x / kP][x % kP]
    const int smm = threadIdx.x & (kAM - 1), stt = threadIdx.x / kAM;
    const int pa = threadIdx.x / kP, pe = threadIdx.x % kP;
    float pf[kAQ];
    float pg0 = 0.f, pg1 = 0.f;
    auto tap = [&](int m0, int i) {
        int d = n0 - m0 - (kAM - 1) + S * i;   // |d| < nt + 2*kAN: int suffices
        d %= nt;
        if (d < 0) d += nt;
        return g[d];
    };
    auto load = [&](int m0) {
        const int m = m0 + smm;
#pragma unroll
        for (int q = 0; q < kAQ; ++q) {
            const long long t = tb + stt + (kAW * 32 / kAM) * q;
            pf[q] = (t < ntr && m < nt) ? out[2 * (t * nt + m)] : 0.f;
        }
        if (threadIdx.x < 2 * kP) {
            pg0 = tap(m0, 2 * pe + pa);
            pg1 = tap(m0, 2 * pe + pa + 1);
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int q = 0; q < kAQ; ++q) xs[buf][stt + (kAW * 32 / kAM) * q][smm] = pf[q];
        if (threadIdx.x < 2 * kP) tp[buf][pa][pe] = make_float2(pg0, pg1);
    };
    float2 A0[kH], A1[kH];   // (output 2j, output 2j+1) of each trace
#pragma unroll
    for (int j = 0; j < kH; ++j) A0[j] = A1[j] = make_float2(0.f, 0.f);
    load(0);
    store(0);
    __syncthreads();
    int buf = 0;
    for (int m0 = 0; m0 < nt; m0 += kAM) {
        const bool more = m0 + kAM < nt;
        if (more) load(m0 + kAM);
        // step k of this stage is input m0 + par + S*k.  Even steps k = 2u use
        // the pairs starting at cw - 2u + 2j (alignment cw & 1), odd steps
        // k = 2u + 1 those at cw - 2u - 1 + 2j; both index ranges lie inside
        // tp for every warp (cw - k >= 0, cw + kAB <= 2*kP)
        const float* x0 = &xs[buf][lane][par];
        const float* x1 = &xs[buf][lane + 32][par];
        const float2* pE = &tp[buf][cw & 1][cw >> 1];
        const float2* pO = &tp[buf][(cw & 1) ^ 1][(cw - 1) >> 1];
        float2 RE[kH], RO[kH];   // slot (j - u) & (kH-1) holds pair j of step 2u / 2u + 1
#pragma unroll
        for (int j = 1; j < kH; ++j) {
            RE[j] = pE[j];
            RO[j] = pO[j];
        }
        for (int k0 = 0; k0 < kAM / S; k0 += kAB) {
            const int u0 = k0 / 2;
#pragma unroll
            for (int k = 0; k < kAB; ++k) {
                const int u = k >> 1;
                const int kk = k0 + k;
                if ((k & 1) == 0)
                    RE[(kH - u) & (kH - 1)] = pE[-(u0 + u)];
                else
                    RO[(kH - u) & (kH - 1)] = pO[-(u0 + u)];
                const float xv0 = x0[S * kk], xv1 = x1[S * kk];
                const float2 X0 = make_float2(xv0, xv0), X1 = make_float2(xv1, xv1);
#pragma unroll
                for (int j = 0; j < kH; ++j) {
                    const float2 gv = (k & 1) ? RO[(j - u) & (kH - 1)] : RE[(j - u) & (kH - 1)];
                    A0[j] = __ffma2_rn(X0, gv, A0[j]);
                    A1[j] = __ffma2_rn(X1, gv, A1[j]);
                }
            }
        }
        if (more) store(buf ^ 1);   // the other buffer: every warp left it at the last barrier
        __syncthreads();
        buf ^= 1;
    }
    // the imaginary parts only: other blocks still read the real parts
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const long long t = tb + lane + 32 * h;
        if (t >= ntr) continue;
#pragma unroll
        for (int j = 0; j < kH; ++j) {
            const float2 v = h ? A1[j] : A0[j];
            const int n = nb + S * 2 * j;
            if (n < nt) out[2 * (t * nt + n) + 1] = v.x;
            if (n + S < nt) out[2 * (t * nt + n + S) + 1] = v.y;
        }
    }
}

using usct_cvt::f32_to_f64;
using usct_cvt::f64_to_f32;

// out[i][j][m] = (data[i][m][j], 0): the Dataset layout to trace-major, each
// FP64 sample converted to FP32 once.  32 x 32 tiles (m, j) through shared
// memory, so both the reads (along j) and the writes (along m) are coalesced.
__global__ void __launch_bounds__(256) k_real(const double* __restrict__ data,
                                              float2* __restrict__ out, int nt, int n_rx) {
    __shared__ float tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long long i = blockIdx.z;
    const int m0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
    for (int r = ty; r < 32; r += 8) {
        const int m = m0 + r, j = j0 + tx;
        if (m < nt && j < n_rx) tile[r][tx] = f64_to_f32(data[(i * nt + m) * n_rx + j]);
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int j = j0 + r, m = m0 + tx;
        if (j < n_rx && m < nt) out[(i * n_rx + j) * nt + m] = make_float2(tile[tx][r], 0.f);
    }
}

// |r - p_e| with the reference's order: ((dx^2 + dy^2) [+ dz^2]) then sqrt
template <int DIM>
__device__ __forceinline__ double dist(const double (&r)[3], const double* __restrict__ pos, int e) {
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
        const double d = r[a] - pos[e * DIM + a];
        s = (a == 0) ? d * d : s + d * d;
    }
    return sqrt(s);
}

// ---- float-float (FP32 pair) arithmetic: value = x + y, |y| <= ulp(x)/2 ----
// (exact error-free transformations: Knuth's two-sum, Dekker's fast two-sum,
// the fused multiply-add product error; the build contracts nothing)
__device__ __forceinline__ float2 ff_two_sum(float a, float b) {
    const float s = a + b, bb = s - a;
    return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 ff_fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
    const float s = a + b;
    return make_float2(s, b - (s - a));
}
__device__ __forceinline__ float2 ff_from(double x) {
    const float h = f64_to_f32(x);
    return make_float2(h, f64_to_f32(x - f32_to_f64(h)));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    const float2 s = ff_two_sum(a.x, b.x);
    return ff_fast_two_sum(s.x, s.y + (a.y + b.y));
}
__device__ __forceinline__ float2 ff_sq(float2 a) {
    const float p = a.x * a.x;
    float e = __fmaf_rn(a.x, a.x, -p);
    e = __fmaf_rn(2.f * a.x, a.y, e);
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ float2 ff_sqrt(float2 a) {   // one Newton step from sqrtf
    if (!(a.x > 0.f)) return make_float2(0.f, 0.f);
    const float s = sqrtf(a.x);
    const float r = __fmaf_rn(-s, s, a.x) + a.y;
    return ff_fast_two_sum(s, r / (2.f * s));
}
// |r - p| from float-float coordinates
template <int DIM>
__device__ __forceinline__ float2 ff_dist(const float2 (&r)[3], const float2* __restrict__ p) {
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
        const float2 q = ff_sq(ff_add(r[a], make_float2(-p[a].x, -p[a].y)));
        s = (a == 0) ? q : ff_add(s, q);
    }
    return ff_sqrt(s);
}

// Block (kTP * kTG): kTP pixels, kTG threads per pixel.  The threads of a
// pixel first write its receiver distances to the pixel's column of shared
// memory, then thread g of the pixel forms the sums of transmits g, g + kTG,
// ... (FP32 over the receivers, in receiver order) and parks them in shared
// memory, where the pixel's first thread adds them to the FP64 sums in
// transmit order -- the same sums, in the same order, as one thread per
// pixel, with kTG times the threads in flight.
//
// The sample index: v = (d_tx + d_rx) * (fs / c) is formed first in FP32 from
// the leading halves of the distances below (within 2.4e-7 * v of the FP64
// value: four roundings of 6e-8), which decides it unless v lies within
// 1e-6 * v + 1e-5 of a half-integer (about 0.2 % of pairs).  There it is
// formed in float-float from float-float coordinates (the element
// coordinates of the current receiver chunk and transmit window staged in
// shared memory).  That error
// against the reference's FP64 (d_tx + d_rx) / c * fs is below
// 1e-11 * v + 4e-13 * (fs / c) * |r|_1 (the second term: the coordinates'
// float-float rounding, 4 u^2 per coordinate, through |p| <= |r| + |r - p|;
// over 5e6 random pairs and geometries, arrays offset up to 1000 times their
// size included, the error stayed below 1.5 % of that bound), and frac(v) - 1/2
// is then formed with 6e-8 error.  Only where that lies within
// 1e-11 * v + 2e-7 + 4e-13 * (fs / c) * |r|_1 of zero (about 2 pairs in a
// million) are the FP64 distances and expression formed, in the reference's
// order -- so every index equals NumPy's np.round, and FP64 work (slow on
// this part, and paid by the whole warp when one lane needs it) stays rare.
constexpr int kTP = 16;    // pixels per block
constexpr int kTG = 8;     // threads per pixel
constexpr int kTW = 64;    // transmits per window of parked sums
constexpr int kTB = kTP * kTG;
constexpr int kRxChunk = 256;   // receivers whose distances are held at once
template <int DIM>
__global__ void __launch_bounds__(kTB) k_tfm(const float2* __restrict__ A, int n_tx, int n_rx,
                                             int nt, const double* __restrict__ tx_pos,
                                             const double* __restrict__ rx_pos,
                                             const double* __restrict__ axes, int npix,
                                             long long npts, int rx_chunk, double c, double fs,
                                             double* __restrict__ out_re,
                                             double* __restrict__ out_im) {
    extern __shared__ float2 drx[];              // [rx_chunk][kTP] float-float distances
    __shared__ float2 rxc[kRxChunk * DIM];       // the chunk's receiver coordinates
    __shared__ float2 txc[kTW * DIM];            // the window's transmit coordinates
    __shared__ float2 part[kTW][kTP];            // parked per-transmit sums
    const int px = threadIdx.x % kTP, grp = threadIdx.x / kTP;
    const long long p = blockIdx.x * (long long)kTP + px;
    const bool live = p < npts;
    // pixel p of the C-order (ij) grid: the last axis varies fastest
    double r[3] = {0.0, 0.0, 0.0};
    if (live) {
        long long q = p;
#pragma unroll
        for (int a = DIM - 1; a >= 0; --a) {
            r[a] = axes[a * npix + (int)(q % npix)];
            q /= npix;
        }
    }
    float2 rf[3];
    float r1 = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        rf[a] = ff_from(r[a]);
        r1 += fabsf(rf[a].x);
    }
    const float2 rate = ff_from(fs / c);
    const float mabs = 2e-7f + 4e-13f * rate.x * (1.01f * r1);
    const float ntf = (float)nt;
    const float2* col = drx + px;
    double sre = 0.0, sim = 0.0;
    for (int j0 = 0; j0 < n_rx; j0 += rx_chunk) {
        const int nj = min(rx_chunk, n_rx - j0);
        __syncthreads();   // the previous chunk's coordinates and distances are no longer read
        for (int e = threadIdx.x; e < nj * DIM; e += kTB)
            rxc[e] = ff_from(rx_pos[(long long)j0 * DIM + e]);
        __syncthreads();
        for (int jj = grp; jj < nj; jj += kTG)
            drx[jj * kTP + px] = ff_dist<DIM>(rf, rxc + jj * DIM);
        for (int i0 = 0; i0 < n_tx; i0 += kTW) {
            const int ni = min(kTW, n_tx - i0);
            for (int e = threadIdx.x; e < ni * DIM; e += kTB)
                txc[e] = ff_from(tx_pos[(long long)i0 * DIM + e]);
            __syncthreads();   // distances and transmit coordinates written
            for (int ii = grp; ii < ni; ii += kTG) {
                const int i = i0 + ii;
                float pre = 0.f, pim = 0.f;   // this transmit's sum over the receivers
                if (live) {
                    const float2 dtx = ff_dist<DIM>(rf, txc + ii * DIM);
                    const float2* slab = A + ((long long)i * n_rx + j0) * nt;
                    // eight receivers at a time: all eight indices first, then
                    // eight independent gathers in flight, then the sums in
                    // receiver order (a skipped sample adds 0, which leaves
                    // the sum unchanged)
                    for (int jb = 0; jb < nj; jb += 8) {
                        int kk[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int jj = jb + u;
                            kk[u] = -1;
                            if (jj < nj) {
                                const float2 drj = col[jj * kTP];
                                // FP32 first: within 2.4e-7 * v of the FP64 value
                                const float v32 = (dtx.x + drj.x) * rate.x;
                                float kf = rintf(v32);
                                if (fabsf((v32 - floorf(v32)) - 0.5f) <= 1e-6f * v32 + 1e-5f) {
                                    const float2 v = ff_mul(ff_add(dtx, drj), rate);
                                    const float fl = floorf(v.x);
                                    const float g = ((v.x - fl) - 0.5f) + v.y;
                                    if (fabsf(g) <= 1e-11f * v.x + mabs) {
                                        const double s = dist<DIM>(r, tx_pos, i) +
                                                         dist<DIM>(r, rx_pos, j0 + jj);
                                        kf = (float)rint((s / c) * fs);
                                    } else {
                                        kf = g > 0.f ? fl + 1.f : fl;
                                    }
                                }
                                if (kf >= 0.f && kf < ntf) kk[u] = (int)kf;
                            }
                        }
                        float2 a[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u)
                            a[u] = kk[u] >= 0 ? slab[(long long)(jb + u) * nt + kk[u]]
                                              : make_float2(0.f, 0.f);
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            pre += a[u].x;
                            pim += a[u].y;
                        }
                    }
                }
                part[ii][px] = make_float2(pre, pim);
            }
            __syncthreads();
            if (grp == 0 && live) {
                for (int ii = 0; ii < ni; ++ii) {
                    const float2 v = part[ii][px];
                    sre += f32_to_f64(v.x);
                    sim += f32_to_f64(v.y);
                }
            }
            __syncthreads();   // parked sums and transmit coordinates consumed
        }
    }
    if (grp == 0 && live) {
        out_re[p] = sre;
        out_im[p] = sim;
    }
}

// P-arrival mute windows (fwi.py:663-699): one warp per trace of the
// trace-major analytic signal; envelope |A| (FP32 hypot), its maximum, the first
// sample above onset_frac * (max + 1e-30), then the cosine roll-off in FP64,
// written to W[tx][n][rx] (the time_weights layout).
__global__ void __launch_bounds__(256) k_pwindow(const float2* __restrict__ A, int n_tx, int nt,
                                                 int n_rx, double onset_frac, double keep,
                                                 double taper, double* __restrict__ W) {
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long ntr = (long long)n_tx * n_rx;
    if (warp >= ntr) return;
    const float2* tr = A + warp * nt;
    float mx = 0.f;
    for (int n = lane; n < nt; n += 32) mx = fmaxf(mx, hypotf(tr[n].x, tr[n].y));
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const double thresh = onset_frac * ((double)mx + 1e-30);
    int onset = nt;
    for (int n0 = 0; n0 < nt && onset == nt; n0 += 32) {
        const int n = n0 + lane;
        const bool above = n < nt && (double)hypotf(tr[n].x, tr[n].y) > thresh;
        const unsigned b = __ballot_sync(0xffffffffu, above);
        if (b) onset = n0 + __ffs(b) - 1;
    }
    if (onset == nt) onset = 0;   // np.argmax of an all-false column is 0
    const long long i = warp / n_rx, j = warp % n_rx;
    const double end = (double)onset + keep;
    for (int n = lane; n < nt; n += 32) {
        double r = (end + taper - (double)n) / taper;
        r = r < 0.0 ? 0.0 : (r > 1.0 ? 1.0 : r);
        W[(i * nt + n) * n_rx + j] = 0.5 - 0.5 * cos(3.14159265358979323846 * r);
    }
}

}  // namespace

extern "C" int usct_pwindow_dev(const float* analytic, int n_tx, int nt, int n_rx,
                                double onset_frac, double keep, double taper, double* weights,
                                void* stream) {
    if (!analytic || !weights) return usct_internal_error(USCT_ERR_ARG, "null argument");
    if (n_tx < 1 || nt < 1 || n_rx < 1) return usct_internal_error(USCT_ERR_ARG, "empty data");
    if (!(taper > 0.0)) return usct_internal_error(USCT_ERR_ARG, "taper must be > 0");
    const long long threads = (long long)n_tx * n_rx * 32;
    const long long blocks = (threads + 255) / 256;
    if (blocks > 0x7fffffffLL) return usct_internal_error(USCT_ERR_ARG, "too many traces");
    k_pwindow<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float2*>(analytic), n_tx, nt, n_rx, onset_frac, keep, taper,
        weights);
    return cuda_status(cudaGetLastError());
}

extern "C" int usct_analytic_dev(const double* data, float* analytic, int n_tx, int nt, int n_rx,
                                 const float* taps, void* stream) {
    if (!data || !analytic || !taps) return usct_internal_error(USCT_ERR_ARG, "null argument");
    if (n_tx < 1 || nt < 1 || n_rx < 1) return usct_internal_error(USCT_ERR_ARG, "empty data");
    const long long ntr = (long long)n_tx * n_rx;
    if (n_tx > 65535) return usct_internal_error(USCT_ERR_ARG, "n_tx > 65535");
    if ((nt + 31) / 32 > 65535)
        return usct_internal_error(USCT_ERR_ARG, "nt too large (> 2097120 samples)");
    if ((ntr + kAT - 1) / kAT > 0x7fffffffLL)
        return usct_internal_error(USCT_ERR_ARG, "too many traces");
    cudaStream_t s = (cudaStream_t)stream;
    k_real<<<dim3((n_rx + 31) / 32, (nt + 31) / 32, n_tx), 256, 0, s>>>(
        data, reinterpret_cast<float2*>(analytic), nt, n_rx);
    const dim3 grid((unsigned)((ntr + kAT - 1) / kAT), (nt + kAN - 1) / kAN);
    if (nt % 2 == 0)
        k_analytic<2><<<grid, kAW * 32, 0, s>>>(analytic, ntr, nt, taps);
    else
        k_analytic<1><<<grid, kAW * 32, 0, s>>>(analytic, ntr, nt, taps);
    return cuda_status(cudaGetLastError());
}

extern "C" int usct_tfm_dev(const float* analytic, int n_tx, int n_rx, int nt, const double* tx_pos,
                            const double* rx_pos, int dim, const double* axes, int npix, double c,
                            double fs, double* out_re, double* out_im, void* stream) {
    if (!analytic || !tx_pos || !rx_pos || !axes || !out_re || !out_im)
        return usct_internal_error(USCT_ERR_ARG, "null argument");
    if (dim != 2 && dim != 3) return usct_internal_error(USCT_ERR_ARG, "dim must be 2 or 3");
    if (n_tx < 1 || n_rx < 1 || nt < 1 || npix < 1)
        return usct_internal_error(USCT_ERR_ARG, "empty acquisition or image");
    if (!(c > 0.0) || !(fs > 0.0)) return usct_internal_error(USCT_ERR_ARG, "c and fs must be > 0");
    long long npts = 1;
    for (int a = 0; a < dim; ++a) npts *= npix;
    // every receiver in one pass (the reference's summation order) up to
    // kRxChunk receivers; beyond that in chunks of kRxChunk
    const int rx_chunk = n_rx < kRxChunk ? n_rx : kRxChunk;
    const size_t smem = (size_t)rx_chunk * kTP * sizeof(float2);
    const long long blocks = (npts + kTP - 1) / kTP;
    if (blocks > 0x7fffffffLL) return usct_internal_error(USCT_ERR_ARG, "image too large");
    const float2* A = reinterpret_cast<const float2*>(analytic);
    cudaStream_t s = (cudaStream_t)stream;
    if (dim == 2)
        k_tfm<2><<<(unsigned)blocks, kTB, smem, s>>>(A, n_tx, n_rx, nt, tx_pos, rx_pos, axes, npix,
                                                     npts, rx_chunk, c, fs, out_re, out_im);
    else
        k_tfm<3><<<(unsigned)blocks, kTB, smem, s>>>(A, n_tx, n_rx, nt, tx_pos, rx_pos, axes, npix,
                                                     npts, rx_chunk, c, fs, out_re, out_im);
    return cuda_status(cudaGetLastError());
}
