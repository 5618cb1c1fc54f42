// usct_tfm.cu -- total focusing method (delay-and-sum) imaging of an FMC.
//
// Restates simulation/ringfwi/imaging.py:27-74 on the device:
//   I(r) = sum_{tx i, rx j} A_{i,j}[ round((|r - p_tx(i)| + |r - p_j|) / c * fs) ]
// with A the analytic signal of each trace (scipy.signal.hilbert along time)
// and samples outside [0, nt) skipped; the envelope image is |I|.
//
// Two kernels:
//  * k_analytic -- A = x + i (x (*) g): the FFT-based analytic signal written
//    as a circular convolution of each trace with the imaginary part g of the
//    inverse DFT of scipy's spectral multiplier (computed on the host, FP64,
//    handed over as FP32 taps).  FP32 multiply-adds, one block per 16 traces x
//    256 samples, traces and taps staged in shared memory.  It also transposes
//    the data from the Dataset layout [tx][n][rx] (FP64) to trace-major
//    [tx][rx][n] (float2 re/im), so the gathers of neighbouring pixels hit
//    neighbouring samples of one trace.
//  * k_tfm -- one thread per pixel: distances in FP64 with the reference's
//    operation order, kept as FP32 per receiver in shared memory; the sample
//    index equals NumPy's np.round((d_tx + d_rx) / c * fs) (an FP32 product
//    decides it except near a half-integer, where the FP64 expression is
//    formed); the complex samples of one transmit are summed in FP32 over
//    the receivers (in the reference's order), the transmits in FP64.
#include <cuda_runtime.h>

#include <cstdint>

#include "usct_gb300.h"

int usct_internal_error(int code, const char* msg);   // usct_engine.cu

namespace {

constexpr int kHT = 16;     // traces per block
constexpr int kHN = 256;    // output samples per block
constexpr int kHM = 64;     // input samples per stage

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return USCT_OK;
    return usct_internal_error(e == cudaErrorMemoryAllocation ? USCT_ERR_NOMEM : USCT_ERR_CUDA,
                               cudaGetErrorString(e));
}

// block (64, 4): thread (tx, ty) accumulates traces 4*ty..4*ty+3 of the block
// at output samples n0 + tx + 64*b, b = 0..3 (a variant with 8 traces per
// thread and paired multiply-adds measured 11 % slower).  For even nt the taps
// are zero at even offsets (the host passes exact zeros there) and are skipped.
__global__ void __launch_bounds__(256) k_analytic(const double* __restrict__ data,
                                                  float2* __restrict__ out, int n_tx, int nt,
                                                  int n_rx, const float* __restrict__ g) {
    __shared__ float xs[kHT][kHM + 1];
    __shared__ float gs[kHN + kHM];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + 64 * ty;
    const long long ntr = (long long)n_tx * n_rx;
    const long long t0 = (long long)blockIdx.y * kHT;
    const int n0 = blockIdx.x * kHN;
    float acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
    for (int m0 = 0; m0 < nt; m0 += kHM) {
        // traces t0..t0+15, samples m0..m0+63 (trace t = i*n_rx + j reads data[i][m][j])
        for (int e = tid; e < kHT * kHM; e += 256) {
            const int tt = e / kHM, mm = e % kHM;
            const long long t = t0 + tt;
            const int m = m0 + mm;
            float v = 0.f;
            if (t < ntr && m < nt) {
                const long long i = t / n_rx, j = t % n_rx;
                v = (float)data[(i * nt + m) * n_rx + j];
            }
            xs[tt][mm] = v;
        }
        // taps g[(n - m) mod nt] for n - m in [n0 - m0 - 63, n0 - m0 + 255]
        for (int e = tid; e < kHN + kHM; e += 256) {
            long long d = (long long)n0 - m0 - (kHM - 1) + e;
            d %= nt;
            if (d < 0) d += nt;
            gs[e] = g[d];
        }
        __syncthreads();
        const int mlim = min(kHM, nt - m0);
        // for even nt the taps vanish at even offsets: a thread's outputs all
        // have the parity of tx (n0, m0 and 64*b are even), so only inputs of
        // the other parity contribute
        const int mstart = (nt & 1) ? 0 : ((tx + 1) & 1);
        const int mstep = (nt & 1) ? 1 : 2;
        for (int mm = mstart; mm < mlim; mm += mstep) {
            float xv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) xv[a] = xs[4 * ty + a][mm];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const float gv = gs[tx + 64 * b - mm + (kHM - 1)];
#pragma unroll
                for (int a = 0; a < 4; ++a) acc[a][b] = __fmaf_rn(xv[a], gv, acc[a][b]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const long long t = t0 + 4 * ty + a;
        if (t >= ntr) continue;
        const long long i = t / n_rx, j = t % n_rx;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int n = n0 + tx + 64 * b;
            if (n < nt)
                out[t * nt + n] = make_float2((float)data[(i * nt + n) * n_rx + j], acc[a][b]);
        }
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

// One thread per pixel, 128 pixels per block.  Each thread first writes its
// pixel's receiver distances (FP32) to its own column of shared memory, then
// for every transmit adds the samples of all receivers (FP32 within a
// transmit, FP64 across transmits).  The index is decided
// in FP32, (d_tx + d_rx) * (fs / c), whose error against the reference's FP64
// round((d_tx + d_rx) / c * fs) is below 1e-6 * v + 1e-5 samples; only when the
// FP32 value lies within that margin of a half-integer is the FP64 expression
// formed, in the reference's order -- so every index equals NumPy's.
constexpr int kTB = 128;
template <int DIM>
__global__ void __launch_bounds__(kTB) k_tfm(const float2* __restrict__ A, int n_tx, int n_rx,
                                             int nt, const double* __restrict__ tx_pos,
                                             const double* __restrict__ rx_pos,
                                             const double* __restrict__ axes, int npix,
                                             long long npts, int rx_chunk, double c, double fs,
                                             double* __restrict__ out_re,
                                             double* __restrict__ out_im) {
    extern __shared__ float drx[];   // [rx_chunk][kTB]
    const long long p = blockIdx.x * (long long)kTB + threadIdx.x;
    if (p >= npts) return;
    // pixel p of the C-order (ij) grid: the last axis varies fastest
    double r[3] = {0.0, 0.0, 0.0};
    long long q = p;
#pragma unroll
    for (int a = DIM - 1; a >= 0; --a) {
        r[a] = axes[a * npix + (int)(q % npix)];
        q /= npix;
    }
    const float rate = (float)(fs / c);
    const float ntf = (float)nt;
    float* col = drx + threadIdx.x;
    double sre = 0.0, sim = 0.0;
    for (int j0 = 0; j0 < n_rx; j0 += rx_chunk) {
        const int nj = min(rx_chunk, n_rx - j0);
        for (int jj = 0; jj < nj; ++jj) col[jj * kTB] = (float)dist<DIM>(r, rx_pos, j0 + jj);
        for (int i = 0; i < n_tx; ++i) {
            const double dtx = dist<DIM>(r, tx_pos, i);
            const float dtx32 = (float)dtx;
            const float2* slab = A + ((long long)i * n_rx + j0) * nt;
            float pre = 0.f, pim = 0.f;   // this transmit's sum over the receivers
            // eight receivers at a time: all eight indices first, then eight
            // independent gathers in flight, then the sums in receiver order
            // (a skipped sample adds 0, which leaves the sum unchanged)
            for (int jb = 0; jb < nj; jb += 8) {
                int kk[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int jj = jb + u;
                    kk[u] = -1;
                    if (jj < nj) {
                        const float v = (dtx32 + col[jj * kTB]) * rate;
                        const float fr = v - floorf(v);
                        float kf;
                        if (fabsf(fr - 0.5f) <= 1e-6f * v + 1e-5f) {
                            const double s = dtx + dist<DIM>(r, rx_pos, j0 + jj);
                            kf = (float)rint((s / c) * fs);
                        } else {
                            kf = rintf(v);
                        }
                        if (kf >= 0.f && kf < ntf) kk[u] = (int)kf;
                    }
                }
                float2 a[8];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    a[u] = kk[u] >= 0 ? slab[(long long)(jb + u) * nt + kk[u]] : make_float2(0.f, 0.f);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    pre += a[u].x;
                    pim += a[u].y;
                }
            }
            sre += (double)pre;
            sim += (double)pim;
        }
    }
    out_re[p] = sre;
    out_im[p] = sim;
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
    if ((ntr + kHT - 1) / kHT > 65535)
        return usct_internal_error(USCT_ERR_ARG, "too many traces (n_tx * n_rx > 1048560)");
    const dim3 grid((nt + kHN - 1) / kHN, (unsigned)((ntr + kHT - 1) / kHT));
    k_analytic<<<grid, dim3(64, 4), 0, (cudaStream_t)stream>>>(
        data, reinterpret_cast<float2*>(analytic), n_tx, nt, n_rx, taps);
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
    // every receiver in one pass (the reference's summation order) up to 320
    // receivers; beyond that in chunks of 320
    const int rx_chunk = n_rx < 320 ? n_rx : 320;
    const size_t smem = (size_t)rx_chunk * kTB * sizeof(float);
    const long long blocks = (npts + kTB - 1) / kTB;
    if (blocks > 0x7fffffffLL) return usct_internal_error(USCT_ERR_ARG, "image too large");
    const float2* A = reinterpret_cast<const float2*>(analytic);
    cudaStream_t s = (cudaStream_t)stream;
    if (dim == 2) {
        cudaFuncSetAttribute(k_tfm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 320 * kTB * 4);
        k_tfm<2><<<(unsigned)blocks, kTB, smem, s>>>(A, n_tx, n_rx, nt, tx_pos, rx_pos, axes, npix,
                                                     npts, rx_chunk, c, fs, out_re, out_im);
    } else {
        cudaFuncSetAttribute(k_tfm<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, 320 * kTB * 4);
        k_tfm<3><<<(unsigned)blocks, kTB, smem, s>>>(A, n_tx, n_rx, nt, tx_pos, rx_pos, axes, npix,
                                                     npts, rx_chunk, c, fs, out_re, out_im);
    }
    return cuda_status(cudaGetLastError());
}
