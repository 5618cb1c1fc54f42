// usct_invert.cu -- the device side of the FWI model-update loop.
//
// fwi.invert (simulation/ringfwi/fwi.py:535-660) and its Gauss-Newton variant
// (fwi.py:434-532) wrap the gradient in a few whole-model FP64 operations per
// iteration: mask, Gaussian smoothing of the gradient (scipy.ndimage
// gaussian_filter, fwi.py:633-636), max|g|, the trial model m + step*d with
// effective bounds inside the update mask (fwi.py:641-650), and for
// Gauss-Newton the conjugate-gradient vector algebra (fwi.py:485-504).  Run on
// the host these force the model and gradient across PCIe every iteration;
// these kernels keep both resident.
//
// Every elementwise operation rounds exactly as the NumPy expression it
// replaces (FP64, no contraction: the library is built with -fmad=false), the
// smoothing adds its taps in scipy's order for symmetric kernels (centre tap
// first, then the pairs from the outermost in), and the reductions use a fixed
// partition and a fixed tree, so every result is reproducible run to run.
// Dot products and sums therefore differ from NumPy's pairwise/BLAS order in
// the last bits; max|x| is exact.
//
// All of these are memory-bound streams of N doubles (N = model cells); the
// smoothing reads 2r+1 neighbours per output along one axis per pass, served
// from L1/L2 after the first touch.
#include <cuda_runtime.h>

#include <cstdint>

#include "usct_gb300.h"

int usct_internal_error(int code, const char* msg);   // usct_engine.cu

namespace {

constexpr int kMaxRadius = USCT_SMOOTH_MAX_RADIUS;
constexpr int kRedBlocks = 608;                         // 4 x 152 SMs
constexpr int kRedThreads = 256;

struct Taps {
    double w[kMaxRadius + 1];   // w[0] centre, w[j] the weight at distance j
    int r;
};

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return USCT_OK;
    return usct_internal_error(e == cudaErrorMemoryAllocation ? USCT_ERR_NOMEM : USCT_ERR_CUDA,
                               cudaGetErrorString(e));
}

int blocks_for(size_t n) {
    const size_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b ? b : 1) : 152 * 16);
}

// scipy 'reflect' (half-sample symmetric) extension, periodic with period 2n
__device__ __forceinline__ long long reflect(long long i, long long n) {
    const long long p = 2 * n;
    long long k = i % p;
    if (k < 0) k += p;
    return k >= n ? p - 1 - k : k;
}

// One separable pass along an axis of length len and element stride stride.
__global__ void k_smooth_axis(const double* __restrict__ in, double* __restrict__ out,
                              long long n, long long len, long long stride, Taps t) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const long long i = (e / stride) % len;
        const long long base = e - i * stride;
        double acc = in[e] * t.w[0];
        for (int j = t.r; j >= 1; --j) {
            const double a = in[base + reflect(i - j, len) * stride];
            const double b = in[base + reflect(i + j, len) * stride];
            acc = acc + (a + b) * t.w[j];
        }
        out[e] = acc;
    }
}

__global__ void k_mul(const double* __restrict__ x, const double* __restrict__ mask, double* out,
                      long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = mask ? x[i] * mask[i] : x[i];
}

__global__ void k_axpy(const double* y, double a, const double* x, double* out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double ax = a * x[i];
        out[i] = y ? y[i] + ax : ax;
    }
}

// m + a*d, then np.clip to [lo, hi] where mask > 0 (everywhere without a mask)
__global__ void k_trial(const double* __restrict__ m, double a, const double* __restrict__ d,
                        const double* __restrict__ lo, const double* __restrict__ hi,
                        const double* __restrict__ mask, double* out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double v = m[i] + a * d[i];
        if (lo && (!mask || mask[i] > 0.0)) {
            double c = v < lo[i] ? lo[i] : v;
            c = c > hi[i] ? hi[i] : c;
            v = c;
        }
        out[i] = v;
    }
}

// max|x| over the grid: per-block tree, then an atomic max on the bit pattern
// (non-negative doubles order like their unsigned 64-bit images)
__global__ void k_absmax(const double* __restrict__ x, long long n, unsigned long long* out) {
    __shared__ double s[kRedThreads];
    double v = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double a = fabs(x[i]);
        v = a > v ? a : v;
    }
    s[threadIdx.x] = v;
    __syncthreads();
    for (int k = kRedThreads / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) s[threadIdx.x] = s[threadIdx.x + k] > s[threadIdx.x]
                                                      ? s[threadIdx.x + k] : s[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(s[0]));
}

// sum_i x_i * y_i (y == NULL: sum_i x_i) in a fixed order: thread t of block b
// adds elements b*256 + t + k*608*256 in k order, each block reduces by a
// fixed tree into ws[1 + b], and one thread adds the 608 partials in b order.
__global__ void k_dot_part(const double* __restrict__ x, const double* __restrict__ y, long long n,
                           double* ws) {
    __shared__ double s[kRedThreads];
    double v = 0.0;
    for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n;
         i += (long long)kRedBlocks * kRedThreads)
        v = v + (y ? x[i] * y[i] : x[i]);
    s[threadIdx.x] = v;
    __syncthreads();
    for (int k = kRedThreads / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) s[threadIdx.x] = s[threadIdx.x] + s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) ws[1 + blockIdx.x] = s[0];
}

__global__ void k_dot_final(double* ws) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double v = 0.0;
        for (int b = 0; b < kRedBlocks; ++b) v = v + ws[1 + b];
        ws[0] = v;
    }
}

}  // namespace

extern "C" int usct_smooth_dev(const double* in, double* out, double* tmp, int ndim,
                               const int* dims, const double* taps, int radius, void* stream) {
    if (!in || !out || !dims || !taps) return usct_internal_error(USCT_ERR_ARG, "null argument");
    if (ndim < 1 || ndim > 3) return usct_internal_error(USCT_ERR_ARG, "ndim must be 1..3");
    if (radius < 0 || radius > kMaxRadius)
        return usct_internal_error(USCT_ERR_ARG, "smoothing radius must be 0..USCT_SMOOTH_MAX_RADIUS");
    if (ndim > 1 && !tmp) return usct_internal_error(USCT_ERR_ARG, "tmp is null");
    if (out == in || (ndim > 1 && (tmp == in || tmp == out)))
        return usct_internal_error(USCT_ERR_ARG, "in, out and tmp must be distinct buffers");
    long long n = 1;
    for (int d = 0; d < ndim; ++d) {
        if (dims[d] < 1) return usct_internal_error(USCT_ERR_ARG, "dims must be >= 1");
        n *= dims[d];
    }
    Taps t{};
    t.r = radius;
    for (int j = 0; j <= radius; ++j) t.w[j] = taps[j];
    cudaStream_t s = (cudaStream_t)stream;
    // axis 0 first (scipy applies the 1-D passes in axis order); the passes
    // alternate between tmp and out so the last one lands in out
    const double* src = in;
    long long stride = n;
    for (int d = 0; d < ndim; ++d) {
        stride /= dims[d];
        double* dst = ((ndim - 1 - d) % 2 == 0) ? out : tmp;
        k_smooth_axis<<<blocks_for((size_t)n), 256, 0, s>>>(src, dst, n, dims[d], stride, t);
        src = dst;
    }
    return cuda_status(cudaGetLastError());
}

extern "C" int usct_vec_mul_dev(const double* x, const double* mask, double* out, size_t n,
                                void* stream) {
    if (!x || !out) return usct_internal_error(USCT_ERR_ARG, "null argument");
    k_mul<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(x, mask, out, (long long)n);
    return cuda_status(cudaGetLastError());
}

extern "C" int usct_vec_axpy_dev(const double* y, double a, const double* x, double* out,
                                 size_t n, void* stream) {
    if (!x || !out) return usct_internal_error(USCT_ERR_ARG, "null argument");
    k_axpy<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(y, a, x, out, (long long)n);
    return cuda_status(cudaGetLastError());
}

extern "C" int usct_model_trial_dev(const double* m, double a, const double* d, const double* lo,
                                    const double* hi, const double* mask, double* out, size_t n,
                                    void* stream) {
    if (!m || !d || !out) return usct_internal_error(USCT_ERR_ARG, "null argument");
    if ((lo == nullptr) != (hi == nullptr))
        return usct_internal_error(USCT_ERR_ARG, "lo and hi must both be given or both be null");
    k_trial<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(m, a, d, lo, hi, mask, out,
                                                            (long long)n);
    return cuda_status(cudaGetLastError());
}

extern "C" int usct_vec_absmax_dev(const double* x, size_t n, double* out, void* stream) {
    if (!x || !out) return usct_internal_error(USCT_ERR_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t ce = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (ce != cudaSuccess) return cuda_status(ce);
    k_absmax<<<blocks_for(n), kRedThreads, 0, s>>>(x, (long long)n,
                                                   reinterpret_cast<unsigned long long*>(out));
    return cuda_status(cudaGetLastError());
}

extern "C" int usct_vec_dot_dev(const double* x, const double* y, size_t n, double* ws,
                                void* stream) {
    if (!x || !ws) return usct_internal_error(USCT_ERR_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    k_dot_part<<<kRedBlocks, kRedThreads, 0, s>>>(x, y, (long long)n, ws);
    k_dot_final<<<1, 32, 0, s>>>(ws);
    return cuda_status(cudaGetLastError());
}
