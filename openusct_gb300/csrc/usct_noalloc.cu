// usct_noalloc.cu -- a forward FMC entry point that allocates no device memory.
//
// Who needs it: callers whose device memory is owned by someone else and who
// therefore may not call cudaMalloc themselves or let a library do it -- a
// host application that has reserved the whole GPU for its own pool allocator,
// a plugin running inside such a host (a MATLAB MEX file, a GUI previewing one
// transmit at a time), or a real-time acquisition loop that must never enter
// the CUDA allocator.  The regular entry points need a plan (whose creation
// allocates the per-tile source/receiver lists) and caller-sized workspaces;
// this one needs neither.
//
// How: every piece of scratch -- the FP32 model S = dt^2/m, the sponge, the
// FP32 wavelet, the two wavefield levels, the per-tile source and receiver
// lists and the receiver slot samples -- lives in one file-scope static device
// array of USCT_NOALLOC_SCRATCH_BYTES (64 MiB).  Every GPU that loads this
// library holds that array until the process exits.  The caller still passes
// the device model, wavelet and output buffer.  Problems whose scratch does not
// fit are rejected with USCT_ERR_ARG and a message giving the bytes needed.
//
// The array's name is not a device address in host code, so the first call on
// each device resolves it once with cudaGetSymbolAddress (that device must be
// current); make that first call before any stream capture.  The address is
// kept per device together with the context it was resolved in, and resolved
// again when another context is current on that device (after a
// cudaDeviceReset, or a context the caller made current itself).  Every call
// uploads its per-tile source and receiver lists from host memory local to the
// call, so a call on a stream that is capturing is refused with USCT_ERR_ARG
// before it enqueues anything.  All calls share the array and it keeps the
// previous call's contents: each call clears the wavefield levels and the
// level-0 receiver row it relies on being zero, and calls that overlap on the
// GPU (two streams, two host threads) race on the array -- serialise them.
//
// The stencil is the same k_forward kernel as the batched engine, run one
// transmit at a time (one shot channel), so the traces equal those of
// usct_forward_fmc_dev.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "usct_gb300.h"
#include "usct_kernels.cuh"

using namespace usct;

int usct_internal_error(int code, const char* msg);   // usct_engine.cu

static __device__ __align__(256) unsigned char g_noalloc_scratch[USCT_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_scratch_mu;
void* g_scratch_ptr[256] = {};
CUcontext g_scratch_ctx[256] = {};

// the driver's cuCtxGetCurrent, looked up once through the runtime (the
// library links no driver library of its own)
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (CtxGetCurrentFn)f;
    });
    return fn;
}

int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return usct_internal_error(USCT_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= 256) return usct_internal_error(USCT_ERR_ARG, "device ordinal out of range");
    CtxGetCurrentFn get = ctx_get_current();
    if (!get) return usct_internal_error(USCT_ERR_CUDA, "cuCtxGetCurrent is not available");
    CUcontext ctx = nullptr;
    if (get(&ctx) != CUDA_SUCCESS) ctx = nullptr;   // none yet: the runtime makes one below
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!ctx || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);   // makes the primary context current if needed
        if (e != cudaSuccess || !p) {
            char msg[256];
            snprintf(msg, sizeof(msg), "cudaGetSymbolAddress of the static scratch failed: %s",
                     cudaGetErrorString(e));
            return usct_internal_error(USCT_ERR_CUDA, msg);
        }
        if (get(&ctx) != CUDA_SUCCESS || !ctx)
            return usct_internal_error(USCT_ERR_CUDA, "no current CUDA context for the static scratch");
        g_scratch_ptr[dev] = p;
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_ptr[dev];
    return USCT_OK;
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

__global__ void k_na_prepare(const double* __restrict__ m, const double* __restrict__ sp, float* S,
                             float* spo, double dt2, int nx, int nxs, long long ncp) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncp;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % nxs);
        const long long r = i / nxs;
        if (x < nx) {
            const long long u = r * nx + x;
            S[i] = (float)(dt2 / m[u]);
            if (spo) spo[i] = sp ? (float)sp[u] : 1.f;
        } else {
            S[i] = 0.f;
            if (spo) spo[i] = 0.f;
        }
    }
}

__global__ void k_na_wavelet(const double* __restrict__ w, float* o, int nt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nt) o[i] = (float)w[i];
}

// trace of receiver j = ordered sum of its slot samples (one shot channel)
__global__ void k_na_gather(const float* __restrict__ rs, int nslot, int nt, int nrx,
                            const int* __restrict__ rx_ptr, float* out) {
    const long long rows = (long long)nt * nrx;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows;
         r += (long long)gridDim.x * blockDim.x) {
        const int n = (int)(r / nrx), j = (int)(r % nrx);
        float tr = 0.f;
        for (int e = rx_ptr[j]; e < rx_ptr[j + 1]; ++e) tr = tr + rs[(long long)n * nslot + e];
        out[r] = tr;
    }
}

}  // namespace

extern "C" int usct_forward_fmc_noalloc(int ndim, const int* dims, double h, double dt, int nt,
                                        int n_tx, const int* tx_ptr, const int64_t* tx_cell,
                                        const double* tx_w, int n_rx, const int* rx_ptr,
                                        const int64_t* rx_cell, const double* rx_w,
                                        const double* m, const double* sponge,
                                        const double* wavelet, float* data, void* stream) {
    // ---- host-side checks and layout (no CUDA call before the size check) ----
    if (ndim != 2 && ndim != 3) return usct_internal_error(USCT_ERR_ARG, "ndim must be 2 or 3");
    if (!dims || !tx_ptr || !rx_ptr || !m || !wavelet || !data)
        return usct_internal_error(USCT_ERR_ARG, "null argument");
    if (n_tx >= 1 && tx_ptr[n_tx] > 0 && (!tx_cell || !tx_w))
        return usct_internal_error(USCT_ERR_ARG, "null source cell or weight array");
    if (n_rx >= 1 && (!rx_cell || !rx_w))
        return usct_internal_error(USCT_ERR_ARG, "null receiver cell or weight array");
    for (int d = 0; d < ndim; ++d)
        if (dims[d] < 3) return usct_internal_error(USCT_ERR_ARG, "every grid extent must be >= 3");
    if (nt < 2 || n_tx < 1 || n_rx < 1 || !(h > 0) || !(dt > 0))
        return usct_internal_error(USCT_ERR_ARG, "need nt >= 2, h, dt > 0 and at least one element");
    Geo g{};
    if (ndim == 3) { g.nz = dims[0]; g.ny = dims[1]; g.nx = dims[2]; }
    else { g.nz = dims[0]; g.ny = 1; g.nx = dims[1]; }
    const long long ncell = (long long)g.nz * g.ny * g.nx;
    const int nse = tx_ptr[n_tx], nre = rx_ptr[n_rx];
    if (tx_ptr[0] != 0 || rx_ptr[0] != 0 || nse < 0 || nre < 1)
        return usct_internal_error(USCT_ERR_ARG, "malformed source/receiver CSR");
    for (int t = 0; t < n_tx; ++t)
        if (tx_ptr[t + 1] < tx_ptr[t]) return usct_internal_error(USCT_ERR_ARG, "source CSR not monotone");
    for (int j = 0; j < n_rx; ++j)
        if (rx_ptr[j + 1] < rx_ptr[j]) return usct_internal_error(USCT_ERR_ARG, "receiver CSR not monotone");
    for (int e = 0; e < nse; ++e)
        if (tx_cell[e] < 0 || tx_cell[e] >= ncell) return usct_internal_error(USCT_ERR_ARG, "source cell outside the grid");
    for (int e = 0; e < nre; ++e)
        if (rx_cell[e] < 0 || rx_cell[e] >= ncell) return usct_internal_error(USCT_ERR_ARG, "receiver cell outside the grid");

    g.C = 1; g.logC = 0;
    g.nxs = (g.nx + 3) & ~3;
    g.RP = g.nxs;
    g.PP = (long long)g.RP * g.ny;
    g.CPP = (long long)g.nxs * g.ny;
    g.inv_h2 = (float)(1.0 / (h * h));
    const bool is3d = ndim == 3;
    const int txv = is3d ? 32 : 128, ty = is3d ? 8 : 1, TXF = 4 * txv;
    const int ntx_t = (g.RP + TXF - 1) / TXF, nty_t = (g.ny + ty - 1) / ty, ntiles = ntx_t * nty_t;
    g.ntiles_x = ntx_t;
    {
        long long nzc = (152LL * 16 + ntiles - 1) / ntiles;
        nzc = std::max<long long>(1, std::min<long long>(nzc, g.nz / 8 > 0 ? g.nz / 8 : 1));
        g.zc = (int)((g.nz + nzc - 1) / nzc);
    }
    const int nzc = (g.nz + g.zc - 1) / g.zc;
    const size_t cells_p = (size_t)g.CPP * g.nz;

    const size_t b_S = al256(cells_p * 4), b_sp = sponge ? al256(cells_p * 4) : 0;
    const size_t b_wav = al256((size_t)nt * 4), b_lv = al256(cells_p * 4);
    const size_t b_rs = al256((size_t)nt * nre * 4);
    const size_t b_sptr = al256((size_t)n_tx * (ntiles + 1) * 4);
    const size_t b_sent = al256((size_t)std::max(nse, 1) * sizeof(SrcEnt));
    const size_t b_rptr = al256((size_t)(ntiles + 1) * 4);
    const size_t b_rent = al256((size_t)nre * sizeof(RxEnt));
    const size_t b_rxp = al256((size_t)(n_rx + 1) * 4);
    const size_t need = b_S + b_sp + b_wav + 2 * b_lv + b_rs + b_sptr + b_sent + b_rptr + b_rent + b_rxp;
    if (need > (size_t)USCT_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "problem needs %zu bytes of scratch; the static no-alloc area holds %u bytes",
                 need, (unsigned)USCT_NOALLOC_SCRATCH_BYTES);
        return usct_internal_error(USCT_ERR_ARG, msg);
    }

    // per-tile source lists (one per transmit) and receiver list, host side
    std::vector<int> sptr((size_t)n_tx * (ntiles + 1));
    std::vector<SrcEnt> sent;
    sent.reserve(nse);
    for (int t = 0; t < n_tx; ++t) {
        std::vector<std::pair<int, SrcEnt>> tmp;
        for (int e = tx_ptr[t]; e < tx_ptr[t + 1]; ++e) {
            const int x = (int)(tx_cell[e] % g.nx);
            const long long r = tx_cell[e] / g.nx;
            const int y = (int)(r % g.ny), z = (int)(r / g.ny);
            const int xt = x / TXF, yt = y / ty;
            tmp.push_back({xt + ntx_t * yt, SrcEnt{z, y - yt * ty, x - xt * TXF, (float)tx_w[e]}});
        }
        std::stable_sort(tmp.begin(), tmp.end(), [](const auto& a, const auto& b) {
            return a.first != b.first ? a.first < b.first : a.second.z < b.second.z;
        });
        size_t q = 0;
        const int base = (int)sent.size();
        for (int tl = 0; tl < ntiles; ++tl) {
            sptr[(size_t)t * (ntiles + 1) + tl] = base + (int)q;
            while (q < tmp.size() && tmp[q].first == tl) sent.push_back(tmp[q++].second);
        }
        sptr[(size_t)t * (ntiles + 1) + ntiles] = base + (int)q;
    }
    std::vector<std::pair<int, RxEnt>> rtmp;
    for (int j = 0; j < n_rx; ++j)
        for (int e = rx_ptr[j]; e < rx_ptr[j + 1]; ++e) {
            const int x = (int)(rx_cell[e] % g.nx);
            const long long r = rx_cell[e] / g.nx;
            const int y = (int)(r % g.ny), z = (int)(r / g.ny);
            const int xt = x / TXF, yt = y / ty;
            rtmp.push_back({xt + ntx_t * yt, RxEnt{z, y - yt * ty, x - xt * TXF, e, j, (float)rx_w[e], 0, 0}});
        }
    std::stable_sort(rtmp.begin(), rtmp.end(), [](const auto& a, const auto& b) {
        if (a.first != b.first) return a.first < b.first;
        if (a.second.z != b.second.z) return a.second.z < b.second.z;
        if (a.second.ly != b.second.ly) return a.second.ly < b.second.ly;
        return a.second.lcell < b.second.lcell;
    });
    std::vector<int> rptr(ntiles + 1);
    std::vector<RxEnt> rent;
    {
        size_t q = 0;
        for (int tl = 0; tl < ntiles; ++tl) {
            rptr[tl] = (int)q;
            while (q < rtmp.size() && rtmp[q].first == tl) rent.push_back(rtmp[q++].second);
        }
        rptr[ntiles] = (int)q;
    }

    // ---- device side: carve the static scratch ----
    cudaStream_t s = (cudaStream_t)stream;
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        const cudaError_t e = cudaStreamIsCapturing(s, &cs);
        if (e != cudaSuccess) return usct_internal_error(USCT_ERR_CUDA, cudaGetErrorString(e));
        if (cs != cudaStreamCaptureStatusNone)
            return usct_internal_error(USCT_ERR_ARG,
                                       "usct_forward_fmc_noalloc: the stream is capturing; this "
                                       "entry point uploads host lists local to the call and "
                                       "cannot be captured");
    }
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != USCT_OK) return rc;
    char* c = (char*)base;
    float* S = (float*)c; c += b_S;
    float* sp = sponge ? (float*)c : nullptr; c += b_sp;
    float* wav = (float*)c; c += b_wav;
    float* P0 = (float*)c; c += b_lv;
    float* P1 = (float*)c; c += b_lv;
    float* rs = (float*)c; c += b_rs;
    int* d_sptr = (int*)c; c += b_sptr;
    SrcEnt* d_sent = (SrcEnt*)c; c += b_sent;
    int* d_rptr = (int*)c; c += b_rptr;
    RxEnt* d_rent = (RxEnt*)c; c += b_rent;
    int* d_rxp = (int*)c;

#define NA_CUDA(x)                                                                   \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess) return usct_internal_error(USCT_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

    NA_CUDA(cudaMemcpyAsync(d_sptr, sptr.data(), sptr.size() * 4, cudaMemcpyHostToDevice, s));
    if (!sent.empty())
        NA_CUDA(cudaMemcpyAsync(d_sent, sent.data(), sent.size() * sizeof(SrcEnt), cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(d_rptr, rptr.data(), rptr.size() * 4, cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(d_rent, rent.data(), rent.size() * sizeof(RxEnt), cudaMemcpyHostToDevice, s));
    NA_CUDA(cudaMemcpyAsync(d_rxp, rx_ptr, (size_t)(n_rx + 1) * 4, cudaMemcpyHostToDevice, s));
    const int pg = (int)std::min<long long>(((long long)cells_p + 255) / 256, 152LL * 32);
    k_na_prepare<<<pg, 256, 0, s>>>(m, sponge, S, sp, dt * dt, g.nx, g.nxs, (long long)cells_p);
    k_na_wavelet<<<(nt + 255) / 256, 256, 0, s>>>(wavelet, wav, nt);
    NA_CUDA(cudaGetLastError());

    const dim3 grid(ntx_t, nty_t, nzc);
    const size_t smem = sizeof(float) * 2 * (ty + 2) * (TXF + 2 * 4);
    for (int t = 0; t < n_tx; ++t) {
        NA_CUDA(cudaMemsetAsync(P0, 0, 2 * b_lv, s));
        NA_CUDA(cudaMemsetAsync(rs, 0, (size_t)nre * 4, s));
        for (int n = 1; n < nt; ++n) {
            FwdArgs a{};
            a.g = g;
            a.pc = (n & 1) ? P0 : P1;
            a.pp = (n & 1) ? P1 : P0;
            a.pn = (n & 1) ? P1 : P0;
            a.S = S;
            a.sp = sp;
            a.wav = wav;
            a.n = n;
            a.s_ptr = d_sptr + (size_t)t * (ntiles + 1);
            a.s_ent = d_sent;
            a.r_ptr = d_rptr;
            a.r_ent = d_rent;
            a.rs = rs + (size_t)n * nre;
            if (is3d) k_forward<32, 8, true, false><<<grid, dim3(32, 8), smem, s>>>(a);
            else k_forward<128, 1, false, false><<<grid, dim3(128, 1), smem, s>>>(a);
        }
        NA_CUDA(cudaGetLastError());
        const long long rows = (long long)nt * n_rx;
        k_na_gather<<<(int)std::min<long long>((rows + 255) / 256, 152LL * 16), 256, 0, s>>>(
            rs, nre, nt, n_rx, d_rxp, data + (size_t)t * rows);
        NA_CUDA(cudaGetLastError());
    }
#undef NA_CUDA
    return USCT_OK;
}
