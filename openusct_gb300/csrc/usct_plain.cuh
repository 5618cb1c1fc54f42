// usct_plain.cuh -- the plain one-shot-per-launch GPU form, included by
// usct_engine.cu (it reads the plan internals).
//
// It restates the structure of the reference's CuPy backend
// (software/python/uap_gpu.py:28-64 kernels, :100-140 loops): one thread per
// cell, a 7-point (5-point) stencil read straight from global memory, and per
// time step separate launches for the stencil update, the source injection
// (p[src] += S*w*wavelet[n-1], uap_gpu.py:112), the receiver gather
// (uap_gpu.py:116), the adjoint update (uap_gpu.py:45-60), the adjoint
// injection (uap_gpu.py:135) and the imaging condition (uap_gpu.py:62-64).
// Shots run one after another; the forward history of every level is kept in
// HBM (written in place by the stencil launch rather than copied).  The
// gradient accumulator is FP64 so both forms meet the same accuracy bar.  It
// is the denominator of the batched-vs-plain comparison and shares no kernel
// with the batched engine.  Point elements only, like the reference GPU path.

__global__ void k_plain_S(const double* __restrict__ m, float* S, double dt2, long long N) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x)
        S[i] = (float)(dt2 / m[i]);
}

__global__ void k_plain_fwd(const float* __restrict__ pc, const float* pp, const float* __restrict__ S,
                            float* pn, int nz, int ny, int nx, int is3d, float inv_h2, long long N) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int ix = (int)(c % nx);
    const long long r = c / nx;
    const int iy = (int)(r % ny);
    const int iz = (int)(r / ny);
    const long long syz = (long long)ny * nx;
    float lap = 0.0f;
    if (ix > 0 && ix < nx - 1 && iz > 0 && iz < nz - 1) {
        if (is3d) {
            if (iy > 0 && iy < ny - 1)
                lap = (pc[c + 1] + pc[c - 1] + pc[c + nx] + pc[c - nx] + pc[c + syz] + pc[c - syz] -
                       6.0f * pc[c]) * inv_h2;
        } else {
            lap = (pc[c + 1] + pc[c - 1] + pc[c + syz] + pc[c - syz] - 4.0f * pc[c]) * inv_h2;
        }
    }
    pn[c] = 2.0f * pc[c] - pp[c] + S[c] * lap;
}

__global__ void k_plain_inject(float* pn, const float* __restrict__ S, const int64_t* __restrict__ cell,
                               const float* __restrict__ w, int ns, const float* __restrict__ wav, int n) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const float wv = wav[n - 1];
        for (int e = 0; e < ns; ++e) pn[cell[e]] += S[cell[e]] * (w[e] * wv);
    }
}

__global__ void k_plain_gather(const float* __restrict__ p, const int64_t* __restrict__ rcell, int nrx,
                               float* row) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nrx) row[j] = p[rcell[j]];
}

__global__ void k_plain_adj(const float* __restrict__ l1, const float* l2, const float* __restrict__ S,
                            float* lk, int nz, int ny, int nx, int is3d, float inv_h2, long long N) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int ix = (int)(c % nx);
    const long long r = c / nx;
    const int iy = (int)(r % ny);
    const int iz = (int)(r / ny);
    const long long syz = (long long)ny * nx;
    float lap = 0.0f;
    if (ix > 0 && ix < nx - 1 && iz > 0 && iz < nz - 1) {
        if (is3d) {
            if (iy > 0 && iy < ny - 1)
                lap = (S[c + 1] * l1[c + 1] + S[c - 1] * l1[c - 1] + S[c + nx] * l1[c + nx] +
                       S[c - nx] * l1[c - nx] + S[c + syz] * l1[c + syz] + S[c - syz] * l1[c - syz] -
                       6.0f * S[c] * l1[c]) * inv_h2;
        } else {
            lap = (S[c + 1] * l1[c + 1] + S[c - 1] * l1[c - 1] + S[c + syz] * l1[c + syz] +
                   S[c - syz] * l1[c - syz] - 4.0f * S[c] * l1[c]) * inv_h2;
        }
    }
    lk[c] = 2.0f * l1[c] - l2[c] + lap;
}

__global__ void k_plain_adj_inject(float* lk, const int64_t* __restrict__ rcell, int nrx,
                                   const float* __restrict__ res_k) {
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (int j = 0; j < nrx; ++j) lk[rcell[j]] -= res_k[j];
}

__global__ void k_plain_grad(double* g, const float* __restrict__ lk, const float* __restrict__ uk,
                             const float* __restrict__ uk1, const float* __restrict__ uk2, long long N) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const float d2p = uk[c] - 2.0f * uk1[c] + (uk2 ? uk2[c] : 0.0f);
    g[c] += (double)(lk[c] * d2p);
}

__global__ void __launch_bounds__(1024) k_plain_residual(const float* __restrict__ rec,
                                                         const float* __restrict__ dobs, float* res,
                                                         long long n, double* J) {
    __shared__ double sj[1024];
    double acc = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const float r = rec[i] - dobs[i];
        res[i] = r;
        acc += 0.5 * (double)r * (double)r;
    }
    sj[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sj[threadIdx.x] += sj[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *J = sj[0];
}

__global__ void k_plain_final(const double* __restrict__ g, const double* __restrict__ m, double* grad,
                              long long N) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x)
        grad[i] = g[i] / m[i];
}

struct PlainWS {
    float* S; float* hist; float* L[3]; float* rec; float* res; float* wav; double* jt; double* g;
};

static bool plain_point_elements(const usct_plan* p) {
    for (int t = 0; t < p->n_tx; ++t)
        if (p->h_tx_ptr[t + 1] - p->h_tx_ptr[t] != 1) return false;
    for (int j = 0; j < p->n_rx; ++j)
        if (p->h_rx_ptr[j + 1] - p->h_rx_ptr[j] != 1 || p->h_rx_w[j] != 1.0) return false;
    return true;
}

static PlainWS carve_plain(const usct_plan* p, void* base, int gradient) {
    char* c = (char*)base;
    PlainWS w{};
    const size_t lv = al256(p->N * sizeof(float));
    w.S = (float*)c; c += lv;
    const int nlev = gradient ? p->nt : 3;
    w.hist = (float*)c; c += (size_t)nlev * lv;
    for (int i = 0; i < 3; ++i) { w.L[i] = (float*)c; c += lv; }
    w.rec = (float*)c; c += al256((size_t)p->nt * p->n_rx * sizeof(float));
    w.res = (float*)c; c += al256((size_t)p->nt * p->n_rx * sizeof(float));
    w.wav = (float*)c; c += al256((size_t)p->nt * sizeof(float));
    w.jt = (double*)c; c += al256((size_t)p->n_tx * sizeof(double));
    w.g = (double*)c;
    return w;
}

extern "C" size_t usct_plain_bytes(const usct_plan* p, int gradient) {
    if (!p) return 0;
    const size_t lv = al256(p->N * sizeof(float));
    const int nlev = gradient ? p->nt : 3;
    return lv * (1 + (size_t)nlev + 3) + 2 * al256((size_t)p->nt * p->n_rx * sizeof(float)) +
           al256((size_t)p->nt * sizeof(float)) + al256((size_t)p->n_tx * sizeof(double)) +
           al256(p->N * sizeof(double));
}

static int plain_forward_shot(usct_plan* p, const PlainWS& w, int t, bool keep_hist, float* rec_out,
                              const float* wav, cudaStream_t s) {
    const Geo& g = p->geo;
    const long long N = (long long)p->N;
    const int bs = 256;
    const int nblk = (int)((N + bs - 1) / bs);
    const size_t lvf = al256(p->N * sizeof(float)) / sizeof(float);
    const int is3d = p->ndim == 3;
    CUDA_TRY(cudaMemsetAsync(rec_out, 0, (size_t)p->n_rx * sizeof(float), s));
    if (keep_hist) {
        CUDA_TRY(cudaMemsetAsync(w.hist, 0, p->N * sizeof(float), s));
        CUDA_TRY(cudaMemsetAsync(w.L[2], 0, p->N * sizeof(float), s));
    } else {
        CUDA_TRY(cudaMemsetAsync(w.hist, 0, 3 * lvf * sizeof(float), s));
    }
    const int e0 = p->h_tx_ptr[t], ns = p->h_tx_ptr[t + 1] - e0;
    for (int n = 1; n < p->nt; ++n) {
        const float* pc;
        const float* pp;
        float* pn;
        if (keep_hist) {
            pc = w.hist + (size_t)(n - 1) * lvf;
            pp = n >= 2 ? w.hist + (size_t)(n - 2) * lvf : w.L[2];
            pn = w.hist + (size_t)n * lvf;
        } else {
            pc = w.hist + (size_t)((n - 1) % 3) * lvf;
            pp = w.hist + (size_t)((n + 1) % 3) * lvf;   // level n-2
            pn = w.hist + (size_t)(n % 3) * lvf;
        }
        k_plain_fwd<<<nblk, bs, 0, s>>>(pc, pp, w.S, pn, g.nz, g.ny, g.nx, is3d, g.inv_h2, N);
        k_plain_inject<<<1, 32, 0, s>>>(pn, w.S, p->d_tx_cell + e0, p->d_tx_w + e0, ns, wav, n);
        k_plain_gather<<<(p->n_rx + 255) / 256, 256, 0, s>>>(pn, p->d_rx_cell, p->n_rx,
                                                             rec_out + (size_t)n * p->n_rx);
        p->launches += 3;
    }
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}

extern "C" int usct_plain_forward_fmc_dev(usct_plan* p, const double* m, const double* wavelet,
                                          float* data, void* ws, void* stream) {
    if (!p || !m || !wavelet || !data || !ws) return set_err(USCT_ERR_ARG, "null argument");
    if (!plain_point_elements(p)) return set_err(USCT_ERR_ARG, "plain form supports point elements only");
    cudaStream_t s = (cudaStream_t)stream;
    PlainWS w = carve_plain(p, ws, 0);
    k_plain_S<<<grid1d((long long)p->N), 256, 0, s>>>(m, w.S, p->dt * p->dt, (long long)p->N);
    float* wav = w.wav;
    k_wavelet<<<(p->nt + 255) / 256, 256, 0, s>>>(wavelet, wav, p->nt);
    p->launches += 2;
    for (int t = 0; t < p->n_tx; ++t)
        TRY(plain_forward_shot(p, w, t, false, data + (size_t)t * p->nt * p->n_rx, wav, s));
    return USCT_OK;
}

extern "C" int usct_plain_misfit_and_gradient_dev(usct_plan* p, const double* m, const double* wavelet,
                                                  const float* dobs, double* J, double* grad, void* ws,
                                                  void* stream) {
    if (!p || !m || !wavelet || !dobs || !grad || !ws) return set_err(USCT_ERR_ARG, "null argument");
    if (!plain_point_elements(p)) return set_err(USCT_ERR_ARG, "plain form supports point elements only");
    cudaStream_t s = (cudaStream_t)stream;
    PlainWS w = carve_plain(p, ws, 1);
    const Geo& g = p->geo;
    const long long N = (long long)p->N;
    const int bs = 256;
    const int nblk = (int)((N + bs - 1) / bs);
    const size_t lvf = al256(p->N * sizeof(float)) / sizeof(float);
    const int is3d = p->ndim == 3;
    k_plain_S<<<grid1d(N), 256, 0, s>>>(m, w.S, p->dt * p->dt, N);
    float* wav = w.wav;
    k_wavelet<<<(p->nt + 255) / 256, 256, 0, s>>>(wavelet, wav, p->nt);
    CUDA_TRY(cudaMemsetAsync(w.g, 0, p->N * sizeof(double), s));
    p->launches += 2;
    const long long nrec = (long long)p->nt * p->n_rx;
    for (int t = 0; t < p->n_tx; ++t) {
        TRY(plain_forward_shot(p, w, t, true, w.rec, wav, s));
        double* Jt = J ? J + t : w.jt + t;
        k_plain_residual<<<1, 1024, 0, s>>>(w.rec, dobs + (size_t)t * nrec, w.res, nrec, Jt);
        ++p->launches;
        CUDA_TRY(cudaMemsetAsync(w.L[0], 0, 2 * lvf * sizeof(float), s));
        for (int k = p->nt - 1; k >= 1; --k) {
            const float* l1 = w.L[(k + 1) & 1];
            float* lk = w.L[k & 1];   // in place over lam^{k+2}
            k_plain_adj<<<nblk, bs, 0, s>>>(l1, lk, w.S, lk, g.nz, g.ny, g.nx, is3d, g.inv_h2, N);
            k_plain_adj_inject<<<1, 32, 0, s>>>(lk, p->d_rx_cell, p->n_rx, w.res + (size_t)k * p->n_rx);
            k_plain_grad<<<nblk, bs, 0, s>>>(w.g, lk, w.hist + (size_t)k * lvf,
                                             w.hist + (size_t)(k - 1) * lvf,
                                             k >= 2 ? w.hist + (size_t)(k - 2) * lvf : nullptr, N);
            p->launches += 3;
        }
        CUDA_TRY(cudaGetLastError());
    }
    k_plain_final<<<grid1d(N), 256, 0, s>>>(w.g, m, grad, N);
    ++p->launches;
    CUDA_TRY(cudaGetLastError());
    return USCT_OK;
}
