/*
 * usct_oracle.c -- CPU oracle for the ringfwi acoustic hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links, loads or calls
 * this file: it is imported by tests/, by __graft_entry__.smoke() as the
 * checker, and by bench.py's CPU-baseline leg.  It restates, in plain C, the
 * reference's algorithm for the forward leapfrog, the exact discrete adjoint
 * and the gradient accumulation:
 *
 *   libuap.hpp = software/core/libuap.hpp            (C++ FP64 core)
 *   fwi.py     = simulation/ringfwi/fwi.py           (Python FP64 reference)
 *
 * Two restatements live here.
 *
 *  (1) FP64, "o64_*": follows libuap.hpp op for op (laplacian :29-56, forward
 *      :63-105, forward_fmc :109-116, adjoint_residual L2 :125-132,
 *      misfit_and_gradient :169-224) so that on point elements it is
 *      bit-identical to the reference C++ core.  Finite-aperture footprints,
 *      the sponge mask and the Born / Gauss-Newton operators are not in
 *      libuap.hpp; they follow fwi.py (_forward :63-79, misfit_and_gradient
 *      :306-331, _born_forward :366-378, _adjoint_apply :391-407,
 *      gn_hessian_vector :417-431), keeping libuap's Laplacian op order.
 *      A checkpointed variant recomputes each segment of k steps from a stored
 *      pair of levels; it reproduces the full-history result bit for bit and is
 *      what makes FP64 gradients at 3D sizes fit in host memory.
 *
 *  (2) FP32, "o32_*": the same scheme in single precision, in the exact
 *      operation order of the CUDA kernels (explicit fmaf where the kernels use
 *      __fmaf_rn, the same neighbour summation order, the same per-cell shot
 *      reduction tree).  Compiled with -ffp-contract=off it reproduces the GPU
 *      results bit for bit on small grids, which pins indexing, halos, the
 *      batched shot layout and the checkpoint recompute exactly.
 *
 * Conventions shared by both: fields are row-major ([iy][ix] or [iz][iy][ix]);
 * level n is p^n, the source sample used to advance to level n is
 * wavelet[n-1]; p^0 = 0; rec[0] = 0; sources and receivers are CSR lists of
 * (linear cell index, weight) -- a point element is one entry of weight 1.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef long long i64;

static size_t cell_count(const int* dims, int ndim) {
    size_t n = 1;
    for (int d = 0; d < ndim; ++d) n *= (size_t)dims[d];
    return n;
}

/* ------------------------------------------------------------------------- */
/* FP64 restatement                                                          */
/* ------------------------------------------------------------------------- */

/* libuap.hpp:29-56: zero the field, then the 5/7-point stencil on the
 * interior, neighbour order +x, -x, +y, -y, (+z, -z), minus 2*ndim*centre. */
static void lap64(const double* p, double* out, const int* dims, int ndim, double inv_h2) {
    const size_t N = cell_count(dims, ndim);
    for (size_t i = 0; i < N; ++i) out[i] = 0.0;
    if (ndim == 2) {
        const int ny = dims[0], nx = dims[1];
        #pragma omp parallel for schedule(static)
        for (int iy = 1; iy < ny - 1; ++iy)
            for (int ix = 1; ix < nx - 1; ++ix) {
                const size_t c = (size_t)iy * nx + ix;
                out[c] = (p[c + 1] + p[c - 1] + p[c + nx] + p[c - nx] - 4.0 * p[c]) * inv_h2;
            }
    } else {
        const int nz = dims[0], ny = dims[1], nx = dims[2];
        const size_t syz = (size_t)ny * nx;
        #pragma omp parallel for schedule(static)
        for (int iz = 1; iz < nz - 1; ++iz)
            for (int iy = 1; iy < ny - 1; ++iy)
                for (int ix = 1; ix < nx - 1; ++ix) {
                    const size_t c = (size_t)iz * syz + (size_t)iy * nx + ix;
                    out[c] = (p[c + 1] + p[c - 1] + p[c + nx] + p[c - nx] + p[c + syz] + p[c - syz]
                              - 6.0 * p[c]) * inv_h2;
                }
    }
}

static int nseg_of(int nt, int k) { return (nt - 1 + k - 1) / k; }

typedef struct {
    const int* dims;
    int ndim;
    size_t N;
    double inv_h2;
    int nt;
    const double* S;       /* dt^2 / m */
    const double* sponge;  /* NULL = none */
    const double* wav;     /* nt */
    int nrx;
    const int* rx_ptr;     /* nrx+1 */
    const i64* rx_idx;
    const double* rx_w;
} G64;

/* One leapfrog step to level n (libuap.hpp:84-88, fwi.py:64-69):
 *   lap = L p^{n-1};  lap[src] += w * wavelet[n-1];
 *   p^n = 2 p^{n-1} - p^{n-2} + S * lap;  p^n *= sponge. */
static void step64(const G64* g, const double* pp, const double* pc, double* pn, double* lap,
                   int n, int ns, const i64* s_idx, const double* s_w) {
    lap64(pc, lap, g->dims, g->ndim, g->inv_h2);
    for (int e = 0; e < ns; ++e) lap[s_idx[e]] += g->wav[n - 1] * s_w[e];
    const i64 N = (i64)g->N;
    const double* S = g->S;
    #pragma omp parallel for schedule(static)
    for (i64 i = 0; i < N; ++i) pn[i] = 2.0 * pc[i] - pp[i] + S[i] * lap[i];
    if (g->sponge) {
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < N; ++i) pn[i] *= g->sponge[i];
    }
}

/* Receiver sample at level n (libuap.hpp:100-103; fwi.py:74-76 for groups). */
static void sample64(const G64* g, const double* p, double* row) {
    for (int j = 0; j < g->nrx; ++j) {
        double acc = 0.0;
        for (int e = g->rx_ptr[j]; e < g->rx_ptr[j + 1]; ++e) acc += g->rx_w[e] * p[g->rx_idx[e]];
        row[j] = acc;
    }
}

/* One transmit: forward sweep.  rec (nt*nrx) may be NULL; hist (nt*N) may be
 * NULL; ck (nseg*2*N) receives (p^{a-1}, p^a) at a = j*k when k > 0. */
static void forward64(const G64* g, int ns, const i64* s_idx, const double* s_w,
                      double* rec, double* hist, int k, double* ck) {
    const size_t N = g->N;
    double* a = (double*)calloc(N, sizeof(double));
    double* b = (double*)calloc(N, sizeof(double));
    double* c = (double*)calloc(N, sizeof(double));
    double* lap = (double*)calloc(N, sizeof(double));
    double *pp = a, *pc = b, *pn = c;
    if (hist) memset(hist, 0, N * sizeof(double));
    if (rec) memset(rec, 0, (size_t)g->nrx * sizeof(double));
    if (ck) memset(ck, 0, (size_t)nseg_of(g->nt, k) * 2 * N * sizeof(double));
    for (int n = 1; n < g->nt; ++n) {
        step64(g, pp, pc, pn, lap, n, ns, s_idx, s_w);
        double* t = pp; pp = pc; pc = pn; pn = t;
        if (hist) memcpy(hist + (size_t)n * N, pc, N * sizeof(double));
        if (rec) sample64(g, pc, rec + (size_t)n * g->nrx);
        if (ck && (n + 1) % k == 0 && n + 1 < g->nt - 1) {
            /* level n is p^{a-1} of the segment starting at a = n+1 */
            memcpy(ck + (size_t)((n + 1) / k) * 2 * N, pc, N * sizeof(double));
        }
        if (ck && n % k == 0 && n < g->nt - 1) {
            memcpy(ck + ((size_t)(n / k) * 2 + 1) * N, pc, N * sizeof(double));
        }
    }
    free(a); free(b); free(c); free(lap);
}

/* L2 adjoint source (libuap.hpp:125-132): res = dsyn - dobs, J = sum 0.5 r^2. */
static double residual64(const double* dsyn, const double* dobs, size_t total, double* res) {
    double J = 0.0;
    for (size_t q = 0; q < total; ++q) {
        res[q] = dsyn[q] - dobs[q];
        J += 0.5 * res[q] * res[q];
    }
    return J;
}

/* GCN adjoint source (libuap.hpp:133-162, fwi.py:158-167): per receiver trace
 * ns = |dsyn|+eps, no = |dobs|+eps, c = <dsyn/ns, dobs/no>, J = sum (1 - c),
 * res = -(dobs/no - c dsyn/ns)/ns. */
static double residual64_gcn(const double* dsyn, const double* dobs, int nt, int nrx, double* res) {
    const double eps = 1e-12;
    double* ns = (double*)calloc((size_t)nrx, sizeof(double));
    double* no = (double*)calloc((size_t)nrx, sizeof(double));
    double* c = (double*)calloc((size_t)nrx, sizeof(double));
    for (int k = 0; k < nt; ++k) {
        const double* srow = dsyn + (size_t)k * nrx;
        const double* orow = dobs + (size_t)k * nrx;
        for (int j = 0; j < nrx; ++j) {
            ns[j] += srow[j] * srow[j];
            no[j] += orow[j] * orow[j];
        }
    }
    for (int j = 0; j < nrx; ++j) {
        ns[j] = sqrt(ns[j]) + eps;
        no[j] = sqrt(no[j]) + eps;
    }
    for (int k = 0; k < nt; ++k) {
        const double* srow = dsyn + (size_t)k * nrx;
        const double* orow = dobs + (size_t)k * nrx;
        for (int j = 0; j < nrx; ++j) c[j] += (srow[j] / ns[j]) * (orow[j] / no[j]);
    }
    double J = 0.0;
    for (int j = 0; j < nrx; ++j) J += 1.0 - c[j];
    for (int k = 0; k < nt; ++k) {
        const double* srow = dsyn + (size_t)k * nrx;
        const double* orow = dobs + (size_t)k * nrx;
        double* rrow = res + (size_t)k * nrx;
        for (int j = 0; j < nrx; ++j) rrow[j] = -(orow[j] / no[j] - c[j] * (srow[j] / ns[j])) / ns[j];
    }
    free(ns); free(no); free(c);
    return J;
}

/* Backward sweep for one transmit (libuap.hpp:196-219, fwi.py:306-326):
 *   lam^k = 2 lam^{k+1} - lam^{k+2} + L(S lam^{k+1});  lam^k *= sponge;
 *   lam^k[rx] -= r^k * w;  g += lam^k * (U^k - 2U^{k-1} + U^{k-2}).
 * U comes either from a full history (k_ck == 0) or from checkpoints with
 * per-segment recompute (the recomputed levels are bit-identical). */
static void backward64(const G64* g, int ns, const i64* s_idx, const double* s_w,
                       const double* res, const double* hist, int kck, const double* ck,
                       double* grad) {
    const size_t N = g->N;
    const i64 Nll = (i64)N;
    const int nt = g->nt;
    double* lp1 = (double*)calloc(N, sizeof(double));
    double* lp2 = (double*)calloc(N, sizeof(double));
    double* lk = (double*)calloc(N, sizeof(double));
    double* tmp = (double*)calloc(N, sizeof(double));
    double* lap = (double*)calloc(N, sizeof(double));
    double* seg = NULL;   /* levels a-1 .. b of the current segment */
    int seg_a = -1;
    if (!hist) seg = (double*)malloc((size_t)(kck + 2) * N * sizeof(double));
    for (int k = nt - 1; k >= 1; --k) {
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < Nll; ++i) tmp[i] = g->S[i] * lp1[i];
        lap64(tmp, lap, g->dims, g->ndim, g->inv_h2);
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < Nll; ++i) lk[i] = 2.0 * lp1[i] - lp2[i] + lap[i];
        if (g->sponge) {
            #pragma omp parallel for schedule(static)
            for (i64 i = 0; i < Nll; ++i) lk[i] *= g->sponge[i];
        }
        const double* rrow = res + (size_t)k * g->nrx;
        for (int j = 0; j < g->nrx; ++j)
            for (int e = g->rx_ptr[j]; e < g->rx_ptr[j + 1]; ++e) lk[g->rx_idx[e]] -= rrow[j] * g->rx_w[e];

        const double *Uk, *Uk1, *Uk2;
        if (hist) {
            Uk = hist + (size_t)k * N;
            Uk1 = hist + (size_t)(k - 1) * N;
            Uk2 = (k >= 2) ? hist + (size_t)(k - 2) * N : NULL;
        } else {
            const int a = ((k - 1) / kck) * kck;   /* segment (a, b] holding step k */
            if (a != seg_a) {
                int b = a + kck; if (b > nt - 1) b = nt - 1;
                /* restore (p^{a-1}, p^a) and recompute levels a+1..b */
                const size_t j = (size_t)(a / kck);
                memcpy(seg, ck + j * 2 * N, N * sizeof(double));
                memcpy(seg + N, ck + (j * 2 + 1) * N, N * sizeof(double));
                for (int n = a + 1; n <= b; ++n) {
                    double* pp = seg + (size_t)(n - a - 1) * N;
                    double* pc = seg + (size_t)(n - a) * N;
                    double* pn = seg + (size_t)(n - a + 1) * N;
                    step64(g, pp, pc, pn, lap, n, ns, s_idx, s_w);
                }
                seg_a = a;
            }
            Uk = seg + (size_t)(k - a + 1) * N;
            Uk1 = seg + (size_t)(k - a) * N;
            Uk2 = (k >= 2) ? seg + (size_t)(k - a - 1) * N : NULL;
        }
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < Nll; ++i) {
            double d2p = Uk[i] - 2.0 * Uk1[i] + (Uk2 ? Uk2[i] : 0.0);
            grad[i] += lk[i] * d2p;
        }
        double* t = lp2; lp2 = lp1; lp1 = lk; lk = t;
    }
    free(lp1); free(lp2); free(lk); free(tmp); free(lap); free(seg);
}

static void setup64(G64* g, const double* m, const int* dims, int ndim, double h, double dt,
                    int nt, const double* wav, const double* sponge, int nrx, const int* rx_ptr,
                    const i64* rx_idx, const double* rx_w, double** S_out) {
    g->dims = dims; g->ndim = ndim; g->N = cell_count(dims, ndim);
    g->inv_h2 = 1.0 / (h * h); g->nt = nt; g->sponge = sponge; g->wav = wav;
    g->nrx = nrx; g->rx_ptr = rx_ptr; g->rx_idx = rx_idx; g->rx_w = rx_w;
    const double dt2 = dt * dt;
    double* S = (double*)malloc(g->N * sizeof(double));
    for (size_t i = 0; i < g->N; ++i) S[i] = dt2 / m[i];
    g->S = S;
    *S_out = S;
}

/* forward_fmc: data (n_tx, nt, nrx). */
int usct_oracle_forward_fmc(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                            int n_tx, const int* tx_ptr, const i64* tx_idx, const double* tx_w,
                            int nrx, const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                            const double* wav, const double* sponge, double* data) {
    G64 g; double* S;
    setup64(&g, m, dims, ndim, h, dt, nt, wav, sponge, nrx, rx_ptr, rx_idx, rx_w, &S);
    for (int t = 0; t < n_tx; ++t)
        forward64(&g, tx_ptr[t + 1] - tx_ptr[t], tx_idx + tx_ptr[t], tx_w + tx_ptr[t],
                  data + (size_t)t * nt * nrx, NULL, 0, NULL);
    free(S);
    return 0;
}

/* misfit_and_gradient (L2).  kck == 0: full history per transmit, exactly the
 * reference's memory plan; kck > 0: checkpoints every kck steps.  grad gets
 * sum_t g_t / m; returns J. */
double usct_oracle_misfit_and_gradient_mt(const double* m, const int* dims, int ndim, double h,
                                          double dt, int nt, int n_tx, const int* tx_ptr,
                                          const i64* tx_idx, const double* tx_w, int nrx,
                                          const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                          const double* wav, const double* sponge, const double* dobs,
                                          double* grad, int kck, int misfit_type);

double usct_oracle_misfit_and_gradient(const double* m, const int* dims, int ndim, double h, double dt,
                                       int nt, int n_tx, const int* tx_ptr, const i64* tx_idx,
                                       const double* tx_w, int nrx, const int* rx_ptr,
                                       const i64* rx_idx, const double* rx_w, const double* wav,
                                       const double* sponge, const double* dobs, double* grad, int kck) {
    return usct_oracle_misfit_and_gradient_mt(m, dims, ndim, h, dt, nt, n_tx, tx_ptr, tx_idx, tx_w,
                                              nrx, rx_ptr, rx_idx, rx_w, wav, sponge, dobs, grad,
                                              kck, 0);
}

double usct_oracle_misfit_and_gradient_tw(const double* m, const int* dims, int ndim, double h,
                                          double dt, int nt, int n_tx, const int* tx_ptr,
                                          const i64* tx_idx, const double* tx_w, int nrx,
                                          const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                          const double* wav, const double* sponge, const double* dobs,
                                          const double* tw, double* grad, int kck, int misfit_type);

/* misfit_type 0 = L2, 1 = GCN (libuap.hpp:169, misfit_type). */
double usct_oracle_misfit_and_gradient_mt(const double* m, const int* dims, int ndim, double h,
                                          double dt, int nt, int n_tx, const int* tx_ptr,
                                          const i64* tx_idx, const double* tx_w, int nrx,
                                          const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                          const double* wav, const double* sponge, const double* dobs,
                                          double* grad, int kck, int misfit_type) {
    return usct_oracle_misfit_and_gradient_tw(m, dims, ndim, h, dt, nt, n_tx, tx_ptr, tx_idx, tx_w,
                                              nrx, rx_ptr, rx_idx, rx_w, wav, sponge, dobs, NULL,
                                              grad, kck, misfit_type);
}

/* With per-transmit data windows tw[t][n][j] (NULL = none), fwi.py:298-301:
 * the misfit of (dsyn W, dobs W), adjoint source multiplied by W. */
double usct_oracle_misfit_and_gradient_tw(const double* m, const int* dims, int ndim, double h,
                                          double dt, int nt, int n_tx, const int* tx_ptr,
                                          const i64* tx_idx, const double* tx_w, int nrx,
                                          const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                          const double* wav, const double* sponge, const double* dobs,
                                          const double* tw, double* grad, int kck, int misfit_type) {
    G64 g; double* S;
    setup64(&g, m, dims, ndim, h, dt, nt, wav, sponge, nrx, rx_ptr, rx_idx, rx_w, &S);
    const size_t N = g.N;
    for (size_t i = 0; i < N; ++i) grad[i] = 0.0;
    double* dsyn = (double*)malloc((size_t)nt * nrx * sizeof(double));
    double* res = (double*)malloc((size_t)nt * nrx * sizeof(double));
    double* hist = kck ? NULL : (double*)malloc((size_t)nt * N * sizeof(double));
    double* ck = kck ? (double*)malloc((size_t)nseg_of(nt, kck) * 2 * N * sizeof(double)) : NULL;
    const size_t nd = (size_t)nt * nrx;
    double* wob = tw ? (double*)malloc(nd * sizeof(double)) : NULL;
    double J = 0.0;
    for (int t = 0; t < n_tx; ++t) {
        const int ns = tx_ptr[t + 1] - tx_ptr[t];
        forward64(&g, ns, tx_idx + tx_ptr[t], tx_w + tx_ptr[t], dsyn, hist, kck, ck);
        const double* ob = dobs + (size_t)t * nd;
        const double* W = tw ? tw + (size_t)t * nd : NULL;
        if (W) {
            for (size_t q = 0; q < nd; ++q) {
                dsyn[q] *= W[q];
                wob[q] = ob[q] * W[q];
            }
            ob = wob;
        }
        if (misfit_type == 1)
            J += residual64_gcn(dsyn, ob, nt, nrx, res);
        else
            J += residual64(dsyn, ob, nd, res);
        if (W)
            for (size_t q = 0; q < nd; ++q) res[q] *= W[q];
        backward64(&g, ns, tx_idx + tx_ptr[t], tx_w + tx_ptr[t], res, hist, kck, ck, grad);
    }
    for (size_t i = 0; i < N; ++i) grad[i] /= m[i];
    free(S); free(dsyn); free(res); free(hist); free(ck); free(wob);
    return J;
}

/* Born forward in lockstep with the background (fwi.py:350-379):
 *   dp^n = 2dp^{n-1} - dp^{n-2} + S L dp^{n-1} - (v/m)(U^n - 2U^{n-1} + U^{n-2});
 * Born traces dd (nt*nrx); checkpoints of U for the adjoint as in forward64. */
static void born64(const G64* g, const double* vm, int ns, const i64* s_idx, const double* s_w,
                   double* dd, int k, double* ck) {
    const size_t N = g->N;
    const i64 Nll = (i64)N;
    double* u[3]; double* d[3];
    for (int q = 0; q < 3; ++q) { u[q] = (double*)calloc(N, sizeof(double)); d[q] = (double*)calloc(N, sizeof(double)); }
    double* lap = (double*)calloc(N, sizeof(double));
    double *up = u[0], *uc = u[1], *un = u[2], *dp = d[0], *dc = d[1], *dn = d[2];
    memset(dd, 0, (size_t)g->nrx * sizeof(double));
    memset(ck, 0, (size_t)nseg_of(g->nt, k) * 2 * N * sizeof(double));
    for (int n = 1; n < g->nt; ++n) {
        step64(g, up, uc, un, lap, n, ns, s_idx, s_w);
        lap64(dc, lap, g->dims, g->ndim, g->inv_h2);
        #pragma omp parallel for schedule(static)
        for (i64 i = 0; i < Nll; ++i) {
            double d2U = un[i] - 2.0 * uc[i] + up[i];
            dn[i] = 2.0 * dc[i] - dp[i] + g->S[i] * lap[i] - vm[i] * d2U;
        }
        if (g->sponge) {
            #pragma omp parallel for schedule(static)
            for (i64 i = 0; i < Nll; ++i) dn[i] *= g->sponge[i];
        }
        double* t = up; up = uc; uc = un; un = t;
        t = dp; dp = dc; dc = dn; dn = t;
        sample64(g, dc, dd + (size_t)n * g->nrx);
        if ((n + 1) % k == 0 && n + 1 < g->nt - 1) memcpy(ck + (size_t)((n + 1) / k) * 2 * N, uc, N * sizeof(double));
        if (n % k == 0 && n < g->nt - 1) memcpy(ck + ((size_t)(n / k) * 2 + 1) * N, uc, N * sizeof(double));
    }
    for (int q = 0; q < 3; ++q) { free(u[q]); free(d[q]); }
    free(lap);
}

/* Gauss-Newton Hessian-vector product (fwi.py:410-431): out = sum_t J_t^T J_t v,
 * each transmit's adjoint result divided by m before the sum (fwi.py:407). */
int usct_oracle_gn_hessian_vector(const double* m, const int* dims, int ndim, double h, double dt,
                                  int nt, int n_tx, const int* tx_ptr, const i64* tx_idx,
                                  const double* tx_w, int nrx, const int* rx_ptr, const i64* rx_idx,
                                  const double* rx_w, const double* wav, const double* sponge,
                                  const double* v, double* out, double* born_out, int kck) {
    G64 g; double* S;
    setup64(&g, m, dims, ndim, h, dt, nt, wav, sponge, nrx, rx_ptr, rx_idx, rx_w, &S);
    const size_t N = g.N;
    if (kck <= 0) kck = 32;
    double* vm = (double*)malloc(N * sizeof(double));
    for (size_t i = 0; i < N; ++i) vm[i] = v[i] / m[i];
    double* dd = (double*)malloc((size_t)nt * nrx * sizeof(double));
    double* ck = (double*)malloc((size_t)nseg_of(nt, kck) * 2 * N * sizeof(double));
    double* gs = (double*)malloc(N * sizeof(double));
    for (size_t i = 0; i < N; ++i) out[i] = 0.0;
    for (int t = 0; t < n_tx; ++t) {
        const int ns = tx_ptr[t + 1] - tx_ptr[t];
        born64(&g, vm, ns, tx_idx + tx_ptr[t], tx_w + tx_ptr[t], dd, kck, ck);
        if (born_out) memcpy(born_out + (size_t)t * nt * nrx, dd, (size_t)nt * nrx * sizeof(double));
        for (size_t i = 0; i < N; ++i) gs[i] = 0.0;
        backward64(&g, ns, tx_idx + tx_ptr[t], tx_w + tx_ptr[t], dd, NULL, kck, ck, gs);
        for (size_t i = 0; i < N; ++i) out[i] += gs[i] / m[i];
    }
    free(S); free(vm); free(dd); free(ck); free(gs);
    return 0;
}

/* Timing hook for the CPU baseline: nsteps forward leapfrog steps of one
 * transmit (no receivers), so a bounded sample of a large workload can be
 * timed and scaled. */
int usct_oracle_forward_steps(const double* m, const int* dims, int ndim, double h, double dt,
                              int nsteps, int ns, const i64* s_idx, const double* s_w,
                              const double* wav, double* p_out) {
    G64 g; double* S;
    setup64(&g, m, dims, ndim, h, dt, nsteps + 1, wav, NULL, 0, NULL, NULL, NULL, &S);
    const size_t N = g.N;
    double* a = (double*)calloc(N, sizeof(double));
    double* b = (double*)calloc(N, sizeof(double));
    double* c = (double*)calloc(N, sizeof(double));
    double* lap = (double*)calloc(N, sizeof(double));
    double *pp = a, *pc = b, *pn = c;
    for (int n = 1; n <= nsteps; ++n) {
        step64(&g, pp, pc, pn, lap, n, ns, s_idx, s_w);
        double* t = pp; pp = pc; pc = pn; pn = t;
    }
    if (p_out) memcpy(p_out, pc, N * sizeof(double));
    free(a); free(b); free(c); free(lap); free(S);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* FP32 restatement in the CUDA kernels' operation order                     */
/* ------------------------------------------------------------------------- */
/*
 * Per cell (interior = not on the one-cell border of any axis), with c the
 * centre value and the marching axis being z in 3D and y in 2D:
 *   forward:  t   = (x- + x+) [+ (y- + y+) in 3D] + (m- + m+)
 *             lap = fmaf(-2*ndim, c, t) * inv_h2          (0 on the border)
 *             lap = lap + w*wav   for each source entry on (cell, shot)
 *             pn  = fmaf(S, lap, 2c - pp);  pn = pn*sponge
 *             d2p = (pn - 2c) + pp
 *   receiver entry (cell, j, w): slot sample w*pn; trace_j = 0 + s_1 + s_2 ...
 *   residual: r = dsyn - (float)dobs
 *   adjoint:  q = S*l1 at every cell of the stencil
 *             lk = (2*l1 - l2) + fmaf(-2*ndim, q_c, tq) * inv_h2;  lk *= sponge
 *             lk = lk - r_j*w  for each receiver entry on the cell, in j order
 *             per cell: sum over the C shot channels of lk*d2p with the
 *             reduction tree below, then g += (double)sum
 *   Born:     t1 = fmaf(S, L dpc, 2dc - dpp);  dpn = fmaf(-vm, d2U, t1); *sponge
 * Shot channel tree for a batch of C channels: C == 1: v0; C == 2: v0 + v1;
 * C >= 4: groups of four (v0+v1)+(v2+v3), then a pairwise tree over groups.
 */

typedef struct {
    int ndim, nz, ny, nx;   /* 2D: nz = ny_grid, ny = 1 (the marching axis is the slowest) */
    size_t N;
    float inv_h2;
    int nt;
    float* S;
    float* sp;              /* NULL = none */
    float* wav;
    int nrx;
    const int* rx_ptr;
    const i64* rx_idx;
    float* rx_w;
} G32;

static int interior32(const G32* g, size_t i) {
    const int ix = (int)(i % (size_t)g->nx);
    const size_t r = i / (size_t)g->nx;
    const int iy = (int)(r % (size_t)g->ny);
    const int iz = (int)(r / (size_t)g->ny);
    if (ix < 1 || ix > g->nx - 2 || iz < 1 || iz > g->nz - 2) return 0;
    if (g->ndim == 3 && (iy < 1 || iy > g->ny - 2)) return 0;
    return 1;
}

/* stencil sum t for field f at interior cell i, kernel order */
static float tsum32(const G32* g, const float* f, size_t i) {
    const size_t sx = 1, sy = (size_t)g->nx, sz = (size_t)g->nx * g->ny;
    float t = f[i - sx] + f[i + sx];
    if (g->ndim == 3) t = t + (f[i - sy] + f[i + sy]);
    t = t + (f[i - sz] + f[i + sz]);
    return t;
}

static void step32(const G32* g, const float* pp, const float* pc, float* pn, float* d2p,
                   int n, int ns, const i64* s_idx, const float* s_w) {
    const i64 N = (i64)g->N;
    const float cen = -2.0f * (float)g->ndim;
    const float wv = g->wav[n - 1];
    #pragma omp parallel for schedule(static)
    for (i64 i = 0; i < N; ++i) {
        const float c = pc[i];
        float lap = 0.0f;
        if (interior32(g, (size_t)i)) lap = fmaf(cen, c, tsum32(g, pc, (size_t)i)) * g->inv_h2;
        for (int e = 0; e < ns; ++e)
            if (s_idx[e] == i) lap = lap + s_w[e] * wv;
        float v = fmaf(g->S[i], lap, 2.0f * c - pp[i]);
        if (g->sp) v = v * g->sp[i];
        if (d2p) d2p[i] = (v - 2.0f * c) + pp[i];
        pn[i] = v;
    }
}

static void sample32(const G32* g, const float* p, float* row) {
    for (int j = 0; j < g->nrx; ++j) {
        float acc = 0.0f;
        for (int e = g->rx_ptr[j]; e < g->rx_ptr[j + 1]; ++e) acc = acc + g->rx_w[e] * p[g->rx_idx[e]];
        row[j] = acc;
    }
}

/* pairwise tree over n values (n a power of two), left-to-right pairing */
static float tree32(const float* v, int n) {
    if (n == 1) return v[0];
    float tmp[64];
    int m = n;
    for (int q = 0; q < m; ++q) tmp[q] = v[q];
    while (m > 1) {
        for (int q = 0; q < m / 2; ++q) tmp[q] = tmp[2 * q] + tmp[2 * q + 1];
        m /= 2;
    }
    return tmp[0];
}

static float chansum32(const float* v, int C) {
    if (C == 1) return v[0];
    if (C == 2) return v[0] + v[1];
    float grp[64];
    const int ng = C / 4;
    for (int q = 0; q < ng; ++q) grp[q] = (v[4 * q] + v[4 * q + 1]) + (v[4 * q + 2] + v[4 * q + 3]);
    return tree32(grp, ng);
}

static void setup32(G32* g, const double* m, const int* dims, int ndim, double h, double dt, int nt,
                    const double* wav, const double* sponge, int nrx, const int* rx_ptr,
                    const i64* rx_idx, const double* rx_w) {
    g->ndim = ndim;
    if (ndim == 3) { g->nz = dims[0]; g->ny = dims[1]; g->nx = dims[2]; }
    else { g->nz = dims[0]; g->ny = 1; g->nx = dims[1]; }
    g->N = cell_count(dims, ndim);
    g->inv_h2 = (float)(1.0 / (h * h));
    g->nt = nt;
    const double dt2 = dt * dt;
    g->S = (float*)malloc(g->N * sizeof(float));
    for (size_t i = 0; i < g->N; ++i) g->S[i] = (float)(dt2 / m[i]);
    g->sp = NULL;
    if (sponge) {
        g->sp = (float*)malloc(g->N * sizeof(float));
        for (size_t i = 0; i < g->N; ++i) g->sp[i] = (float)sponge[i];
    }
    g->wav = (float*)malloc((size_t)nt * sizeof(float));
    for (int q = 0; q < nt; ++q) g->wav[q] = (float)wav[q];
    g->nrx = nrx; g->rx_ptr = rx_ptr; g->rx_idx = rx_idx;
    const int ne = rx_ptr[nrx];
    g->rx_w = (float*)malloc((size_t)(ne > 0 ? ne : 1) * sizeof(float));
    for (int e = 0; e < ne; ++e) g->rx_w[e] = (float)rx_w[e];
}

static void free32(G32* g) { free(g->S); free(g->sp); free(g->wav); free(g->rx_w); }

static float* srcw32(const double* w, int ns) {
    float* o = (float*)malloc((size_t)(ns > 0 ? ns : 1) * sizeof(float));
    for (int e = 0; e < ns; ++e) o[e] = (float)w[e];
    return o;
}

/* forward FMC in FP32 kernel order: data (n_tx, nt, nrx) float32. */
int usct_oracle32_forward_fmc(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                              int n_tx, const int* tx_ptr, const i64* tx_idx, const double* tx_w,
                              int nrx, const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                              const double* wav, const double* sponge, float* data) {
    G32 g;
    setup32(&g, m, dims, ndim, h, dt, nt, wav, sponge, nrx, rx_ptr, rx_idx, rx_w);
    const size_t N = g.N;
    float* a = (float*)calloc(N, sizeof(float));
    float* b = (float*)calloc(N, sizeof(float));
    for (int t = 0; t < n_tx; ++t) {
        const int ns = tx_ptr[t + 1] - tx_ptr[t];
        float* sw = srcw32(tx_w + tx_ptr[t], ns);
        memset(a, 0, N * sizeof(float)); memset(b, 0, N * sizeof(float));
        float* rec = data + (size_t)t * nt * nrx;
        memset(rec, 0, (size_t)nrx * sizeof(float));
        float *pp = a, *pc = b;
        for (int n = 1; n < nt; ++n) {
            step32(&g, pp, pc, pp, NULL, n, ns, tx_idx + tx_ptr[t], sw);  /* in place over pp */
            float* tt = pp; pp = pc; pc = tt;
            sample32(&g, pc, rec + (size_t)n * nrx);
        }
        free(sw);
    }
    free(a); free(b); free32(&g);
    return 0;
}

/* Gradient in FP32 kernel order, shots processed in batches of C channels
 * (shot t -> batch t / C, channel t % C); full-history d2p per shot (the GPU's
 * checkpoint recompute reproduces it bit for bit).  J_out gets the per-shot
 * misfit in double; grad gets g / m in double.  born_v != NULL turns this into
 * the Gauss-Newton product: the adjoint source is the Born data of v and the
 * result is sum_t g_t / m. */
static int grad32_impl(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                       int n_tx, const int* tx_ptr, const i64* tx_idx, const double* tx_w,
                       int nrx, const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                       const double* wav, const double* sponge, const double* dobs, int C,
                       double* J_out, double* grad, const double* born_v, float* born_out,
                       int misfit_type, const double* tw) {
    G32 g;
    setup32(&g, m, dims, ndim, h, dt, nt, wav, sponge, nrx, rx_ptr, rx_idx, rx_w);
    const size_t N = g.N;
    const i64 Nll = (i64)N;
    const float cen = -2.0f * (float)ndim;
    double* gacc = (double*)calloc(N, sizeof(double));
    float* vm = NULL;
    if (born_v) {
        vm = (float*)malloc(N * sizeof(float));
        for (size_t i = 0; i < N; ++i) vm[i] = (float)(born_v[i] / m[i]);
    }
    /* per-channel state for one batch */
    float** d2 = (float**)calloc((size_t)C, sizeof(float*));
    float** l1 = (float**)calloc((size_t)C, sizeof(float*));
    float** l2 = (float**)calloc((size_t)C, sizeof(float*));
    float** res = (float**)calloc((size_t)C, sizeof(float*));
    for (int c = 0; c < C; ++c) {
        d2[c] = (float*)malloc((size_t)nt * N * sizeof(float));
        l1[c] = (float*)malloc(N * sizeof(float));
        l2[c] = (float*)malloc(N * sizeof(float));
        res[c] = (float*)malloc((size_t)nt * nrx * sizeof(float));
    }
    float* pa = (float*)malloc(N * sizeof(float));
    float* pb = (float*)malloc(N * sizeof(float));
    float* da = (float*)malloc(N * sizeof(float));
    float* db = (float*)malloc(N * sizeof(float));
    float* lk = (float*)malloc((size_t)C * N * sizeof(float));
    float* q = (float*)malloc(N * sizeof(float));
    float* dsyn = (float*)malloc((size_t)nt * nrx * sizeof(float));
    for (int b0 = 0; b0 < n_tx; b0 += C) {
        const int nb = (n_tx - b0 < C) ? n_tx - b0 : C;
        for (int c = 0; c < C; ++c) {
            memset(d2[c], 0, (size_t)nt * N * sizeof(float));
            memset(res[c], 0, (size_t)nt * nrx * sizeof(float));
            memset(l1[c], 0, N * sizeof(float));
            memset(l2[c], 0, N * sizeof(float));
        }
        for (int c = 0; c < nb; ++c) {
            const int t = b0 + c;
            const int ns = tx_ptr[t + 1] - tx_ptr[t];
            float* sw = srcw32(tx_w + tx_ptr[t], ns);
            memset(pa, 0, N * sizeof(float)); memset(pb, 0, N * sizeof(float));
            memset(da, 0, N * sizeof(float)); memset(db, 0, N * sizeof(float));
            memset(dsyn, 0, (size_t)nrx * sizeof(float));
            float *pp = pa, *pc = pb, *dp = da, *dc = db;
            for (int n = 1; n < nt; ++n) {
                float* d2n = d2[c] + (size_t)n * N;
                if (!born_v) {
                    step32(&g, pp, pc, pp, d2n, n, ns, tx_idx + tx_ptr[t], sw);
                    float* tt = pp; pp = pc; pc = tt;
                    sample32(&g, pc, dsyn + (size_t)n * nrx);
                } else {
                    /* background step (d2U into the stash) fused with the Born step */
                    const float wv = g.wav[n - 1];
                    #pragma omp parallel for schedule(static)
                    for (i64 i = 0; i < Nll; ++i) {
                        const float c0 = pc[i], dc0 = dc[i];
                        float lap = 0.0f, dl = 0.0f;
                        if (interior32(&g, (size_t)i)) {
                            lap = fmaf(cen, c0, tsum32(&g, pc, (size_t)i)) * g.inv_h2;
                            dl = fmaf(cen, dc0, tsum32(&g, dc, (size_t)i)) * g.inv_h2;
                        }
                        for (int e = 0; e < ns; ++e)
                            if (tx_idx[tx_ptr[t] + e] == i) lap = lap + sw[e] * wv;
                        float v = fmaf(g.S[i], lap, 2.0f * c0 - pp[i]);
                        if (g.sp) v = v * g.sp[i];
                        const float d2u = (v - 2.0f * c0) + pp[i];
                        float dv = fmaf(g.S[i], dl, 2.0f * dc0 - dp[i]);
                        dv = fmaf(-vm[i], d2u, dv);
                        if (g.sp) dv = dv * g.sp[i];
                        d2n[i] = d2u;
                        q[i] = dv;     /* staged so the in-place writes do not race the stencil */
                        lk[i] = v;
                    }
                    memcpy(pp, lk, N * sizeof(float));
                    memcpy(dp, q, N * sizeof(float));
                    float* tt = pp; pp = pc; pc = tt;
                    tt = dp; dp = dc; dc = tt;
                    sample32(&g, dc, dsyn + (size_t)n * nrx);
                }
            }
            /* adjoint source */
            /* windows as the device applies them: FP32 products with the FP32 window */
            const double* W = tw ? tw + (size_t)t * nt * nrx : NULL;
            if (!born_v && misfit_type == 1) {
                /* GCN as the device computes it (k_gcn): per receiver, FP64 sums over
                 * time of the FP32 traces, each with fused multiply-adds over KGS
                 * contiguous time slices and the slices added in order;
                 * c_j = sum sv*ov / (sn*on); adj = a*ov + b*sv with a = -1/(on*sn),
                 * b = c_j/(sn*sn) (the reference's -(ov/on - c_j*sv/sn)/sn);
                 * J = sum_j (1 - c_j) in j order */
                const double* ob = dobs + (size_t)t * nt * nrx;
                if (W)
                    for (size_t z = 0; z < (size_t)nt * nrx; ++z) dsyn[z] = dsyn[z] * (float)W[z];
#define OBS(z) (W ? (double)((float)ob[(z)] * (float)W[(z)]) : (double)(float)ob[(z)])
                const double eps = 1e-12;
                const int KGS = 8;
                const int L = (nt + KGS - 1) / KGS;
                double J = 0.0;
                for (int j = 0; j < nrx; ++j) {
                    double S = 0.0, O = 0.0, D = 0.0;
                    for (int q = 0; q < KGS; ++q) {
                        const int n0 = q * L < nt ? q * L : nt;
                        const int n1 = n0 + L < nt ? n0 + L : nt;
                        double ss = 0.0, oo = 0.0, so = 0.0;
                        for (int n = n0; n < n1; ++n) {
                            const double sv = (double)dsyn[(size_t)n * nrx + j];
                            const double ov = OBS((size_t)n * nrx + j);
                            ss = fma(sv, sv, ss);
                            oo = fma(ov, ov, oo);
                            so = fma(sv, ov, so);
                        }
                        S += ss;
                        O += oo;
                        D += so;
                    }
                    const double sn = sqrt(S) + eps, on = sqrt(O) + eps;
                    const double cc = D / (sn * on);
                    const double A = -1.0 / (on * sn), B = cc / (sn * sn);
                    for (int n = 0; n < nt; ++n) {
                        const size_t z = (size_t)n * nrx + j;
                        const double sv = (double)dsyn[z];
                        const float adj = (float)fma(A, OBS(z), B * sv);
                        res[c][z] = W ? adj * (float)W[z] : adj;
                    }
                    J += 1.0 - cc;
                }
#undef OBS
                if (J_out) J_out[t] = J;
            } else if (!born_v) {
                const double* ob = dobs + (size_t)t * nt * nrx;
                double J = 0.0;
                for (size_t z = 0; z < (size_t)nt * nrx; ++z) {
                    if (W) {
                        const float wv = (float)W[z];
                        const float r = dsyn[z] * wv - (float)ob[z] * wv;
                        res[c][z] = r * wv;
                        J += 0.5 * (double)r * (double)r;
                    } else {
                        const float r = dsyn[z] - (float)ob[z];
                        res[c][z] = r;
                        J += 0.5 * (double)r * (double)r;
                    }
                }
                if (J_out) J_out[t] = J;
            } else {
                memcpy(res[c], dsyn, (size_t)nt * nrx * sizeof(float));
                if (born_out) memcpy(born_out + (size_t)t * nt * nrx, dsyn, (size_t)nt * nrx * sizeof(float));
            }
            free(sw);
        }
        /* backward over the batch */
        for (int k = nt - 1; k >= 1; --k) {
            for (int c = 0; c < C; ++c) {
                const float* L1 = l1[c];
                const float* L2 = l2[c];
                float* LK = lk + (size_t)c * N;
                #pragma omp parallel for schedule(static)
                for (i64 i = 0; i < Nll; ++i) q[i] = g.S[i] * L1[i];
                #pragma omp parallel for schedule(static)
                for (i64 i = 0; i < Nll; ++i) {
                    float lapq = 0.0f;
                    if (interior32(&g, (size_t)i)) lapq = fmaf(cen, q[i], tsum32(&g, q, (size_t)i)) * g.inv_h2;
                    float v = (2.0f * L1[i] - L2[i]) + lapq;
                    if (g.sp) v = v * g.sp[i];
                    LK[i] = v;
                }
                const float* rrow = res[c] + (size_t)k * nrx;
                /* on any one cell the entries land in ascending j, as in the kernels */
                for (int j = 0; j < nrx; ++j)
                    for (int e = rx_ptr[j]; e < rx_ptr[j + 1]; ++e) {
                        const i64 cell = rx_idx[e];
                        LK[cell] = LK[cell] - rrow[j] * g.rx_w[e];
                    }
            }
            #pragma omp parallel for schedule(static)
            for (i64 i = 0; i < Nll; ++i) {
                float v[64];
                for (int c = 0; c < C; ++c) v[c] = lk[(size_t)c * N + i] * d2[c][(size_t)k * N + i];
                gacc[i] += (double)chansum32(v, C);
            }
            for (int c = 0; c < C; ++c) {
                float* t2 = l2[c];
                l2[c] = l1[c];
                memcpy(t2, lk + (size_t)c * N, N * sizeof(float));
                l1[c] = t2;
            }
        }
    }
    for (size_t i = 0; i < N; ++i) grad[i] = gacc[i] / m[i];
    for (int c = 0; c < C; ++c) { free(d2[c]); free(l1[c]); free(l2[c]); free(res[c]); }
    free(d2); free(l1); free(l2); free(res);
    free(pa); free(pb); free(da); free(db); free(lk); free(q); free(dsyn); free(gacc); free(vm);
    free32(&g);
    return 0;
}

int usct_oracle32_misfit_and_gradient(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                                      int n_tx, const int* tx_ptr, const i64* tx_idx, const double* tx_w,
                                      int nrx, const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                      const double* wav, const double* sponge, const double* dobs, int C,
                                      double* J_out, double* grad) {
    if (C < 1 || C > 64 || (C & (C - 1))) return -1;
    return grad32_impl(m, dims, ndim, h, dt, nt, n_tx, tx_ptr, tx_idx, tx_w, nrx, rx_ptr, rx_idx,
                       rx_w, wav, sponge, dobs, C, J_out, grad, NULL, NULL, 0, NULL);
}

int usct_oracle32_misfit_and_gradient_mt(const double* m, const int* dims, int ndim, double h,
                                         double dt, int nt, int n_tx, const int* tx_ptr,
                                         const i64* tx_idx, const double* tx_w, int nrx,
                                         const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                         const double* wav, const double* sponge, const double* dobs,
                                         int C, double* J_out, double* grad, int misfit_type) {
    if (C < 1 || C > 64 || (C & (C - 1))) return -1;
    return grad32_impl(m, dims, ndim, h, dt, nt, n_tx, tx_ptr, tx_idx, tx_w, nrx, rx_ptr, rx_idx,
                       rx_w, wav, sponge, dobs, C, J_out, grad, NULL, NULL, misfit_type, NULL);
}

int usct_oracle32_misfit_and_gradient_tw(const double* m, const int* dims, int ndim, double h,
                                         double dt, int nt, int n_tx, const int* tx_ptr,
                                         const i64* tx_idx, const double* tx_w, int nrx,
                                         const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                         const double* wav, const double* sponge, const double* dobs,
                                         const double* tw, int C, double* J_out, double* grad,
                                         int misfit_type) {
    if (C < 1 || C > 64 || (C & (C - 1))) return -1;
    return grad32_impl(m, dims, ndim, h, dt, nt, n_tx, tx_ptr, tx_idx, tx_w, nrx, rx_ptr, rx_idx,
                       rx_w, wav, sponge, dobs, C, J_out, grad, NULL, NULL, misfit_type, tw);
}

int usct_oracle32_gn_hessian_vector(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                                    int n_tx, const int* tx_ptr, const i64* tx_idx, const double* tx_w,
                                    int nrx, const int* rx_ptr, const i64* rx_idx, const double* rx_w,
                                    const double* wav, const double* sponge, const double* v, int C,
                                    double* out, float* born_out) {
    if (C < 1 || C > 64 || (C & (C - 1))) return -1;
    return grad32_impl(m, dims, ndim, h, dt, nt, n_tx, tx_ptr, tx_idx, tx_w, nrx, rx_ptr, rx_idx,
                       rx_w, wav, sponge, NULL, C, NULL, out, v, born_out, 0, NULL);
}
