/*
 * usct_gb300.h -- C ABI of the GB300 acoustic FWI hot path (libusct_gb300.so).
 *
 * The library is a drop-in for the reference's acoustic wave-propagation core:
 * the leapfrog forward solve, its exact discrete adjoint and the
 * squared-slowness gradient, run over every transmit of a full-matrix capture.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   uap::forward_fmc          software/core/libuap.hpp:109-116
 *   uap::misfit_and_gradient  software/core/libuap.hpp:169-224  (L2 misfit)
 *   _uap.forward_fmc / _uap.misfit_and_gradient
 *                             software/python/_uap.cpp:25-55   (pybind layer)
 *   fwi.forward_fmc / misfit / misfit_and_gradient / gn_hessian_vector
 *                             simulation/ringfwi/fwi.py:102,246,266,410
 *                             (footprints, sponge and Born are only there)
 *   uap_gpu.forward_fmc / misfit_and_gradient
 *                             software/python/uap_gpu.py:166-224 (CuPy FP32)
 *
 * Numerics: FP32 wavefields and traces, FP64 model input, FP64 gradient
 * accumulation and output.  Grids are row-major ([iy][ix] or [iz][iy][ix]),
 * cells are addressed by row-major linear index, exactly as the reference's
 * linear_indices (software/python/uap.py:19-22).  Sources and receivers are CSR
 * lists of (cell, weight); a point element is one entry of weight 1, a
 * finite-aperture footprint (simulation/ringfwi/geometry.py:212-278) is its
 * cell list with weights 1/len.
 *
 * Every function returns 0 on success or a USCT_ERR_* code; usct_last_error()
 * gives a one-line message for the calling thread.  Nothing here falls back to
 * the CPU: without a CUDA device the calls fail with USCT_ERR_CUDA.
 *
 * Device entry points take device pointers and a CUDA stream (a cudaStream_t
 * passed as void*; NULL = legacy default stream) and are asynchronous with
 * respect to the host unless stated.  Scratch memory is caller-provided
 * ("workspaces"), sized by the *_bytes queries, so callers keep control of
 * HBM (the serving engine admits requests against these sizes).
 *
 * Threads: different plans may be used concurrently (from any threads and
 * streams); calls on one plan, or on one workspace, must not overlap -- a plan
 * holds its captured graphs and tensor-map cache.  The host-pointer entry
 * points create a private plan per call and are reentrant, like the
 * reference's core.
 */
#ifndef USCT_GB300_H
#define USCT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define USCT_OK 0
#define USCT_ERR_ARG 1      /* invalid argument (shape, index out of grid, ...) */
#define USCT_ERR_CUDA 2     /* CUDA runtime error (message has the CUDA string) */
#define USCT_ERR_NOMEM 3    /* device allocation failed or workspace too small */
#define USCT_ERR_STATE 4    /* call out of order (e.g. backward before forward) */

/* Workspace modes for usct_batch_bytes / usct_batch_forward. */
#define USCT_MODE_FORWARD 0   /* traces only */
#define USCT_MODE_GRADIENT 1  /* traces + checkpoints + stash + adjoint fields */
#define USCT_MODE_BORN 2      /* GRADIENT + the Born perturbation fields */

/* usct_plan_info keys */
#define USCT_INFO_BATCH 0        /* shot channels per batch C (power of two) */
#define USCT_INFO_NBATCH 1       /* number of batches = ceil(n_tx / C) */
#define USCT_INFO_CKPT_K 2       /* checkpoint interval k */
#define USCT_INFO_NSEG 3         /* checkpoint segments ceil((nt-1)/k) */
#define USCT_INFO_TILE_X 4       /* threads along the row (float4 each) */
#define USCT_INFO_TILE_Y 5       /* rows per tile */
#define USCT_INFO_ZCHUNK 6       /* planes marched per CTA */
#define USCT_INFO_LEVEL_FLOATS 7 /* floats in one batched wavefield level */
#define USCT_INFO_LAUNCHES 8     /* kernels launched by this plan so far */
#define USCT_INFO_VARIANT 9      /* 0 = register-queue stencils, 1 = TMA ring */
#define USCT_INFO_TBLOCK 10      /* two-step tile W*100+H of the forward sweeps, 0 = off */

/* usct_plan_set keys */
#define USCT_SET_VARIANT 0       /* 0 = register-queue stencils, 1 = TMA-fed ring */
#define USCT_SET_STAGES 1        /* planes in the forward TMA ring (3..8; Born uses one fewer) */
#define USCT_SET_STAGES_ADJ 2    /* planes in the adjoint TMA ring (3..8) */
#define USCT_SET_GRAPHS 3        /* 1 = capture each batch sweep as a CUDA graph on first
                                    use (per stream/buffer set) and replay it afterwards */
#define USCT_SET_WAIT_TEST 4     /* test hook: 1 = the TMA ring's first stage expects bytes
                                    that never arrive, so its bounded wait gives up and the
                                    error is reported by usct_plan_check (no fault) */
#define USCT_SET_TBLOCK 5        /* forward sweeps (not Born) two time levels per launch:
                                    0 = off, 1 = the default tile for the batch width, or
                                    W*100+H (W, H in cells: 4x8, 8x4, 8x8, 16x4, 16x8); 3D
                                    TMA plans with >= 8 shot channels.  It adds two levels to
                                    usct_batch_bytes: set it before sizing workspaces */
#define USCT_SET_TBLOCK_STAGES 6 /* two-step rings: 10 * (p^{n-1} stages, 3..6) +
                                    (p^{n-2}/S stages, 2..5) */
#define USCT_SET_TBLOCK_ZCHUNK 7 /* planes per CTA of the two-step launches (0 = default) */


/* One-line message describing the last error on this thread ("" if none). */
const char* usct_last_error(void);

/* ABI version: major*10000 + minor*100 + patch. */
int usct_version(void);

/* ------------------------------------------------------------------------ */
/* Plans: grid, time axis, acquisition geometry and batching, built once.   */
/* ------------------------------------------------------------------------ */
typedef struct usct_plan usct_plan;

/*
 * Build a plan on the current CUDA device (device memory for the per-tile
 * source/receiver lists is allocated here and freed by usct_plan_destroy).
 *   ndim, dims     2 -> (ny, nx), 3 -> (nz, ny, nx); every extent >= 3
 *   h, dt, nt      grid spacing (m), time step (s), number of time levels
 *   n_tx, tx_ptr[n_tx+1], tx_cell[], tx_w[]   source CSR, one row per transmit
 *   n_rx, rx_ptr[n_rx+1], rx_cell[], rx_w[]   receiver CSR, one row per receiver
 *   batch          shot channels per launch (power of two <= 64; 0 = choose)
 *   ckpt_k         checkpoint interval in steps (0 = choose)
 *   tile_x, tile_y, zchunk   launch shape (0 = choose); tile_x in {16,32,64,128,256}
 * Host arrays; cells are row-major linear indices into the grid.
 */
int usct_plan_create(usct_plan** out, int ndim, const int* dims, double h, double dt, int nt,
                     int n_tx, const int* tx_ptr, const int64_t* tx_cell, const double* tx_w,
                     int n_rx, const int* rx_ptr, const int64_t* rx_cell, const double* rx_w,
                     int batch, int ckpt_k, int tile_x, int tile_y, int zchunk);
void usct_plan_destroy(usct_plan* plan);
int usct_plan_info(const usct_plan* plan, int key, int64_t* value);
/* Tuning knobs (USCT_SET_*): the stencil variant and the TMA ring depth.  The
 * default is the TMA ring wherever its box constraints hold. */
int usct_plan_set(usct_plan* plan, int key, int64_t value);
/* Synchronise the stream and report a pipelined stencil that gave up waiting
 * for its tensor copies (bounded waits; USCT_ERR_CUDA), then clear the flag. */
int usct_plan_check(usct_plan* plan, void* stream);

/* Per-channel models (no counterpart in the reference: its core runs one shot
 * at a time on one model).  Shots of several forward requests on different
 * models of the same grid, h, dt, nt and wavelet share one plan, so they
 * advance in one launch: transmit t uses model model_of_tx[t] (host array of
 * n_tx entries, each < n_models), and each group of four transmits
 * (4k .. 4k+3) must share one model (pad a request with transmits that have no
 * source entries to keep the groups whole).  Needs the TMA variant, >= 4 shot
 * channels, one level per launch, no sponge; forward sweeps only
 * (USCT_MODE_FORWARD).  Call before the plan's first sweep: it grows
 * usct_model_bytes by a quarter wavefield level per batch (S once per four
 * channels). */
int usct_plan_set_channel_models(usct_plan* plan, int n_models, const int* model_of_tx);
/* The per-channel model S from n_models device FP64 models [n_models][cells]
 * and the FP64 wavelet, for a plan with per-channel models. */
int usct_model_prepare_channels(usct_plan* plan, void* model_ws, const double* models,
                                const double* wavelet, void* stream);
/* Bytes of the model workspace (S, sponge, v/m, wavelet, FP64 gradient). */
size_t usct_model_bytes(const usct_plan* plan);
/* Bytes of one batch workspace for a USCT_MODE_*. */
size_t usct_batch_bytes(const usct_plan* plan, int mode);

/*
 * Load the model: S = dt^2/m (libuap.hpp:73, fwi.py:52), the optional sponge
 * mask (fwi.py:68, solver.py:22-42; NULL = none), the optional Born
 * perturbation v (fwi.py:358, NULL = none), the wavelet; zero the gradient.
 * m, sponge, v: device FP64, dims-shaped; wavelet: device FP64 [nt].
 */
int usct_model_prepare(usct_plan* plan, void* model_ws, const double* m, const double* sponge,
                       const double* v, const double* wavelet, void* stream);

/*
 * Forward sweep of batch b (transmits b*C .. b*C+C-1) over all nt levels
 * (fwi.py:63-79, libuap.hpp:83-104), one launch per time step for all shots
 * of the batch.  traces (device FP32, user layout [n_tx][nt][n_rx], NULL = do
 * not export) receives this batch's rows.  USCT_MODE_GRADIENT stores
 * checkpoints for usct_batch_backward; USCT_MODE_BORN additionally runs the
 * exact Born linearisation (fwi.py:350-379) in lockstep and exports the Born
 * traces instead, keeping them as the adjoint source.
 */
int usct_batch_forward(usct_plan* plan, const void* model_ws, void* batch_ws, int b, int mode,
                       float* traces, void* stream);

/*
 * L2 adjoint source of batch b from the traces of its last forward sweep:
 * r = dsyn - dobs (libuap.hpp:125-132, fwi.py:155-157).  dobs: device FP32
 * [n_tx][nt][n_rx]; J: device FP64 [n_tx], receives 0.5*sum r^2 per transmit
 * of the batch (NULL = skip).
 */
int usct_batch_misfit(usct_plan* plan, void* batch_ws, int b, const float* dobs, double* J,
                      void* stream);

/*
 * Misfit of batch b with a selectable misfit: misfit_type 0 = L2 (as
 * usct_batch_misfit), 1 = global correlation norm, J = sum_j (1 - c_j) with
 * c_j the normalised zero-lag correlation of trace j and its adjoint source
 * -(dobs/|dobs| - c dsyn/|dsyn|)/|dsyn| (libuap.hpp:133-162, fwi.py:158-167;
 * norms and correlations summed in FP64).
 */
int usct_batch_misfit_mt(usct_plan* plan, void* batch_ws, int b, const float* dobs,
                         int misfit_type, double* J, void* stream);

/*
 * Misfit of batch b on windowed data (fwi.py:247-263, 298-301 time_weights):
 * weights is a device FP32 [n_tx][nt][n_rx] window (NULL = none, then this is
 * usct_batch_misfit_mt).  The misfit is taken between dsyn*W and dobs*W and
 * the adjoint source is multiplied by W again (the chain rule through the
 * window).  No counterpart in libuap, which has no windows; the Python
 * reference's time_weights[i] is row i of weights.
 */
int usct_batch_misfit_tw(usct_plan* plan, void* batch_ws, int b, const float* dobs,
                         const float* weights, int misfit_type, double* J, void* stream);

/* Use an arbitrary adjoint source for batch b (device FP32 [n_tx][nt][n_rx]),
 * e.g. dL/d(traces) from an autograd graph. */
int usct_batch_adjoint_source(usct_plan* plan, void* batch_ws, int b, const float* adj,
                              void* stream);

/*
 * Backward sweep of batch b (fwi.py:306-326, libuap.hpp:196-219): the exact
 * discrete adjoint driven by the current adjoint source, with each checkpoint
 * segment recomputed bit-identically from its stored levels, and the imaging
 * condition g += sum_shots lam^k * d2p^k accumulated in FP64 in model_ws.
 */
int usct_batch_backward(usct_plan* plan, void* model_ws, void* batch_ws, int b, void* stream);

/* grad = g / m (fwi.py:331, libuap.hpp:222) into device FP64 dims-shaped
 * grad; then zero the accumulator. */
int usct_model_gradient(usct_plan* plan, void* model_ws, const double* m, double* grad,
                        void* stream);

/* ---- whole-acquisition device calls (loop over batches, one workspace) ---- */

/* fwi.forward_fmc / uap::forward_fmc: data device FP32 [n_tx][nt][n_rx]. */
int usct_forward_fmc_dev(usct_plan* plan, const double* m, const double* sponge,
                         const double* wavelet, float* data, void* model_ws, void* batch_ws,
                         void* stream);
/* fwi.misfit_and_gradient (L2): J device FP64 [n_tx] per transmit, grad FP64. */
int usct_misfit_and_gradient_dev(usct_plan* plan, const double* m, const double* sponge,
                                 const double* wavelet, const float* dobs, double* J,
                                 double* grad, void* model_ws, void* batch_ws, void* stream);
/* misfit_and_gradient with misfit_type 0 (L2) or 1 (GCN), as uap::misfit_and_gradient's
 * misfit_type argument (libuap.hpp:169-173). */
int usct_misfit_and_gradient_mt_dev(usct_plan* plan, const double* m, const double* sponge,
                                    const double* wavelet, const float* dobs, int misfit_type,
                                    double* J, double* grad, void* model_ws, void* batch_ws,
                                    void* stream);
/* fwi.misfit_and_gradient with time_weights (fwi.py:266-301): weights device
 * FP32 [n_tx][nt][n_rx] (NULL = none, then this is the _mt call). */
int usct_misfit_and_gradient_tw_dev(usct_plan* plan, const double* m, const double* sponge,
                                    const double* wavelet, const float* dobs,
                                    const float* weights, int misfit_type, double* J,
                                    double* grad, void* model_ws, void* batch_ws, void* stream);
/* fwi.gn_hessian_vector: hv device FP64 dims-shaped; born (NULL = skip) FP32
 * [n_tx][nt][n_rx] receives J v. */
int usct_gn_hessian_vector_dev(usct_plan* plan, const double* m, const double* sponge,
                               const double* wavelet, const double* v, double* hv, float* born,
                               void* model_ws, void* batch_ws, void* stream);

/* ---- the plain one-shot-per-launch GPU form (the comparison baseline) ---- */
/*
 * A restatement of the reference's CuPy backend (software/python/uap_gpu.py:
 * 100-140): one thread per cell, separate launches per time step for the
 * stencil, source injection, receiver gather, history copy, adjoint step,
 * adjoint injection and imaging; the full FP32 history is kept in HBM.
 * Point elements only (as the reference's GPU backend).  It exists to measure
 * the batched engine against; it shares no kernel with it.
 */
size_t usct_plain_bytes(const usct_plan* plan, int gradient);
int usct_plain_forward_fmc_dev(usct_plan* plan, const double* m, const double* wavelet,
                               float* data, void* ws, void* stream);
int usct_plain_misfit_and_gradient_dev(usct_plan* plan, const double* m, const double* wavelet,
                                       const float* dobs, double* J, double* grad, void* ws,
                                       void* stream);

/* ---- host-pointer calls with the reference core's own signatures ---- */
/*
 * Same arguments and layouts as uap::forward_fmc (libuap.hpp:109) and
 * uap::misfit_and_gradient (libuap.hpp:169, misfit_type 0 only): host FP64
 * arrays in, host FP64 out; point elements tx_lin[n_tx], rec_lin[n_rec].
 * These allocate device memory for the duration of the call, copy in, run on
 * the legacy default stream and copy out (synchronous).
 */
int usct_forward_fmc(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                     const int* tx_lin, int n_tx, const int* rec_lin, int n_rec,
                     const double* wavelet, double* data);
int usct_misfit_and_gradient(const double* m, const int* dims, int ndim, double h, double dt,
                             int nt, const int* tx_lin, int n_tx, const int* rec_lin, int n_rec,
                             const double* wavelet, const double* dobs, double* grad, double* J);
/* The same with uap::misfit_and_gradient's misfit_type (0 = L2, 1 = GCN), in the
 * reference's argument position (libuap.hpp:169-173); J is returned through *J. */
int usct_misfit_and_gradient_mt(const double* m, const int* dims, int ndim, double h, double dt,
                                int nt, const int* tx_lin, int n_tx, const int* rec_lin,
                                int n_rec, const double* wavelet, const double* dobs, double* grad,
                                int misfit_type, double* J);

/* ---- a forward FMC that allocates no device memory ---- */
/*
 * No counterpart in the reference.  For callers that may not allocate device
 * memory -- a host that has reserved the GPU for its own pool allocator, a
 * plugin inside such a host, a real-time loop that must not enter the CUDA
 * allocator.  Same result as usct_forward_fmc_dev (point or footprint
 * elements, optional sponge), but it needs no plan and no workspace: all
 * scratch lives in one static device array of USCT_NOALLOC_SCRATCH_BYTES that
 * every GPU loading the library holds until exit; larger problems are
 * rejected with USCT_ERR_ARG.  It calls no cudaMalloc/cudaFree.
 *   dims/h/dt/nt and the CSR arrays: as usct_plan_create (host arrays)
 *   m, sponge (NULL = none), wavelet: device FP64; data: device FP32
 *   [n_tx][nt][n_rx], caller-allocated.
 * The first call on a device resolves the array's device address (with that
 * device current); make it before any stream capture.  The address is kept per
 * device and context, and resolved again when another context is current.
 * Each call uploads per-tile source/receiver lists from host memory local to
 * the call, so a call on a capturing stream returns USCT_ERR_ARG before it
 * enqueues anything.  NULL tx_cell/tx_w (with sources) or rx_cell/rx_w give
 * USCT_ERR_ARG.  Calls share the array: calls that overlap on the GPU race on
 * it and must be serialised.
 */
#define USCT_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int usct_forward_fmc_noalloc(int ndim, const int* dims, double h, double dt, int nt,
                             int n_tx, const int* tx_ptr, const int64_t* tx_cell,
                             const double* tx_w, int n_rx, const int* rx_ptr,
                             const int64_t* rx_cell, const double* rx_w, const double* m,
                             const double* sponge, const double* wavelet, float* data,
                             void* stream);

/* ---- the model-update loop of fwi.invert on the device ---- */
/*
 * The whole-model FP64 operations fwi.invert (fwi.py:535-660) and its
 * Gauss-Newton variant (fwi.py:434-532) apply between gradients, so the model
 * and gradient stay in device memory across iterations.  All arrays are device
 * FP64 of n (= cells) elements; NULL optional arrays mean "absent".
 * Elementwise results round as the NumPy expressions they replace; dot and sum
 * use a fixed order (reproducible, not NumPy's order); max|x| is exact.
 */
#define USCT_SMOOTH_MAX_RADIUS 64
/* scipy.ndimage.gaussian_filter with mode 'reflect' (fwi.py:633-634): one 1-D
 * pass per axis in axis order, each adding taps in scipy's order for a
 * symmetric kernel.  taps (host, radius+1 values): taps[0] the centre weight,
 * taps[j] the weight at distance j.  in, out, tmp distinct (tmp unused for
 * ndim 1). */
int usct_smooth_dev(const double* in, double* out, double* tmp, int ndim, const int* dims,
                    const double* taps, int radius, void* stream);
/* out = x * mask (mask NULL: out = x). */
int usct_vec_mul_dev(const double* x, const double* mask, double* out, size_t n, void* stream);
/* out = y + a * x (y NULL: out = a * x); out may alias x or y. */
int usct_vec_axpy_dev(const double* y, double a, const double* x, double* out, size_t n,
                      void* stream);
/* The trial model of the line search (fwi.py:641-646, 510-513):
 * out = m + a * d, clipped to [lo, hi] where mask > 0 (everywhere when mask is
 * NULL; nowhere when lo and hi are NULL). */
int usct_model_trial_dev(const double* m, double a, const double* d, const double* lo,
                         const double* hi, const double* mask, double* out, size_t n,
                         void* stream);
/* *out (device) = max_i |x_i| (fwi.py:637). */
int usct_vec_absmax_dev(const double* x, size_t n, double* out, void* stream);
/* ws[0] (device) = sum_i x_i y_i (y NULL: sum_i x_i); ws holds
 * USCT_DOT_WS_DOUBLES doubles. */
#define USCT_DOT_WS_DOUBLES 609
int usct_vec_dot_dev(const double* x, const double* y, size_t n, double* ws, void* stream);

/* ---- total focusing method (delay-and-sum imaging, imaging.py:27-74) ---- */
/*
 * Analytic signal of every trace of an FMC (scipy.signal.hilbert along time,
 * imaging.py:63), written as x + i (x (*) g): a circular convolution with taps
 * g (device FP32, nt values: the imaginary part of the inverse DFT of scipy's
 * spectral multiplier, computed by the caller).  data: device FP64
 * [n_tx][nt][n_rx] (the Dataset layout); analytic: device FP32 interleaved
 * (re, im) [n_tx][n_rx][nt], trace-major.  For even nt the taps at even
 * offsets must be zero (they are, for scipy's multiplier) and are skipped.
 * n_tx <= 65535, nt <= 2097120.
 */
int usct_analytic_dev(const double* data, float* analytic, int n_tx, int nt, int n_rx,
                      const float* taps, void* stream);
/*
 * TFM image (imaging.py:49-74): for every point r of the C-order grid whose
 * axis a has coordinates axes[a*npix .. a*npix+npix) (device FP64),
 * out = sum_{i < n_tx, j < n_rx} analytic[i][j][round((|r - tx_pos[i]| +
 * |r - rx_pos[j]|) / c * fs)], samples outside [0, nt) skipped; tx_pos
 * (n_tx x dim) and rx_pos (n_rx x dim) device FP64 element positions; out_re,
 * out_im device FP64, npix^dim values.  The sample index equals NumPy's
 * np.round of the same FP64 expression; samples are summed in FP32 over the
 * receivers of one transmit and in FP64 over the transmits.
 */
int usct_tfm_dev(const float* analytic, int n_tx, int n_rx, int nt, const double* tx_pos,
                 const double* rx_pos, int dim, const double* axes, int npix, double c, double fs,
                 double* out_re, double* out_im, void* stream);
/*
 * P-arrival mute windows for time_weights (fwi.p_window_weights,
 * fwi.py:663-699) from the analytic signal of the observed data (as
 * usct_analytic_dev writes it): per trace the first sample whose envelope
 * exceeds onset_frac * (max envelope + 1e-30), kept for `keep` samples, then a
 * cosine roll-off over `taper` samples.  weights: device FP64
 * [n_tx][nt][n_rx].  The envelope is FP32 (the reference's FP64).
 */
int usct_pwindow_dev(const float* analytic, int n_tx, int nt, int n_rx, double onset_frac,
                     double keep, double taper, double* weights, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* USCT_GB300_H */
