"""FWI with the model and gradient resident on the GPU.

``invert`` has the signature and the algorithm of the reference's
``ringfwi.fwi.invert`` (simulation/ringfwi/fwi.py:535-660: preconditioned
steepest descent with a backtracking line search) and of its truncated
Gauss-Newton branch (``_invert_gauss_newton``, fwi.py:434-532).  The misfit,
gradient and Gauss-Newton products come from :mod:`openusct_gb300.backend`
(or any backend module with the same functions that accepts CUDA tensors);
the whole-model FP64 work between them -- mask, Gaussian smoothing of the
gradient, max|g|, trial models with effective bounds, the conjugate-gradient
vector algebra -- runs on the library's update kernels (``usct_smooth_dev``
and friends), so per iteration only scalars cross to the host (J, max|g|, the
mean of m, CG dot products).

Differences from the reference, all deliberate:

* every misfit (l2, gcn), footprints and time_weights run on the device; the
  reference falls back to its Python core for footprints and windows
  (fwi.py:594-615);
* the mean of m and the CG dot products are summed in a fixed device order,
  not NumPy's pairwise/BLAS order, so they can differ in the last bits; every
  elementwise step and the smoothing round exactly as the reference's NumPy /
  scipy expressions;
* ``smooth_sigma`` must be a scalar (the reference only passes scalars).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

__all__ = ["invert", "fwi_from_dataset", "register", "smoothing_taps", "ModelOps"]


def smoothing_taps(sigma, truncate=4.0):
    """Taps of scipy.ndimage.gaussian_filter1d for ``sigma`` (order 0): the
    kernel exp(-x^2 / (2 sigma^2)) on x = -r..r, r = int(truncate*sigma + 0.5),
    normalised by its sum, computed the same way; returned as the centre
    weight followed by the weights at distance 1..r."""
    sigma = float(sigma)
    radius = int(truncate * sigma + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (sigma * sigma) * x ** 2)
    phi = phi / phi.sum()
    return np.ascontiguousarray(phi[radius:], dtype=np.float64)


def _p(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


class ModelOps:
    """The update kernels on one device and stream, on FP64 tensors of one shape."""

    def __init__(self, shape, device, stream=None):
        self.lib = _lib.load()
        self.shape = tuple(int(s) for s in shape)
        self.n = int(np.prod(self.shape))
        self.dev = device
        self.stream = stream if stream is not None else torch.cuda.current_stream(device)
        self.dims = (ctypes.c_int * len(self.shape))(*self.shape)
        self.ws = torch.zeros(_lib.DOT_WS_DOUBLES, dtype=torch.float64, device=device)
        self.scalar = torch.zeros(1, dtype=torch.float64, device=device)
        self._tmp = None

    def _s(self):
        return ctypes.c_void_p(self.stream.cuda_stream)

    def empty(self):
        return torch.empty(self.shape, dtype=torch.float64, device=self.dev)

    def smooth(self, x, out, sigma):
        """out = scipy.ndimage.gaussian_filter(x, sigma) (mode 'reflect')."""
        taps = smoothing_taps(sigma)
        if len(taps) - 1 > _lib.SMOOTH_MAX_RADIUS:
            raise ValueError(f"smooth_sigma {sigma} needs a radius above "
                             f"{_lib.SMOOTH_MAX_RADIUS}")
        if self._tmp is None:
            self._tmp = self.empty()
        _lib.check(self.lib.usct_smooth_dev(
            _p(x), _p(out), _p(self._tmp), len(self.shape), self.dims,
            taps.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(taps) - 1, self._s()))
        return out

    def mul(self, x, mask, out):
        _lib.check(self.lib.usct_vec_mul_dev(_p(x), _p(mask), _p(out), self.n, self._s()))
        return out

    def axpy(self, y, a, x, out):
        """out = y + a*x (y None: a*x)."""
        _lib.check(self.lib.usct_vec_axpy_dev(_p(y), ctypes.c_double(a), _p(x), _p(out), self.n,
                                              self._s()))
        return out

    def trial(self, m, a, d, lo, hi, mask, out):
        _lib.check(self.lib.usct_model_trial_dev(_p(m), ctypes.c_double(a), _p(d), _p(lo),
                                                 _p(hi), _p(mask), _p(out), self.n, self._s()))
        return out

    def absmax(self, x):
        _lib.check(self.lib.usct_vec_absmax_dev(_p(x), self.n, _p(self.scalar), self._s()))
        return float(self.scalar.item())

    def dot(self, x, y=None):
        _lib.check(self.lib.usct_vec_dot_dev(_p(x), _p(y), self.n, _p(self.ws), self._s()))
        return float(self.ws[0].item())

    def mean(self, x):
        return self.dot(x) / self.n


def _dev_tensor(x, dev):
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float64).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(dev)


def _bounds(m_bounds, m0, ops):
    """Effective bounds that never push a cell across its own start value
    (fwi.py:615-621): lo = min(bounds[0], m0), hi = max(bounds[1], m0)."""
    if m_bounds is None:
        return None, None
    lo = torch.broadcast_to(_dev_tensor(np.asarray(m_bounds[0], np.float64)
                                        if not isinstance(m_bounds[0], torch.Tensor)
                                        else m_bounds[0], ops.dev), ops.shape)
    hi = torch.broadcast_to(_dev_tensor(np.asarray(m_bounds[1], np.float64)
                                        if not isinstance(m_bounds[1], torch.Tensor)
                                        else m_bounds[1], ops.dev), ops.shape)
    return torch.minimum(lo, m0).contiguous(), torch.maximum(hi, m0).contiguous()


def _backend(backend):
    if backend is not None and hasattr(backend, "misfit_and_gradient"):
        return backend
    from . import backend as gb
    return gb


class _Evaluator:
    """``misfit`` / ``misfit_and_gradient`` of :mod:`openusct_gb300.backend`
    for one inversion.  The data, wavelet, sponge and windows go up once.
    When the acquisition is one shot batch, a line-search trial runs its
    forward sweep in gradient mode (checkpoints and the last segment's stash)
    and keeps it, so the gradient at the accepted trial model -- the next
    iteration's first call -- only runs the backward sweep: the same engine
    calls in the same order as ``usct_misfit_and_gradient_tw_dev`` (prepare,
    forward, misfit, backward, finalize), so J and g are identical, and one
    forward sweep per iteration is saved."""

    def __init__(self, gb, m0, geom, wavelet, dt, h, nt, dobs, sponge, src_list, misfit_type,
                 footprints, time_weights, batch=None):
        self.gb = gb
        self.mt = gb._check_misfit(misfit_type)
        p = self.plan = gb._setup(m0, geom, h, dt, nt, src_list, footprints, _lib.MODE_GRADIENT,
                                  batch, None, None)
        dev = m0.device
        self.wd = gb._wavelet(wavelet, nt, dev)
        self.sd = gb._grid_array(sponge, tuple(m0.shape), "sponge", dev)
        self.od = gb._to_dev(dobs, torch.float32, dev)
        if tuple(self.od.shape) != (p.n_tx, p.nt, p.n_rx):
            raise ValueError(f"dobs has shape {tuple(self.od.shape)}, expected "
                             f"{(p.n_tx, p.nt, p.n_rx)}")
        self.tw = gb._time_weights(time_weights, p, dev)
        self.J = torch.zeros(p.n_tx, dtype=torch.float64, device=dev)
        # workspaces of its own, not the plan's shared ones: the kept forward
        # state must survive other calls on the same (cached) plan between
        # a trial and its gradient
        self.mws = gb._alloc_bytes(p.model_bytes(), dev)
        self.bws = gb._alloc_bytes(p.batch_bytes(_lib.MODE_GRADIENT), dev)
        self.single = p.nbatch == 1
        # the model tensor whose forward state the workspaces hold.  The
        # caller must not change that tensor before asking for its gradient
        # (the descent loop asks right after the accepted trial; the model
        # updates write through the library, which torch's version counter
        # does not see, so identity is the contract)
        self.kept = None

    def _forward_misfit(self, b, mode, s):
        P, lib, h = self.gb._ptr, self.plan._lib, self.plan.handle
        _lib.check(lib.usct_batch_forward(h, P(self.mws), P(self.bws), b, mode, None, s))
        _lib.check(lib.usct_batch_misfit_tw(h, P(self.bws), b, P(self.od), P(self.tw), self.mt,
                                            P(self.J), s))

    def _prepare(self, m, s):
        P = self.gb._ptr
        _lib.check(self.plan._lib.usct_model_prepare(self.plan.handle, P(self.mws), P(m),
                                                     P(self.sd), None, P(self.wd), s))

    def misfit(self, m):
        gb = self.gb
        with self.plan.lock, gb._on_exec_stream() as st:
            s = gb._stream(st)
            self._prepare(m, s)
            mode = _lib.MODE_GRADIENT if self.single else _lib.MODE_FORWARD
            for b in range(self.plan.nbatch):
                self._forward_misfit(b, mode, s)
            self.plan.check(st)
        self.kept = m if self.single else None
        return float(np.sum(self.J.cpu().numpy()))

    def misfit_and_gradient(self, m):
        gb, P = self.gb, self.gb._ptr
        lib, h = self.plan._lib, self.plan.handle
        g = torch.empty(self.plan.shape, dtype=torch.float64, device=m.device)
        reuse = self.kept is not None and self.kept is m
        with self.plan.lock, gb._on_exec_stream() as st:
            s = gb._stream(st)
            if reuse:
                _lib.check(lib.usct_batch_backward(h, P(self.mws), P(self.bws), 0, s))
            else:
                self._prepare(m, s)
                for b in range(self.plan.nbatch):
                    self._forward_misfit(b, _lib.MODE_GRADIENT, s)
                    _lib.check(lib.usct_batch_backward(h, P(self.mws), P(self.bws), b, s))
            _lib.check(lib.usct_model_gradient(h, P(self.mws), P(m), P(g), s))
            self.plan.check(st)
        self.kept = None
        return float(np.sum(self.J.cpu().numpy())), g


def invert(m0, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None, n_iter=15,
           step_frac=0.02, update_mask=None, m_bounds=None, smooth_sigma=1.0, n_linesearch=8,
           verbose=False, backend=None, misfit_type="l2", footprints=None, progress=None,
           time_weights=None, optimizer="gd", n_cg=8, gn_damp=1e-2, engine_options=None):
    """Device-resident ``fwi.invert``; returns ``(m, history)`` like the reference
    (``m`` a NumPy array, or a CUDA tensor when ``m0`` is one).

    ``engine_options`` (this backend only): ``batch`` (shots per launch) and
    ``ckpt_k`` (checkpoint interval) for every gradient and Gauss-Newton call
    of the Gauss-Newton loop; the default is the backend's own choice."""
    if optimizer in ("gauss-newton", "gn"):
        if misfit_type != "l2":
            raise ValueError("Gauss-Newton is defined for the L2 misfit; "
                             "select misfit_type='l2'.")
        if time_weights is not None:
            raise ValueError("Gauss-Newton does not support time_weights yet.")
    elif optimizer != "gd":
        raise ValueError(f"unknown optimizer {optimizer!r}")
    if smooth_sigma and np.ndim(smooth_sigma) != 0:
        raise NotImplementedError("smooth_sigma must be a scalar")
    if not torch.cuda.is_available():
        raise RuntimeError("openusct_gb300 needs a CUDA device (there is no CPU fallback)")
    be = _backend(backend)
    dev = torch.device("cuda", torch.cuda.current_device())
    as_tensor = isinstance(m0, torch.Tensor) and m0.is_cuda
    m0d = _dev_tensor(m0, dev)
    ops = ModelOps(m0d.shape, dev)
    mask = _dev_tensor(update_mask, dev)
    if mask is not None:
        mask = torch.broadcast_to(mask, ops.shape).contiguous()
    lo, hi = _bounds(m_bounds, m0d, ops)
    src_list = list(range(geom.n_elements if hasattr(geom, "n_elements") else len(geom.idx))) \
        if src_list is None else list(src_list)
    if optimizer in ("gauss-newton", "gn"):
        m, history = _gauss_newton(be, ops, m0d, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                                   n_iter, mask, lo, hi, n_linesearch, verbose, progress,
                                   footprints, n_cg, gn_damp, engine_options)
    else:
        m, history = _descent(be, ops, m0d, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                              n_iter, step_frac, mask, lo, hi, smooth_sigma, n_linesearch,
                              verbose, progress, misfit_type, footprints, time_weights)
    return (m if as_tensor else m.cpu().numpy()), history


def _descent(be, ops, m0, geom, wavelet, dt, h, nt, dobs, sponge, src_list, n_iter, step_frac,
             mask, lo, hi, smooth_sigma, n_linesearch, verbose, progress, misfit_type,
             footprints, time_weights):
    """fwi.py:623-660 on the device."""
    kw = dict(misfit_type=misfit_type, footprints=footprints, time_weights=time_weights)
    from . import backend as gb
    if be is gb and len(src_list) > 0:
        ev = _Evaluator(gb, m0, geom, wavelet, dt, h, nt, dobs, sponge, src_list, misfit_type,
                        footprints, time_weights)
        mg, mf = ev.misfit_and_gradient, ev.misfit
    else:
        def mg(mm):
            return be.misfit_and_gradient(mm, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                                          **kw)

        def mf(mm):
            return be.misfit(mm, geom, wavelet, dt, h, nt, dobs, sponge, src_list, **kw)

    m = m0.clone()
    gm = ops.empty()
    gs = ops.empty()
    m_try = ops.empty()
    history = []
    J, g = mg(m)
    for it in range(n_iter):
        history.append(J)
        if verbose:
            print(f"  iter {it:2d}  misfit = {J:.6e}")
        ops.mul(g, mask, gm)                       # g * update_mask (or a copy)
        if smooth_sigma:
            ops.smooth(gm, gs, smooth_sigma)
            gm, gs = gs, gm
            if mask is not None:
                ops.mul(gm, mask, gm)
        gmax = ops.absmax(gm)
        if gmax == 0.0:
            break
        # direction = -gm; m + step * direction == m + (-step) * gm exactly
        step = step_frac * ops.mean(m) / gmax
        accepted = False
        for _ in range(n_linesearch):
            ops.trial(m, -step, gm, lo, hi, mask, m_try)
            J_try = mf(m_try)
            if J_try < J:
                accepted = True
                break
            step *= 0.5
        if not accepted:
            if verbose:
                print("  line search failed to reduce misfit; stopping")
            break
        m, m_try = m_try, m
        J, g = mg(m)
        if progress is not None:
            progress(it + 1, n_iter)
    history.append(J)
    return m, history


def _gauss_newton(be, ops, m0, geom, wavelet, dt, h, nt, dobs, sponge, src_list, n_iter, mask,
                  lo, hi, n_linesearch, verbose, progress, footprints, n_cg, gn_damp,
                  engine_options=None):
    """fwi.py:447-532 on the device: CG on (J^T J + mu I) dm = -g, then a
    backtracking line search along dm."""
    kw = dict(footprints=footprints)
    eo = dict(engine_options or {})
    kw_mf = dict(batch=eo["batch"]) if "batch" in eo else {}   # misfit takes no interval
    kw.update(eo)
    m = m0.clone()
    m_try = ops.empty()
    gm, xm, hv = ops.empty(), ops.empty(), ops.empty()
    x, r, d, Ad = ops.empty(), ops.empty(), ops.empty(), ops.empty()
    history = []

    def A(v, out):
        ops.mul(v, mask, xm)                                  # x * mask
        hvv = be.gn_hessian_vector(m, geom, wavelet, dt, h, nt, xm, sponge, src_list, **kw)
        return ops.mul(hvv, mask, out)                        # hv * mask

    for it in range(n_iter):
        J, g = be.misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                                      misfit_type="l2", **kw)
        history.append(J)
        if verbose:
            print(f"  GN iter {it:2d}  misfit = {J:.6e}")
        ops.mul(g, mask, gm)
        if ops.absmax(gm) == 0.0:
            break
        A(gm, hv)
        mu = gn_damp * ops.dot(gm, hv) / (ops.dot(gm, gm) + 1e-300)
        ops.axpy(None, -1.0, gm, r)                           # b = -gm; r = b
        x.zero_()
        d.copy_(r)
        rs = ops.dot(r, r)
        rs0 = rs
        for _ in range(n_cg):
            A(d, Ad)
            ops.axpy(Ad, mu, d, Ad)                           # A(d) + mu d
            alpha = rs / (ops.dot(d, Ad) + 1e-300)
            ops.axpy(x, alpha, d, x)
            ops.axpy(r, -alpha, Ad, r)
            rs_new = ops.dot(r, r)
            if rs_new < 1e-10 * rs0:
                break
            ops.axpy(r, rs_new / rs, d, d)
            rs = rs_new
        step = 1.0
        accepted = False
        for _ in range(n_linesearch):
            ops.trial(m, step, x, lo, hi, mask, m_try)
            J_try = be.misfit(m_try, geom, wavelet, dt, h, nt, dobs, sponge, src_list, "l2",
                              footprints, **kw_mf)
            if J_try < J:
                accepted = True
                break
            step *= 0.5
        if not accepted:
            if verbose:
                print("  GN line search failed to reduce misfit; stopping")
            break
        m, m_try = m_try, m
        if progress is not None:
            progress(it + 1, n_iter)
    history.append(be.misfit(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list, "l2",
                             footprints, **kw_mf))
    return m, history


def fwi_from_dataset(dataset, start_c=None, update_frac=0.95, m_bounds=None, n_iter=12,
                     step_frac=0.03, verbose=False, **invert_kw):
    """FWI of a portable Dataset on the device (fwi.py:702-775, the reference's
    ``"fwi"`` plugin): the reconstruction grid from the dataset's ground truth
    (or from the wavelength), element positions mapped to grid indices, a
    homogeneous or given start model, a radial update mask within
    ``update_frac`` of the array radius, then :func:`invert`.

    Returns the reference's dict: ``c`` (recovered velocity), ``history``,
    ``extent``, ``h``, ``geom``.
    """
    from .geometry import IndexGeometry
    ds = dataset
    dim = int(ds.geometry.dim)
    if ds.ground_truth is not None:
        h = ds.ground_truth["h_m"]
        shape = np.shape(ds.ground_truth["c"])
    else:
        ppw = 5.0
        h = ds.nominal_speed_m_s / (ds.tx_centre_freq_hz * ppw)
        npix = int(round(2.2 * ds.geometry.radius_m / h)) + 1
        shape = (npix,) * dim
    n = shape[0]
    domain = (n - 1) * h
    abspos = np.asarray(ds.geometry.element_pos) + domain / 2.0
    idx = [tuple(int(round(p[a] / h)) for a in reversed(range(dim))) for p in abspos]
    geom = IndexGeometry(idx)
    if start_c is None:
        start_c = np.full(shape, ds.nominal_speed_m_s)
    start_c = np.asarray(start_c, np.float64)
    m0 = 1.0 / (start_c * start_c)
    centre = domain / 2.0
    coords = np.mgrid[tuple(slice(0, n) for _ in range(dim))].astype(float) * h
    # transverse radius: both axes in 2D, axes (1, 2) in 3D (the array axis is z)
    transverse = range(dim) if dim == 2 else range(1, dim)
    r = np.sqrt(sum((coords[a] - centre) ** 2 for a in transverse))
    update_mask = (r <= ds.geometry.radius_m * update_frac).astype(float)
    m_rec, history = invert(m0, geom, ds.tx_wavelet, 1.0 / ds.sample_rate_hz, h,
                            int(np.shape(ds.data)[1]), ds.data,
                            src_list=[int(e) for e in ds.tx_elements], n_iter=n_iter,
                            step_frac=step_frac, update_mask=update_mask, m_bounds=m_bounds,
                            verbose=verbose, **invert_kw)
    return {"c": 1.0 / np.sqrt(m_rec), "history": history, "extent": (-centre, domain - centre),
            "h": h, "geom": geom}


def register(plugins):
    """Install :func:`fwi_from_dataset` as the reference plugin registry's
    ``"fwi"`` entry (plugins.py:62-66)."""
    plugins.register("fwi", description="Adjoint-state FWI on the GB300 (sound-speed model)",
                     output="model")(fwi_from_dataset)
    return fwi_from_dataset
