"""Host restatement of the reference's FWI loops -- TEST INFRASTRUCTURE ONLY.

``invert`` follows ``ringfwi.fwi.invert`` (simulation/ringfwi/fwi.py:535-660,
steepest descent with Gaussian-smoothed gradient and backtracking line search)
and ``_invert_gauss_newton`` (fwi.py:434-532, CG on (J^T J + mu I) dm = -g),
step for step in NumPy/scipy on host arrays, with the misfit, gradient and
Gauss-Newton product taken from a pluggable backend module (the FP64 oracle
here, or the GB300 backend when checking the device-resident loop).  It is
pinned against the reference's own ``invert`` by the ``invert2d`` golden
fixture.
"""

from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter


def invert(m0, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None, n_iter=15,
           step_frac=0.02, update_mask=None, m_bounds=None, smooth_sigma=1.0, n_linesearch=8,
           backend=None, misfit_type="l2", footprints=None, time_weights=None, optimizer="gd",
           n_cg=8, gn_damp=1e-2):
    if src_list is None:
        src_list = list(range(len(geom.idx)))
    else:
        src_list = list(src_list)
    m0 = np.asarray(m0, np.float64)
    eff_lo = eff_hi = None
    if m_bounds is not None:                                       # fwi.py:615-621
        eff_lo = np.minimum(m_bounds[0], m0)
        eff_hi = np.maximum(m_bounds[1], m0)

    def bound(m_try):
        if m_bounds is None:
            return m_try
        clipped = np.clip(m_try, eff_lo, eff_hi)
        return np.where(update_mask > 0, clipped, m_try) if update_mask is not None else clipped

    if optimizer in ("gauss-newton", "gn"):
        return _gauss_newton(backend, m0, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                             n_iter, update_mask, bound, n_linesearch, footprints, n_cg, gn_damp)

    kw = dict(misfit_type=misfit_type, footprints=footprints, time_weights=time_weights)
    m = m0.copy()
    history = []
    J, g = backend.misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list, **kw)
    for _ in range(n_iter):                                        # fwi.py:624-660
        history.append(J)
        gm = g * update_mask if update_mask is not None else g.copy()
        if smooth_sigma:
            gm = gaussian_filter(gm, smooth_sigma)
            if update_mask is not None:
                gm = gm * update_mask
        gmax = float(np.max(np.abs(gm)))
        if gmax == 0.0:
            break
        direction = -gm
        step = step_frac * float(np.mean(m)) / gmax
        accepted = False
        for _ in range(n_linesearch):
            m_try = bound(m + step * direction)
            J_try = backend.misfit(m_try, geom, wavelet, dt, h, nt, dobs, sponge, src_list, **kw)
            if J_try < J:
                accepted = True
                break
            step *= 0.5
        if not accepted:
            break
        m = m_try
        J, g = backend.misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                                           **kw)
    history.append(J)
    return m, history


def _gauss_newton(backend, m0, geom, wavelet, dt, h, nt, dobs, sponge, src_list, n_iter,
                  update_mask, bound, n_linesearch, footprints, n_cg, gn_damp):
    m = m0.copy()
    mask = update_mask if update_mask is not None else 1.0
    history = []
    for _ in range(n_iter):                                        # fwi.py:459-527
        J, g = backend.misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                                           misfit_type="l2", footprints=footprints)
        history.append(J)
        gm = g * mask
        if float(np.max(np.abs(gm))) == 0.0:
            break

        def A(x):
            hv = backend.gn_hessian_vector(m, geom, wavelet, dt, h, nt, x * mask, sponge,
                                           src_list, footprints)
            return hv * mask

        Hg = A(gm)
        mu = gn_damp * float(gm.ravel() @ Hg.ravel()) / (float(gm.ravel() @ gm.ravel()) + 1e-300)
        b = -gm
        x = np.zeros_like(m)
        r = b.copy()
        d = r.copy()
        rs = float(r.ravel() @ r.ravel())
        rs0 = rs
        for _ in range(n_cg):
            Ad = A(d) + mu * d
            alpha = rs / (float(d.ravel() @ Ad.ravel()) + 1e-300)
            x += alpha * d
            r -= alpha * Ad
            rs_new = float(r.ravel() @ r.ravel())
            if rs_new < 1e-10 * rs0:
                break
            d = r + (rs_new / rs) * d
            rs = rs_new
        step = 1.0
        accepted = False
        for _ in range(n_linesearch):
            m_try = bound(m + step * x)
            J_try = backend.misfit(m_try, geom, wavelet, dt, h, nt, dobs, sponge, src_list, "l2",
                                   footprints)
            if J_try < J:
                accepted = True
                break
            step *= 0.5
        if not accepted:
            break
        m = m_try
    history.append(backend.misfit(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list, "l2",
                                  footprints))
    return m, history


class FP64Backend:
    """The FP64 oracle behind the backend protocol (misfit_type / footprints /
    time_weights keywords, the reference's positional order)."""

    def __init__(self, k=0):
        self.k = k

    def misfit_and_gradient(self, m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None,
                            misfit_type="l2", footprints=None, time_weights=None):
        from . import misfit_and_gradient
        return misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
                                   footprints, k=self.k, misfit_type=misfit_type,
                                   time_weights=time_weights)

    def misfit(self, m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None,
               misfit_type="l2", footprints=None, time_weights=None):
        from . import misfit
        return misfit(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list, footprints,
                      misfit_type=misfit_type, time_weights=time_weights)

    def gn_hessian_vector(self, m, geom, wavelet, dt, h, nt, v, sponge=None, src_list=None,
                          footprints=None, wavefields=None):
        from . import gn_hessian_vector
        return gn_hessian_vector(m, geom, wavelet, dt, h, nt, v, sponge, src_list, footprints,
                                 k=max(self.k, 8))
