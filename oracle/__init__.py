"""CPU oracle for the ringfwi acoustic hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` (to check the GPU result) and ``bench.py``'s
CPU-baseline leg import this package.  The product (``openusct_gb300``) never
does: it has no CPU fallback.

Wraps ``oracle/usct_oracle.c`` (built to ``oracle/liboracle.so`` by
``oracle/Makefile``) and, when it has been built from the reference checkout,
``oracle/_ref/libuap_ref.so`` (the reference's own ``software/core/libuap.hpp``
behind a C shim).  The geometry arguments mirror the reference's Python API
(``simulation/ringfwi/fwi.py:102,266,410``): ``geom`` is anything with an
``idx`` list of grid-index tuples (RingArray, CylinderArray, GridArray) or the
list itself; ``footprints`` is the list of ``(idx_list, weights)`` that
``geometry.build_footprints`` returns.  The conversion to flat CSR arrays is
written here independently of the product's own host code.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_REF = os.path.join(_HERE, "_ref", "libuap_ref.so")
_lock = threading.Lock()
_lib = None
_ref = None

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_longlong)


def build(ref: bool = False) -> None:
    """Compile the restatement (and, with ``ref``, the reference core)."""
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", _HERE, "ref"], check=True)


def _load():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(
                    os.path.join(_HERE, "usct_oracle.c")):
                build()
            lib = ctypes.CDLL(_LIB)
            lib.usct_oracle_misfit_and_gradient.restype = ctypes.c_double
            lib.usct_oracle_misfit_and_gradient_mt.restype = ctypes.c_double
            lib.usct_oracle_misfit_and_gradient_tw.restype = ctypes.c_double
            _lib = lib
    return _lib


def ref_available() -> bool:
    return os.path.exists(_REF)


def _load_ref():
    global _ref
    with _lock:
        if _ref is None:
            lib = ctypes.CDLL(_REF)
            lib.usct_ref_misfit_and_gradient.restype = ctypes.c_double
            _ref = lib
    return _ref


def _p(a, t):
    return a.ctypes.data_as(t)


def _idx_list(geom):
    return list(geom.idx) if hasattr(geom, "idx") else list(geom)


def _lin(t, shape):
    lin = 0
    for a, n in zip(t, shape):
        lin = lin * int(n) + int(a)
    return lin


def _csr(groups, shape):
    """groups: list of (idx_list, weights) -> ptr int32, idx int64, w float64."""
    ptr = [0]
    idx, w = [], []
    for cells, ws in groups:
        for c, wi in zip(cells, ws):
            idx.append(_lin(c, shape))
            w.append(float(wi))
        ptr.append(len(idx))
    return (np.asarray(ptr, np.int32), np.asarray(idx, np.int64).reshape(-1),
            np.asarray(w, np.float64).reshape(-1))


def _geometry(geom, shape, src_list, footprints):
    idx = _idx_list(geom)
    if footprints is None:
        groups = [([t], [1.0]) for t in idx]
    else:
        groups = [(list(c), list(w)) for c, w in footprints]
    if src_list is None:
        src_list = list(range(len(idx)))
    tx = _csr([groups[s] for s in src_list], shape)
    rx = _csr(groups, shape)
    return tx, rx, len(src_list), len(groups)


def _common(m, wavelet, sponge):
    m = np.ascontiguousarray(m, np.float64)
    dims = np.asarray(m.shape, np.int32)
    wav = np.ascontiguousarray(wavelet, np.float64)
    sp = None if sponge is None else np.ascontiguousarray(sponge, np.float64)
    return m, dims, wav, sp


def forward_fmc(m, geom, wavelet, dt, h, nt, sponge=None, src_list=None, footprints=None):
    """FP64 restatement of fwi.forward_fmc / uap::forward_fmc."""
    lib = _load()
    m, dims, wav, sp = _common(m, wavelet, sponge)
    (tp, ti, tw), (rp, ri, rw), ntx, nrx = _geometry(geom, m.shape, src_list, footprints)
    data = np.zeros((ntx, nt, nrx))
    lib.usct_oracle_forward_fmc(_p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h),
                                ctypes.c_double(dt), int(nt), ntx, _p(tp, _ip), _p(ti, _lp),
                                _p(tw, _dp), nrx, _p(rp, _ip), _p(ri, _lp), _p(rw, _dp),
                                _p(wav, _dp), None if sp is None else _p(sp, _dp), _p(data, _dp))
    return data


_MT = {"l2": 0, "gcn": 1}


def _windows(time_weights, shape):
    """time_weights (fwi.py:250-253: one (nt, n_rx) window per transmit) as a
    contiguous float64 (n_tx, nt, n_rx) array, or None."""
    if time_weights is None:
        return None
    w = np.ascontiguousarray(np.stack([np.asarray(t, np.float64) for t in time_weights]))
    if w.shape != tuple(shape):
        raise ValueError(f"time_weights shape {w.shape} != {tuple(shape)}")
    return w


def misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None,
                        footprints=None, k=0, misfit_type="l2", time_weights=None):
    """FP64 restatement of fwi.misfit_and_gradient (L2 or GCN, optional
    time_weights as fwi.py:298-301).  k = 0: full history (the reference's
    memory plan); k > 0: checkpoints every k steps."""
    lib = _load()
    m, dims, wav, sp = _common(m, wavelet, sponge)
    (tp, ti, tw), (rp, ri, rw), ntx, nrx = _geometry(geom, m.shape, src_list, footprints)
    dobs = np.ascontiguousarray(dobs, np.float64)
    win = _windows(time_weights, (ntx, nt, nrx))
    g = np.zeros(m.shape)
    J = lib.usct_oracle_misfit_and_gradient_tw(
        _p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h), ctypes.c_double(dt), int(nt),
        ntx, _p(tp, _ip), _p(ti, _lp), _p(tw, _dp), nrx, _p(rp, _ip), _p(ri, _lp), _p(rw, _dp),
        _p(wav, _dp), None if sp is None else _p(sp, _dp), _p(dobs, _dp),
        None if win is None else _p(win, _dp), _p(g, _dp), int(k), _MT[misfit_type])
    return float(J), g


def misfit(m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None, footprints=None,
           misfit_type="l2", time_weights=None):
    """FP64 fwi.misfit (fwi.py:246-263): forward FMC, then the per-transmit
    misfit of the (optionally windowed) traces."""
    d = forward_fmc(m, geom, wavelet, dt, h, nt, sponge, src_list, footprints)
    dobs = np.asarray(dobs, np.float64)
    win = _windows(time_weights, d.shape)
    J = 0.0
    for i in range(d.shape[0]):
        di, oi = d[i], dobs[i]
        if win is not None:
            di, oi = di * win[i], oi * win[i]
        if misfit_type == "gcn":   # libuap.hpp:133-154
            eps = 1e-12
            ns = np.sqrt(np.sum(di * di, axis=0)) + eps
            no = np.sqrt(np.sum(oi * oi, axis=0)) + eps
            J += float(np.sum(1.0 - np.sum((di / ns) * (oi / no), axis=0)))
        else:
            r = di - oi
            J += 0.5 * float(np.sum(r * r))
    return J


def gn_hessian_vector(m, geom, wavelet, dt, h, nt, v, sponge=None, src_list=None,
                      footprints=None, k=32, return_born=False):
    """FP64 restatement of fwi.gn_hessian_vector (checkpointed background)."""
    lib = _load()
    m, dims, wav, sp = _common(m, wavelet, sponge)
    (tp, ti, tw), (rp, ri, rw), ntx, nrx = _geometry(geom, m.shape, src_list, footprints)
    v = np.ascontiguousarray(v, np.float64)
    out = np.zeros(m.shape)
    born = np.zeros((ntx, nt, nrx)) if return_born else None
    lib.usct_oracle_gn_hessian_vector(
        _p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h), ctypes.c_double(dt), int(nt),
        ntx, _p(tp, _ip), _p(ti, _lp), _p(tw, _dp), nrx, _p(rp, _ip), _p(ri, _lp), _p(rw, _dp),
        _p(wav, _dp), None if sp is None else _p(sp, _dp), _p(v, _dp), _p(out, _dp),
        None if born is None else _p(born, _dp), int(k))
    return (out, born) if return_born else out


def forward_steps(m, h, dt, nsteps, src_cell, wavelet):
    """CPU-baseline timing hook: nsteps FP64 leapfrog steps of one point source."""
    lib = _load()
    m = np.ascontiguousarray(m, np.float64)
    dims = np.asarray(m.shape, np.int32)
    wav = np.ascontiguousarray(wavelet, np.float64)
    si = np.asarray([_lin(src_cell, m.shape)], np.int64)
    sw = np.ones(1)
    out = np.zeros(m.shape)
    lib.usct_oracle_forward_steps(_p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h),
                                  ctypes.c_double(dt), int(nsteps), 1, _p(si, _lp), _p(sw, _dp),
                                  _p(wav, _dp), _p(out, _dp))
    return out


# --- FP32 restatement in the CUDA kernels' operation order -------------------

def forward_fmc32(m, geom, wavelet, dt, h, nt, sponge=None, src_list=None, footprints=None):
    lib = _load()
    m, dims, wav, sp = _common(m, wavelet, sponge)
    (tp, ti, tw), (rp, ri, rw), ntx, nrx = _geometry(geom, m.shape, src_list, footprints)
    data = np.zeros((ntx, nt, nrx), np.float32)
    lib.usct_oracle32_forward_fmc(_p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h),
                                  ctypes.c_double(dt), int(nt), ntx, _p(tp, _ip), _p(ti, _lp),
                                  _p(tw, _dp), nrx, _p(rp, _ip), _p(ri, _lp), _p(rw, _dp),
                                  _p(wav, _dp), None if sp is None else _p(sp, _dp),
                                  _p(data, _fp))
    return data


def misfit_and_gradient32(m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None,
                          footprints=None, C=1, misfit_type="l2", time_weights=None):
    """Returns (J per transmit float64 array, g float64) in kernel order for a
    batch width of C shot channels."""
    lib = _load()
    m, dims, wav, sp = _common(m, wavelet, sponge)
    (tp, ti, tw), (rp, ri, rw), ntx, nrx = _geometry(geom, m.shape, src_list, footprints)
    dobs = np.ascontiguousarray(dobs, np.float64)
    win = _windows(time_weights, (ntx, nt, nrx))
    g = np.zeros(m.shape)
    J = np.zeros(ntx)
    rc = lib.usct_oracle32_misfit_and_gradient_tw(
        _p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h), ctypes.c_double(dt), int(nt),
        ntx, _p(tp, _ip), _p(ti, _lp), _p(tw, _dp), nrx, _p(rp, _ip), _p(ri, _lp), _p(rw, _dp),
        _p(wav, _dp), None if sp is None else _p(sp, _dp), _p(dobs, _dp),
        None if win is None else _p(win, _dp), int(C), _p(J, _dp), _p(g, _dp),
        _MT[misfit_type])
    if rc != 0:
        raise ValueError("C must be a power of two <= 64")
    return J, g


def gn_hessian_vector32(m, geom, wavelet, dt, h, nt, v, sponge=None, src_list=None,
                        footprints=None, C=1):
    lib = _load()
    m, dims, wav, sp = _common(m, wavelet, sponge)
    (tp, ti, tw), (rp, ri, rw), ntx, nrx = _geometry(geom, m.shape, src_list, footprints)
    v = np.ascontiguousarray(v, np.float64)
    out = np.zeros(m.shape)
    born = np.zeros((ntx, nt, nrx), np.float32)
    rc = lib.usct_oracle32_gn_hessian_vector(
        _p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h), ctypes.c_double(dt), int(nt),
        ntx, _p(tp, _ip), _p(ti, _lp), _p(tw, _dp), nrx, _p(rp, _ip), _p(ri, _lp), _p(rw, _dp),
        _p(wav, _dp), None if sp is None else _p(sp, _dp), _p(v, _dp), int(C), _p(out, _dp),
        _p(born, _fp))
    if rc != 0:
        raise ValueError("C must be a power of two <= 64")
    return out, born


# --- the reference's own C++ core (built from the reference checkout) --------

def ref_forward_fmc(m, geom, wavelet, dt, h, nt, src_list=None):
    lib = _load_ref()
    m = np.ascontiguousarray(m, np.float64)
    dims = np.asarray(m.shape, np.int32)
    idx = _idx_list(geom)
    rec = np.asarray([_lin(t, m.shape) for t in idx], np.int32)
    tx = rec.copy() if src_list is None else np.asarray([rec[s] for s in src_list], np.int32)
    wav = np.ascontiguousarray(wavelet, np.float64)
    data = np.zeros((len(tx), nt, len(rec)))
    lib.usct_ref_forward_fmc(_p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h),
                             ctypes.c_double(dt), int(nt), _p(tx, _ip), len(tx), _p(rec, _ip),
                             len(rec), _p(wav, _dp), _p(data, _dp))
    return data


def ref_misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, src_list=None, misfit_type="l2"):
    lib = _load_ref()
    m = np.ascontiguousarray(m, np.float64)
    dims = np.asarray(m.shape, np.int32)
    idx = _idx_list(geom)
    rec = np.asarray([_lin(t, m.shape) for t in idx], np.int32)
    tx = rec.copy() if src_list is None else np.asarray([rec[s] for s in src_list], np.int32)
    wav = np.ascontiguousarray(wavelet, np.float64)
    dobs = np.ascontiguousarray(dobs, np.float64)
    g = np.zeros(m.shape)
    J = lib.usct_ref_misfit_and_gradient(_p(m, _dp), _p(dims, _ip), m.ndim, ctypes.c_double(h),
                                         ctypes.c_double(dt), int(nt), _p(tx, _ip), len(tx),
                                         _p(rec, _ip), len(rec), _p(wav, _dp), _p(dobs, _dp),
                                         _p(g, _dp), _MT[misfit_type])
    return float(J), g
