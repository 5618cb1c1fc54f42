"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""

from __future__ import annotations

import os

import numpy as np

from openusct_gb300.geometry import IndexGeometry, footprints_from_csr

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["ring2d_point", "ring2d_sponge", "ring2d_aperture", "cyl3d_point", "cyl3d_aperture",
         "odd2d", "odd3d", "parity2d", "parity3d", "gpu3d"]

# FP32-vs-FP64 tolerances per fixture (relative L2).  Traces: 1e-5 on smooth
# models; the odd* models are per-cell white noise (high-wavenumber fields) and
# get 1e-4.  Gradients: 1e-4 where the residual is a sizeable part of the data
# (the benchmark configurations' regime: the reference's own parity problems
# and most test setups).  cyl3d_point / cyl3d_aperture are nearly converged (|r|/|d| = 0.15%
# and 0.6%): there the FP32 trace noise (~2e-7 of the data) is 1e-4 of the
# residual and the FP64 adjoint of that residual alone reproduces the observed
# 3e-3 / 3e-4 gradient error, so their bound is the conditioning, not the
# kernels (which match the FP32 restatement bit for bit).  cyl3d_window is the
# cyl3d_point problem with a data window and shares its bound.
TRACE_TOL = {"odd2d": 1e-4, "odd3d": 1e-4}
GRAD_TOL = {"cyl3d_point": 5e-3, "cyl3d_aperture": 5e-4, "cyl3d_window": 5e-3}


def trace_tol(name):
    return TRACE_TOL.get(name, 1e-5)


def grad_tol(name):
    return GRAD_TOL.get(name, 1e-4)


class Case:
    def __init__(self, name):
        self.name = name
        z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        self.z = z
        self.geom = IndexGeometry([tuple(int(v) for v in r) for r in z["idx"]])
        self.wavelet = z["wavelet"]
        self.dt = float(z["dt"])
        self.h = float(z["h"])
        self.nt = int(z["nt"])
        self.src_list = [int(s) for s in z["src_list"]]
        self.sponge = z["sponge"] if z["sponge"].size else None
        self.footprints = (footprints_from_csr(z["fp_ptr"], z["fp_idx"], z["fp_w"])
                           if "fp_ptr" in z else None)

    def __getitem__(self, k):
        return self.z[k]

    def __contains__(self, k):
        return k in self.z

    def args(self):
        return dict(wavelet=self.wavelet, dt=self.dt, h=self.h, nt=self.nt, sponge=self.sponge,
                    src_list=self.src_list, footprints=self.footprints)


def load(name):
    return Case(name)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def rel_max(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
