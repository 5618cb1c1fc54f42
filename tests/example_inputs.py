"""The inputs of openusct_gb300/csrc/usct_example.cpp, restated in NumPy so the
example's printed checksums can be checked against the oracle."""

import numpy as np


def example_problem():
    n, h, dt, f0, nt = 48, 1.0e-3, 1.4e-7, 0.35e6, 320
    t = np.arange(nt) * dt - 1.0 / f0
    u = np.pi * f0 * t
    wavelet = (1.0 - 2.0 * u * u) * np.exp(-u * u)
    L = (n - 1) * h
    iy, ix = np.mgrid[0:n, 0:n]
    dx = ix * h - 0.60 * L
    dy = iy * h - 0.45 * L
    c = np.where(dx * dx + dy * dy <= 0.005 * 0.005, 2500.0, 2950.0)
    m_true = 1.0 / (c * c)
    m0 = np.full((n, n), 1.0 / (2950.0 * 2950.0))
    a = 2.0 * np.pi * np.arange(16) / 16
    ex = [int(np.floor(v + 0.5)) for v in (0.5 * L + 0.018 * np.cos(a)) / h]
    ey = [int(np.floor(v + 0.5)) for v in (0.5 * L + 0.018 * np.sin(a)) / h]
    idx = [(y, x) for y, x in zip(ey, ex)]
    return dict(n=n, h=h, dt=dt, nt=nt, wavelet=wavelet, m_true=m_true, m0=m0, idx=idx)
