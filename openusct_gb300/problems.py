"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved anywhere: every model is generated from a seed.

* ``ring2d``      2D ring FWI gradient: 256^2 grid, dx = 0.15 mm, 64-element
                  ring of radius 16 mm, water (1500 m/s) with two seeded discs
                  (r = 3 mm at 1450 m/s, r = 5 mm at 1580 m/s) inside r < 10 mm,
                  1 MHz Ricker, dt from CFL 0.3, nt = 1500, start model 1500.
* ``cylinder3d``  3D cylinder FMC: 192^3, dx = 0.2 mm, 8 rings x 32 elements on
                  r = 15 mm over z in [-10, 10] mm, 1500 m/s times (1 + f) with
                  f a Gaussian-smoothed (sigma = 2 mm) seeded field scaled to
                  max|f| = 0.03, 1 MHz Ricker, nt = 2000.
* ``cylinder3d_large``  the 320^3 variant (dx = 0.12 mm, 16 x 32 elements, nt = 3000).
* ``gn3d``        Gauss-Newton: 224^3, dx = 0.18 mm, 256 shots, nt = 2500,
                  seeded smooth perturbation v.
Each builder takes ``n``/``nt``/element-count overrides so tests can run
scaled-down versions of the same construction.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .geometry import CylinderGeometry, RingGeometry, ricker


@dataclass
class Problem:
    name: str
    geom: object
    c_true: np.ndarray
    m_true: np.ndarray
    m0: np.ndarray
    h: float
    dt: float
    nt: int
    wavelet: np.ndarray
    f0: float
    v: np.ndarray | None = None

    @property
    def shape(self):
        return self.m_true.shape

    @property
    def n_shots(self):
        return len(self.geom.idx)


def _discs(n, h, rng, r_max=0.010):
    """Two non-overlapping discs fully inside r < r_max (centre convention (n-1)h/2)."""
    centre = (n - 1) * h / 2.0
    discs = [(0.003, 1450.0), (0.005, 1580.0)]
    placed = []
    for rad, _c in discs:
        for _ in range(10000):
            r = (r_max - rad) * np.sqrt(rng.uniform())
            th = rng.uniform(0, 2 * np.pi)
            x, y = centre + r * np.cos(th), centre + r * np.sin(th)
            if all(np.hypot(x - px, y - py) > rad + pr for px, py, pr in placed):
                placed.append((x, y, rad))
                break
    yy, xx = np.mgrid[0:n, 0:n] * h
    c = np.full((n, n), 1500.0)
    for (x, y, rad), (_r, cv) in zip(placed, discs):
        c[np.hypot(xx - x, yy - y) <= rad] = cv
    return c


def ring2d(seed=0, n=256, h=0.15e-3, n_el=64, radius=0.016, nt=1500, f0=1e6):
    rng = np.random.default_rng(seed)
    geom = RingGeometry(n_el, radius, (n - 1) * h, h)
    c = _discs(n, h, rng)
    dt = 0.3 * h / float(c.max())
    return Problem("ring2d", geom, c, 1.0 / c ** 2, np.full((n, n), 1.0 / 1500.0 ** 2), h, dt, nt,
                   ricker(nt, dt, f0), f0)


def random_field(shape, sigma_cells, amp, rng):
    from scipy.ndimage import gaussian_filter
    f = gaussian_filter(rng.standard_normal(shape), sigma_cells)
    return f * (amp / np.abs(f).max())


def cylinder3d(seed=0, n=192, h=0.2e-3, n_rings=8, per_ring=32, radius=0.015, height=0.020,
               nt=2000, f0=1e6):
    rng = np.random.default_rng(seed)
    geom = CylinderGeometry(n_rings, per_ring, radius, height, (n - 1) * h, h)
    f = random_field((n, n, n), 0.002 / h, 0.03, rng)
    c = 1500.0 * (1.0 + f)
    dt = 0.3 * h / float(c.max())
    return Problem("cylinder3d", geom, c, 1.0 / c ** 2, np.full((n, n, n), 1.0 / 1500.0 ** 2), h,
                   dt, nt, ricker(nt, dt, f0), f0)


def cylinder3d_large(seed=0):
    return cylinder3d(seed, n=320, h=0.12e-3, n_rings=16, per_ring=32, nt=3000)


def gn3d(seed=0, n=224, h=0.18e-3, n_rings=8, per_ring=32, nt=2500, f0=1e6):
    p = cylinder3d(seed, n=n, h=h, n_rings=n_rings, per_ring=per_ring, nt=nt, f0=f0)
    rng = np.random.default_rng(seed + 1)
    p.v = random_field(p.shape, 0.002 / h, 1.0, rng) * float(np.mean(p.m0)) * 0.01
    p.name = "gn3d"
    return p
