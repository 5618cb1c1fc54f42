"""Acquisition geometry on the finite-difference grid (host side).

The engine consumes elements as CSR lists of (row-major linear cell, weight).
``element_csr`` builds them from the reference's own geometry objects (anything
with an ``idx`` list of grid-index tuples -- ``RingArray``, ``CylinderArray``,
``GridArray`` in simulation/ringfwi/geometry.py) and, optionally, from the
finite-aperture footprints of ``build_footprints`` (geometry.py:212-278).

``RingGeometry`` / ``CylinderGeometry`` place elements exactly as the
reference's ``RingArray.__post_init__`` (geometry.py:39-50) and
``CylinderArray.__post_init__`` (geometry.py:103-123) do, for hosts where the
reference package is not installed; ``ricker`` is the wavelet of
simulation/ringfwi/sources.py:8-26.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def linear_indices(idx, shape) -> np.ndarray:
    """Row-major linear indices of grid-index tuples (software/python/uap.py:19-22)."""
    idx = np.asarray(idx, dtype=np.int64).reshape(len(idx), -1)
    if idx.shape[1] != len(shape):
        raise ValueError(f"element indices have {idx.shape[1]} axes, grid has {len(shape)}")
    if np.any(idx < 0) or np.any(idx >= np.asarray(shape)[None, :]):
        raise ValueError("element index outside the grid")
    strides = np.cumprod((1,) + tuple(int(s) for s in shape[::-1][:-1]))[::-1]
    return (idx * strides[None, :]).sum(axis=1).astype(np.int64)


@dataclass
class CSR:
    ptr: np.ndarray    # int32 [rows+1]
    cell: np.ndarray   # int64 [entries]
    w: np.ndarray      # float64 [entries]

    @property
    def rows(self) -> int:
        return len(self.ptr) - 1

    def key(self) -> bytes:
        return self.ptr.tobytes() + b"|" + self.cell.tobytes() + b"|" + self.w.tobytes()


def _groups_csr(groups, shape) -> CSR:
    ptr = [0]
    cells, ws = [], []
    for idxs, w in groups:
        lin = linear_indices(list(idxs), shape)
        w = np.asarray(w, dtype=np.float64).reshape(-1)
        if len(w) != len(lin):
            raise ValueError("footprint weights and cells differ in length")
        cells.append(lin)
        ws.append(w)
        ptr.append(ptr[-1] + len(lin))
    return CSR(np.asarray(ptr, np.int32),
               np.concatenate(cells) if cells else np.zeros(0, np.int64),
               np.concatenate(ws) if ws else np.zeros(0, np.float64))


def element_csr(geom, shape, src_list=None, footprints=None):
    """Transmit and receive CSR lists for ``forward_fmc`` semantics.

    Every listed element transmits in turn and all elements receive
    (fwi.py:109-118); with ``footprints`` each element is its aperture's cell
    list with weights summing to one, on transmit and on receive (fwi.py:84-89,
    74-76), otherwise a single cell of weight 1.
    """
    idx = list(geom.idx) if hasattr(geom, "idx") else list(geom)
    n_el = len(idx)
    if footprints is not None and len(footprints) != n_el:
        raise ValueError("one footprint per element is required")
    if src_list is None:
        src_list = list(range(n_el))
    src = np.asarray([int(s) for s in src_list], np.int64)
    for s in src:
        if not 0 <= s < n_el:
            raise ValueError(f"src_list entry {s} outside 0..{n_el - 1}")
    if n_el == 0:
        rx = _groups_csr([], shape)
    elif footprints is None:        # one cell of weight 1 per element
        rx = CSR(np.arange(n_el + 1, dtype=np.int32), linear_indices(idx, shape),
                 np.ones(n_el, np.float64))
    else:
        rx = _groups_csr([(list(c), list(w)) for c, w in footprints], shape)
    return _select_rows(rx, src), rx


def _select_rows(c: CSR, rows) -> CSR:
    """The listed rows of ``c``, in the listed order (rows may repeat)."""
    rows = np.asarray(rows, np.int64)
    lens = (c.ptr[1:] - c.ptr[:-1])[rows].astype(np.int64)
    ptr = np.zeros(len(rows) + 1, np.int64)
    np.cumsum(lens, out=ptr[1:])
    at = np.arange(int(ptr[-1]), dtype=np.int64) - np.repeat(ptr[:-1], lens) \
        + np.repeat(c.ptr[:-1][rows].astype(np.int64), lens)
    return CSR(ptr.astype(np.int32), c.cell[at].astype(np.int64), c.w[at].astype(np.float64))


# ---------------------------------------------------------------------------
# element placement (same formulas as the reference geometry classes)
# ---------------------------------------------------------------------------
@dataclass
class RingGeometry:
    """Planar ring of ``n_elements`` on a square grid (RingArray semantics)."""

    n_elements: int
    radius_m: float
    domain_m: float
    h: float
    idx: list = field(init=False)
    n: int = field(init=False)
    array_type = "ring"

    def __post_init__(self):
        self.n = int(round(self.domain_m / self.h)) + 1
        c = self.domain_m / 2.0
        ang = np.linspace(0.0, 2.0 * np.pi, self.n_elements, endpoint=False)
        self.xy = np.column_stack([c + self.radius_m * np.cos(ang), c + self.radius_m * np.sin(ang)])
        self.idx = [(int(round(y / self.h)), int(round(x / self.h))) for x, y in self.xy]

    @property
    def grid_shape(self):
        return (self.n, self.n)

    def element_index(self, k):
        return self.idx[k]

    @property
    def element_positions(self):
        return self.xy - self.domain_m / 2.0


@dataclass
class CylinderGeometry:
    """Rings stacked along z on a cubic grid (CylinderArray semantics)."""

    n_rings: int
    per_ring: int
    radius_m: float
    height_m: float
    domain_m: float
    h: float
    idx: list = field(init=False)
    n: int = field(init=False)
    array_type = "cylinder"

    def __post_init__(self):
        self.n = int(round(self.domain_m / self.h)) + 1
        c = self.domain_m / 2.0
        if self.n_rings == 1:
            zs = np.array([c])
        else:
            zs = c + np.linspace(-self.height_m / 2.0, self.height_m / 2.0, self.n_rings)
        ang = np.linspace(0.0, 2.0 * np.pi, self.per_ring, endpoint=False)
        xyz = [[c + self.radius_m * np.cos(a), c + self.radius_m * np.sin(a), z] for z in zs for a in ang]
        self.xyz = np.asarray(xyz)
        self.idx = [(int(round(z / self.h)), int(round(y / self.h)), int(round(x / self.h)))
                    for x, y, z in self.xyz]

    @property
    def n_elements(self):
        return len(self.idx)

    @property
    def grid_shape(self):
        return (self.n, self.n, self.n)

    def element_index(self, k):
        return self.idx[k]

    @property
    def element_positions(self):
        return self.xyz - self.domain_m / 2.0


def fibonacci_directions(n, hemisphere=False):
    """n near-uniform unit vectors on the sphere (or its upper half) along a
    golden-angle spiral (geometry.py:140-147): cos(polar) steps uniformly,
    azimuth advances by pi (1 + sqrt 5) per element."""
    i = np.arange(n) + 0.5
    cz = (1.0 - i / n) if hemisphere else (1.0 - 2.0 * i / n)
    rr = np.sqrt(np.clip(1.0 - cz * cz, 0.0, 1.0))
    az = np.pi * (1.0 + 5.0 ** 0.5) * i
    return np.column_stack([rr * np.cos(az), rr * np.sin(az), cz])


@dataclass
class ShellGeometry:
    """Elements on a spherical shell or its upper half (ShellArray, SphereArray,
    HemisphereArray semantics, geometry.py:150-196), on a cubic grid."""

    n_elements: int
    radius_m: float
    domain_m: float
    h: float
    hemisphere: bool = False
    idx: list = field(init=False)
    n: int = field(init=False)

    def __post_init__(self):
        self.n = int(round(self.domain_m / self.h)) + 1
        c = self.domain_m / 2.0
        self.xyz = c + self.radius_m * fibonacci_directions(self.n_elements, self.hemisphere)
        self.idx = [(int(round(z / self.h)), int(round(y / self.h)), int(round(x / self.h)))
                    for x, y, z in self.xyz]

    @property
    def grid_shape(self):
        return (self.n, self.n, self.n)

    def element_index(self, k):
        return self.idx[k]

    @property
    def element_positions(self):
        return self.xyz - self.domain_m / 2.0

    @property
    def array_type(self):
        return "hemisphere" if self.hemisphere else "sphere"


def tangent_basis(normal):
    """Unit vector(s) spanning the plane normal to ``normal``: one in 2D (the
    normal turned by 90 degrees), two in 3D from cross products with the z axis
    (the x axis when the normal is within ~25 degrees of z) (geometry.py:199-209)."""
    normal = np.asarray(normal, float)
    if normal.size == 2:
        return [np.array([-normal[1], normal[0]])]
    ax = np.array([0.0, 0.0, 1.0])
    if abs(np.dot(normal, ax)) > 0.9:
        ax = np.array([1.0, 0.0, 0.0])
    u = np.cross(normal, ax)
    u /= np.linalg.norm(u)
    return [u, np.cross(normal, u)]


def build_footprints(geom, width_m, shape="flat", height_m=None, max_pts=9):
    """Finite-aperture footprints on the grid (geometry.build_footprints,
    geometry.py:212-278): each element is a flat aperture in the plane tangent to
    the array surface -- "rect" (width x height; in 2D a segment), "disc" (an
    ellipse with those axes), "flat" (a width x width square) or "point" (also
    any aperture no wider than a cell) -- sampled on an up to ``max_pts``-point
    grid per axis, snapped to the nearest cells (clipped to the grid), each cell
    once in first-hit order, equal weights summing to one.  For cylinders the
    normal is radial in the ring plane, so width runs around the ring and height
    along its axis.  Returns a list over elements of (idx_list, weights)."""
    pos = np.asarray(geom.element_positions, float)
    dim = pos.shape[1]
    half = geom.domain_m / 2.0
    h = geom.h
    n = geom.n
    if height_m is None or shape == "flat":
        height_m = width_m
    as_point = shape == "point" or (width_m <= h and height_m <= h)
    cylinder = getattr(geom, "array_type", "") == "cylinder"

    def samples(extent):
        npt = int(np.clip(round(extent / h) + 1, 1, max_pts))
        return np.linspace(-extent / 2.0, extent / 2.0, npt) if npt > 1 else np.zeros(1)

    out = []
    for k in range(len(pos)):
        if as_point:
            out.append(([geom.element_index(k)], np.array([1.0])))
            continue
        p = pos[k]
        radial = p.copy()
        if cylinder:
            radial[2] = 0.0
        norm = np.linalg.norm(radial)
        normal = radial / norm if norm > 0 else np.eye(dim)[0]
        tangents = tangent_basis(normal)
        extents = [width_m] + ([height_m] if len(tangents) > 1 else [])
        axes = [samples(e) for e in extents]
        cells = {}
        for off in np.array(np.meshgrid(*axes)).reshape(len(axes), -1).T:
            if shape == "disc":
                u = off[0] / (width_m / 2.0 + 1e-30)
                v = (off[1] / (height_m / 2.0 + 1e-30)) if len(off) > 1 else 0.0
                if u * u + v * v > 1.0 + 1e-9:
                    continue
            disp = sum(o * t for o, t in zip(off, tangents))
            xyz = p + half + disp
            cell = tuple(int(np.clip(round(xyz[d] / h), 0, n - 1)) for d in range(dim - 1, -1, -1))
            cells[cell] = True
        idx_list = list(cells.keys())
        out.append((idx_list, np.full(len(idx_list), 1.0 / len(idx_list))))
    return out


@dataclass
class IndexGeometry:
    """Elements given directly as grid-index tuples (GridArray semantics)."""

    idx: list

    @property
    def n_elements(self):
        return len(self.idx)

    def element_index(self, k):
        return self.idx[k]


def footprints_from_csr(ptr, cells, w):
    """(idx_list, weights) list from a CSR of grid-index tuples."""
    out = []
    for a, b in zip(ptr[:-1], ptr[1:]):
        out.append(([tuple(int(v) for v in c) for c in cells[a:b]], np.asarray(w[a:b], float)))
    return out


def ricker(nt, dt, f0, t0=None):
    """Ricker wavelet (1 - 2a) exp(-a), a = (pi f0 (t - t0))^2, t0 = 1/f0."""
    if t0 is None:
        t0 = 1.0 / f0
    t = np.arange(nt) * dt - t0
    a = (math.pi * f0 * t) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def make_sponge(shape, width=25, strength=0.08):
    """Multiplicative damping mask for the ``sponge=`` argument
    (solver.make_sponge, simulation/ringfwi/solver.py:22-42): 1 in the
    interior; on the k-th cell from an edge (k < width) of every axis the
    factor exp(-(strength * (width - k))^2).  A 2D mask is the outer product
    of the row and column profiles, equal to the reference's; for 3D grids the
    three axis profiles multiply (the reference builds 2D masks only).  As in
    the reference, an axis shorter than ``width`` is an error."""
    shape = tuple(int(n) for n in shape)
    if len(shape) not in (2, 3):
        raise ValueError("make_sponge needs a 2D or 3D shape")
    k = np.arange(width)
    ramp = np.exp(-((strength * (width - k)) ** 2))

    def axis(n):
        if n < width or width < 1:
            raise ValueError(f"axis of {n} cells cannot hold a {width}-cell sponge")
        f = np.ones(n)
        f[:width] = ramp
        f[n - width:] = ramp[::-1]
        return f

    mask = np.outer(axis(shape[-2]), axis(shape[-1]))
    if len(shape) == 3:
        mask = axis(shape[0])[:, None, None] * mask[None, :, :]
    return mask
