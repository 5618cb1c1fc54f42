"""Host-side logic: element placement, CSR construction, batching arithmetic."""

import numpy as np
import pytest

from golden_util import load
from openusct_gb300 import geometry
from openusct_gb300.backend import batch_bytes_estimate, choose_batch


def test_ring_geometry_matches_reference_placement():
    # the golden ring was made by ringfwi.geometry.RingArray(8, 0.024, 0.06, 1e-3)
    c = load("ring2d_point")
    ring = geometry.RingGeometry(8, 0.024, 0.06, 1e-3)
    assert ring.n == c["m0"].shape[0]
    assert [tuple(t) for t in ring.idx] == [tuple(int(v) for v in r) for r in c["idx"]]


def test_cylinder_geometry_matches_reference_placement():
    c = load("cyl3d_point")
    cyl = geometry.CylinderGeometry(2, 6, 0.010, 0.012, 0.03, 1.5e-3)
    assert cyl.n == c["m0"].shape[0]
    assert [tuple(t) for t in cyl.idx] == [tuple(int(v) for v in r) for r in c["idx"]]


def test_ricker_matches_reference_wavelet():
    c = load("ring2d_point")
    w = geometry.ricker(c.nt, c.dt, 0.4e6)
    assert np.array_equal(w, c.wavelet)


def test_linear_indices_row_major():
    shape = (5, 7, 11)
    idx = [(0, 0, 0), (4, 6, 10), (2, 3, 4)]
    lin = geometry.linear_indices(idx, shape)
    assert list(lin) == [int(np.ravel_multi_index(t, shape)) for t in idx]
    with pytest.raises(ValueError):
        geometry.linear_indices([(5, 0, 0)], shape)


def test_element_csr_points_and_src_list():
    g = geometry.IndexGeometry([(1, 2), (3, 4), (5, 6)])
    tx, rx = geometry.element_csr(g, (8, 9), src_list=[2, 0])
    assert list(tx.ptr) == [0, 1, 2] and list(tx.cell) == [5 * 9 + 6, 1 * 9 + 2]
    assert list(rx.ptr) == [0, 1, 2, 3] and np.all(rx.w == 1.0)
    with pytest.raises(ValueError):
        geometry.element_csr(g, (8, 9), src_list=[3])


def test_element_csr_footprints():
    c = load("ring2d_aperture")
    tx, rx = geometry.element_csr(c.geom, c["m0"].shape, c.src_list, c.footprints)
    assert rx.rows == len(c.footprints)
    assert tx.rows == len(c.src_list)
    for j, (cells, w) in enumerate(c.footprints):
        a, b = rx.ptr[j], rx.ptr[j + 1]
        assert b - a == len(cells)
        assert np.isclose(rx.w[a:b].sum(), 1.0)
        assert list(rx.cell[a:b]) == list(geometry.linear_indices(cells, c["m0"].shape))


def test_batch_choice_respects_budget():
    shape, nt = (192, 192, 192), 2000
    full = batch_bytes_estimate(shape, nt, 256, 256, 32, 64, 1)
    # 32 shots x (4 + 2*32 + 64) levels of 28.3 MB
    assert 110e9 < full < 125e9
    assert choose_batch(shape, nt, 256, 256, 256, 64, 1, full) == 32
    assert choose_batch(shape, nt, 256, 256, 256, 64, 1, full - 1) == 16
    assert choose_batch((61, 61), 350, 2, 8, 8, 0, 1, 1 << 40) == 2
