"""Host restatement of the reference's TFM imaging -- TEST INFRASTRUCTURE ONLY.

``tfm`` follows ``ringfwi.imaging.tfm`` (simulation/ringfwi/imaging.py:27-74)
operation for operation in NumPy/scipy FP64: the centred image grid
(imaging.py:21-24, 47-49), point-to-element distances, the analytic signal
along time (scipy.signal.hilbert), and the delay-and-sum over (tx, rx) with
``np.round`` sample indices.  Pinned against the reference by the ``tfm2d`` /
``tfm3d`` golden fixtures.
"""

from __future__ import annotations

import numpy as np


def image_axes(radius_m, dim, npix, half_size=None):
    half = half_size if half_size is not None else radius_m * 0.95
    return [np.linspace(-half, half, npix) for _ in range(dim)]


def tfm(data, element_pos, tx_elements, c, fs, radius_m, npix=120, half_size=None,
        envelope=True):
    from scipy.signal import hilbert
    epos = np.asarray(element_pos, np.float64)
    dim = epos.shape[1]
    axes = image_axes(radius_m, dim, npix, half_size)
    grids = np.meshgrid(*axes, indexing="ij")
    pts = np.stack([g.ravel() for g in grids], axis=1)
    nt = data.shape[1]
    n_rx = data.shape[2]
    d = np.sqrt(((pts[:, None, :] - epos[None, :, :]) ** 2).sum(axis=2))
    analytic = hilbert(data, axis=1)
    acc = np.zeros(pts.shape[0], dtype=complex)
    for i, te in enumerate(np.asarray(tx_elements)):
        d_tx = d[:, te]
        for j in range(n_rx):
            t = (d_tx + d[:, j]) / c
            k = np.round(t * fs).astype(np.int64)
            valid = (k >= 0) & (k < nt)
            acc[valid] += analytic[i, k[valid], j]
    image = np.abs(acc) if envelope else acc.real
    return image.reshape([npix] * dim), axes


def sample_indices(data_shape, element_pos, tx_elements, c, fs, radius_m, npix, half_size=None):
    """The (P, n_tx, n_rx) int64 travel-time sample indices of tfm()."""
    epos = np.asarray(element_pos, np.float64)
    dim = epos.shape[1]
    axes = image_axes(radius_m, dim, npix, half_size)
    grids = np.meshgrid(*axes, indexing="ij")
    pts = np.stack([g.ravel() for g in grids], axis=1)
    d = np.sqrt(((pts[:, None, :] - epos[None, :, :]) ** 2).sum(axis=2))
    n_rx = data_shape[2]
    out = np.empty((pts.shape[0], len(tx_elements), n_rx), np.int64)
    for i, te in enumerate(np.asarray(tx_elements)):
        for j in range(n_rx):
            out[:, i, j] = np.round(((d[:, te] + d[:, j]) / c) * fs).astype(np.int64)
    return out
