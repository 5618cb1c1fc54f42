"""Total focusing method (delay-and-sum) imaging on the GB300.

``tfm`` has the signature and the result of the reference's
``ringfwi.imaging.tfm`` (simulation/ringfwi/imaging.py:27-74): the image of a
full-matrix capture on a centred ``npix^dim`` grid, summing every
transmit/receive pair's analytic-signal sample at the two-way travel time,
and its envelope.  The analytic signal and the sum run on the library's
kernels (``usct_analytic_dev``, ``usct_tfm_dev``); the travel-time sample
index is the reference's FP64 ``np.round((d_tx + d_rx) / c * fs)`` exactly.
The traces, the Hilbert transform and each transmit's sum over receivers are
FP32 (the reference's are FP64); the sum over transmits is FP64.

``register(plugins)`` installs it in the reference's plugin registry under
``"tfm"`` (plugins.py:55-59), so ``plugins.run("tfm", dataset)`` runs here.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

__all__ = ["image_axes", "hilbert_taps", "analytic_signal", "tfm", "p_window_weights",
           "register"]


def image_axes(dataset, npix, half_size=None):
    """Per-axis coordinate vectors of the centred image grid (imaging.py:21-24)."""
    half = half_size if half_size is not None else dataset.geometry.radius_m * 0.95
    return [np.linspace(-half, half, npix) for _ in range(dataset.geometry.dim)]


def hilbert_taps(nt):
    """g with hilbert(x) = x + i (x circularly convolved with g): the imaginary
    part of the inverse DFT of scipy.signal.hilbert's multiplier h (1 at DC and,
    for even nt, at Nyquist; 2 on the positive frequencies; 0 on the negative).
    For even nt that is (2/nt) cot(pi n / nt) at odd n and exactly 0 at even n
    (the analytic-signal kernel skips the zeros)."""
    if nt % 2 == 0:
        n = np.arange(nt)
        g = np.zeros(nt)
        odd = n % 2 == 1
        g[odd] = 2.0 / nt / np.tan(np.pi * n[odd] / nt)
        return g
    h = np.zeros(nt)
    h[0] = 1.0
    h[1:(nt + 1) // 2] = 2.0
    return np.ascontiguousarray(np.fft.ifft(h).imag)


def _p(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _dev():
    if not torch.cuda.is_available():
        raise RuntimeError("openusct_gb300 needs a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def analytic_signal(data, stream=None):
    """Analytic signal of FMC data (n_tx, nt, n_rx) along time, on the device:
    a CUDA complex64 tensor of shape (n_tx, n_rx, nt) (trace-major)."""
    lib = _lib.load()
    dev = _dev()
    d = data if isinstance(data, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(data))
    d = d.to(device=dev, dtype=torch.float64).contiguous()
    if d.ndim != 3:
        raise ValueError("data must be (n_tx, nt, n_rx)")
    n_tx, nt, n_rx = (int(s) for s in d.shape)
    taps = torch.from_numpy(hilbert_taps(nt).astype(np.float32)).to(dev)
    out = torch.empty((n_tx, n_rx, nt, 2), dtype=torch.float32, device=dev)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    _lib.check(lib.usct_analytic_dev(_p(d), _p(out), n_tx, nt, n_rx, _p(taps),
                                     ctypes.c_void_p(st.cuda_stream)))
    return torch.view_as_complex(out)


def tfm(dataset, npix=120, half_size=None, envelope=True):
    """Total focusing method image of a Dataset (imaging.py:27-74).

    Returns ``(image, axes)``: the ``(npix,)*dim`` FP64 image (envelope
    magnitude, or the real part with ``envelope=False``) and the coordinate
    vector of each axis in metres.
    """
    lib = _lib.load()
    dev = _dev()
    dim = int(dataset.geometry.dim)
    if dim not in (2, 3):
        raise ValueError("TFM needs 2D or 3D element positions")
    axes = image_axes(dataset, npix, half_size)
    epos = np.asarray(dataset.geometry.element_pos, np.float64)
    tx_elements = np.asarray(dataset.tx_elements, np.int64)
    data = dataset.data
    n_tx, nt, n_rx = (int(s) for s in np.shape(data))
    if len(tx_elements) != n_tx:
        raise ValueError("tx_elements does not match the data's transmit count")
    if n_rx > len(epos):
        raise ValueError("more receivers than element positions")
    tx_pos = epos[tx_elements]                       # IndexError for a bad element
    rx_pos = epos[:n_rx]
    A = analytic_signal(data)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(dev)  # noqa: E731
    txp, rxp, ax = T(tx_pos), T(rx_pos), T(np.stack(axes))
    npts = npix ** dim
    out_re = torch.empty(npts, dtype=torch.float64, device=dev)
    out_im = torch.empty(npts, dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev)
    _lib.check(lib.usct_tfm_dev(_p(torch.view_as_real(A)), n_tx, n_rx, nt, _p(txp), _p(rxp), dim,
                                _p(ax), int(npix), ctypes.c_double(dataset.nominal_speed_m_s),
                                ctypes.c_double(dataset.sample_rate_hz), _p(out_re), _p(out_im),
                                ctypes.c_void_p(st.cuda_stream)))
    re = out_re.cpu().numpy()
    im = out_im.cpu().numpy()
    image = np.hypot(re, im) if envelope else re
    return image.reshape([npix] * dim), axes


def p_window_weights(dobs, dt, f0, onset_frac=0.2, keep_cycles=2.5, taper_cycles=0.75,
                     as_tensor=False):
    """Per-trace P-arrival mute windows (fwi.p_window_weights, fwi.py:663-699)
    computed on the device: the onset is the first sample whose envelope
    exceeds ``onset_frac`` of the trace maximum; the window keeps
    ``keep_cycles`` of f0 after it and rolls off with a cosine over
    ``taper_cycles``.  Returns the reference's list of (nt, n_rx) arrays (or
    one CUDA (n_tx, nt, n_rx) tensor with ``as_tensor``), ready for
    ``time_weights``."""
    lib = _lib.load()
    dev = _dev()
    A = analytic_signal(dobs)
    n_tx, n_rx, nt = (int(s) for s in A.shape)
    keep = keep_cycles / f0 / dt
    taper = max(1.0, taper_cycles / f0 / dt)
    W = torch.empty((n_tx, nt, n_rx), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev)
    _lib.check(lib.usct_pwindow_dev(_p(torch.view_as_real(A)), n_tx, nt, n_rx,
                                    ctypes.c_double(onset_frac), ctypes.c_double(keep),
                                    ctypes.c_double(taper), _p(W),
                                    ctypes.c_void_p(st.cuda_stream)))
    if as_tensor:
        return W
    return list(W.cpu().numpy())


def register(plugins):
    """Install this TFM as the reference plugin registry's ``"tfm"`` entry
    (same parameters and return value as plugins.py:55-59)."""
    def _tfm(dataset, npix=120, half_size=None, envelope=True):
        image, _axes = tfm(dataset, npix=npix, half_size=half_size, envelope=envelope)
        return image
    plugins.register("tfm", description="Total focusing method (GB300)")(_tfm)
    return _tfm
