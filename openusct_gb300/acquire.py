"""Dataset producer on the GB300 backend.

``simulate_dataset`` has the signature of the reference's
``ringfwi.acquire.simulate_dataset`` (simulation/ringfwi/acquire.py:18-68) --
which is hard-wired to the Python ``fwi.forward_fmc`` -- and returns the same
``Dataset`` (simulation/ringfwi/dataset.py:62-109): FMC data ``(n_tx, nt, n_rx)``
in FP64, sample rate 1/dt, the wavelet and its spectral peak frequency, the
element positions in metres about the array centre, and optionally the ground
truth.  When the reference package is importable its own ``Dataset`` and
``ArrayGeometry`` classes are used, so downstream code (``fwi_from_dataset``,
the ``fwi`` and ``tfm`` plugins, ``Dataset.save``) sees no difference;
otherwise field-for-field equivalents defined here are returned.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class ArrayGeometry:
    """Element positions in metres about the array centre (dataset.py:24-59)."""

    element_pos: np.ndarray
    radius_m: float
    centre_freq_hz: float
    array_type: str = "ring"

    @property
    def n_elements(self):
        return self.element_pos.shape[0]

    @property
    def dim(self):
        return self.element_pos.shape[1]


@dataclass
class Dataset:
    """FMC acquisition plus geometry and parameters (dataset.py:62-109)."""

    geometry: ArrayGeometry
    data: np.ndarray
    sample_rate_hz: float
    tx_wavelet: np.ndarray
    tx_centre_freq_hz: float
    nominal_speed_m_s: float
    tx_elements: np.ndarray | None = None
    ground_truth: dict | None = None
    metadata: dict = field(default_factory=dict)

    def __post_init__(self):
        self.tx_elements = (np.arange(self.data.shape[0]) if self.tx_elements is None
                            else np.asarray(self.tx_elements))

    @property
    def n_tx(self):
        return self.data.shape[0]

    @property
    def n_samples(self):
        return self.data.shape[1]

    @property
    def n_rx(self):
        return self.data.shape[2]

    @property
    def dt(self):
        return 1.0 / self.sample_rate_hz

    def save(self, path):
        """Write the platform's HDF5 Dataset file (dataset.py:112-140)."""
        from .dataset_io import save
        save(self, path)

    @classmethod
    def load(cls, path):
        """Read a Dataset file (dataset.py:142-174)."""
        from .dataset_io import load
        return load(path)


def _classes():
    try:
        from ringfwi.dataset import ArrayGeometry as RG, Dataset as RD
        return RG, RD
    except Exception:
        return ArrayGeometry, Dataset


def peak_frequency(wavelet, dt):
    """Frequency of the largest amplitude-spectrum bin (acquire.py:71-77)."""
    spec = np.abs(np.fft.rfft(wavelet))
    freqs = np.fft.rfftfreq(len(wavelet), dt)
    return float(freqs[int(np.argmax(spec))])


def simulate_dataset(c_model, array_geom, wavelet, dt, nominal_speed_m_s, src_list=None,
                     store_ground_truth=True, description="", footprints=None, sponge=None,
                     forward=None):
    """Simulate an FMC acquisition on the GB300 backend and return a Dataset.

    ``forward`` defaults to :func:`openusct_gb300.backend.forward_fmc` (any
    function with its signature may be passed).
    """
    if forward is None:
        from .backend import forward_fmc as forward
    c_model = np.asarray(c_model, dtype=np.float64)
    m = 1.0 / (c_model * c_model)
    data = forward(m, array_geom, wavelet, dt, array_geom.h, len(wavelet), sponge, src_list,
                   footprints)
    RG, RD = _classes()
    f0 = peak_frequency(wavelet, dt)
    geom = RG(element_pos=np.asarray(array_geom.element_positions), radius_m=array_geom.radius_m,
              centre_freq_hz=f0, array_type=getattr(array_geom, "array_type", "ring"))
    n_el = len(array_geom.idx)
    tx = list(range(n_el)) if src_list is None else list(src_list)
    gt = {"c": c_model, "h_m": array_geom.h} if store_ground_truth else None
    return RD(geometry=geom, data=np.asarray(data, dtype=np.float64), sample_rate_hz=1.0 / dt,
              tx_wavelet=wavelet, tx_centre_freq_hz=f0, nominal_speed_m_s=nominal_speed_m_s,
              tx_elements=tx, ground_truth=gt,
              metadata={"description": description, "created_by": "openusct_gb300 simulator"})
