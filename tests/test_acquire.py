"""Dataset production: same fields as the reference's simulate_dataset."""

import os
import sys

import numpy as np
import pytest

import oracle
from golden_util import load
from openusct_gb300 import acquire
from openusct_gb300.geometry import RingGeometry, ricker

# the reference's Python package, when USCT_REFERENCE names the checkout
REF = os.path.join(os.environ.get("USCT_REFERENCE", ""), "simulation") \
    if os.environ.get("USCT_REFERENCE") else ""


def test_peak_frequency_and_fallback_dataset_fields():
    dt = 1e-7
    w = ricker(400, dt, 0.4e6)
    assert abs(acquire.peak_frequency(w, dt) - 0.4e6) < 0.05e6
    ring = RingGeometry(8, 0.024, 0.06, 1e-3)
    c = np.full((ring.n, ring.n), 1500.0)
    ds = acquire.simulate_dataset(c, ring, w, dt, 1500.0, src_list=[0, 3],
                                  forward=oracle.forward_fmc)
    assert ds.data.shape == (2, 400, 8) and ds.data.dtype == np.float64
    assert list(ds.tx_elements) == [0, 3]
    assert ds.sample_rate_hz == pytest.approx(1.0 / dt)
    assert np.allclose(ds.geometry.element_pos, ring.element_positions)
    assert ds.ground_truth["h_m"] == ring.h


@pytest.mark.skipif(not REF or not os.path.isdir(REF),
                    reason="USCT_REFERENCE does not name the reference checkout")
def test_matches_reference_simulate_dataset():
    sys.path.insert(0, REF)
    from ringfwi import acquire as ref_acquire
    from ringfwi.geometry import RingArray
    c = load("ring2d_point")
    ring = RingArray(8, 0.024, 0.06, 1e-3)
    cm = 1.0 / np.sqrt(c["m_true"])
    ref = ref_acquire.simulate_dataset(cm, ring, c.wavelet, c.dt, 1480.0, src_list=[0, 4])
    ours = acquire.simulate_dataset(cm, ring, c.wavelet, c.dt, 1480.0, src_list=[0, 4],
                                    forward=oracle.forward_fmc)
    assert type(ours).__name__ == "Dataset"
    assert np.abs(ours.data - ref.data).max() <= 1e-12 * np.abs(ref.data).max()
    for f in ("sample_rate_hz", "tx_centre_freq_hz", "nominal_speed_m_s"):
        assert getattr(ours, f) == getattr(ref, f)
    assert np.array_equal(ours.tx_elements, ref.tx_elements)
    assert np.array_equal(ours.geometry.element_pos, ref.geometry.element_pos)
    assert ours.geometry.array_type == ref.geometry.array_type
    assert np.array_equal(ours.ground_truth["c"], ref.ground_truth["c"])
