"""TFM imaging on the GPU (openusct_gb300.imaging) against the reference.

* the analytic-signal kernel against scipy.signal.hilbert (FP32 tolerance);
* the travel-time sample indices are the reference's exactly (the image of
  unit impulses placed at the oracle's indices);
* the TFM images of the tfm2d / tfm3d fixtures (made by the reference's own
  imaging.tfm) within 1e-5 relative L2, envelope and real part, same peak;
* the reference's own check (test_imaging.py:41-50): the 2D point scatterer
  is focused within 4 mm; the plugin registry runs it.
"""

import os

import numpy as np
import pytest

from golden_util import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from openusct_gb300 import build
    build.build()
    yield


class _Geom:
    def __init__(self, pos, radius):
        self.element_pos = pos
        self.radius_m = radius
        self.dim = pos.shape[1]


class _Dataset:
    def __init__(self, z):
        self.data = z["data"]
        self.geometry = _Geom(z["element_pos"], float(z["radius_m"]))
        self.tx_elements = z["tx_elements"]
        self.nominal_speed_m_s = float(z["c"])
        self.sample_rate_hz = float(z["fs"])


@pytest.mark.parametrize("shape", [(3, 320, 5), (2, 97, 3), (1, 1500, 64), (4, 64, 17),
                                   (2, 10, 3), (1, 7, 40), (3, 2, 1), (1, 1, 2)])
def test_analytic_signal_matches_scipy(shape):
    from scipy.signal import hilbert
    from openusct_gb300.imaging import analytic_signal
    rng = np.random.default_rng(6)
    x = rng.standard_normal(shape)
    a = analytic_signal(x).cpu().numpy()                   # (n_tx, n_rx, nt)
    ref = np.transpose(hilbert(x, axis=1), (0, 2, 1))
    assert np.array_equal(a.real, x.astype(np.float32).transpose(0, 2, 1))
    # (for nt <= 2 the imaginary part vanishes: scale by the data instead)
    scale = max(np.linalg.norm(ref.imag), np.linalg.norm(x))
    err = np.linalg.norm(a.imag - ref.imag) / scale
    assert err < 1e-5, err


def test_analytic_real_part_rounds_like_numpy():
    """The FP64 -> FP32 conversion of the samples (integer arithmetic on the
    device) equals NumPy's round-to-nearest-even for ties, overflow, the
    subnormal range, signed zeros, infinities and NaN."""
    from openusct_gb300.imaging import analytic_signal
    f = np.float32
    one = 1.0
    vals = [0.0, -0.0, one + 2.0 ** -24, one + 3 * 2.0 ** -24, -(one + 2.0 ** -24),
            2.0 ** -23 * 3 + 1, float(np.finfo(f).max) * (1 + 2.0 ** -25),
            float(np.finfo(f).max) * (1 + 2.0 ** -24), float(np.finfo(f).max),
            2.0 ** -126, 2.0 ** -126 * (1 - 2.0 ** -25), 2.0 ** -140, 2.0 ** -149,
            2.0 ** -150, 2.0 ** -151, 1e-300, -1e-300, 1e300, -1e300, np.inf, -np.inf, np.nan,
            1.0000000596046448, 16777217.0, -16777219.0, 3.4e38, 1.1754942e-38]
    rng = np.random.default_rng(4)
    vals += list(rng.standard_normal(37) * 10.0 ** rng.integers(-40, 40, 37))
    x = np.array(vals, np.float64).reshape(1, -1, 1)
    with np.errstate(over="ignore"):
        want = x.astype(np.float32).ravel()
    got = analytic_signal(x).real.cpu().numpy().ravel()
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))


@pytest.mark.parametrize("name", ["tfm2d", "tfm3d"])
def test_tfm_matches_reference(name):
    from openusct_gb300.imaging import tfm
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    ds = _Dataset(z)
    img, axes = tfm(ds, npix=int(z["npix"]), half_size=float(z["half"]))
    assert img.shape == z["image"].shape
    assert np.array_equal(np.stack(axes), z["axes"])
    assert rel_l2(img, z["image"]) < 1e-5
    # the same peak (the 3D image has near-ties: compare the value at the
    # reference's peak with the maximum)
    assert img.flat[int(np.argmax(z["image"]))] >= img.max() * (1 - 1e-5)
    img_re, _ = tfm(ds, npix=int(z["npix"]), half_size=float(z["half"]), envelope=False)
    assert rel_l2(img_re, z["image_re"]) < 1e-5


def test_tfm_sample_indices_are_the_references():
    """Data with a unit real sample at one (tx, rx, k) and zero elsewhere: the
    real image counts, per pixel, the pairs whose index hits that sample --
    equal to the oracle's np.round indices everywhere."""
    import oracle.tfm as otfm
    from openusct_gb300.imaging import tfm
    z = np.load(os.path.join(GOLDEN, "tfm2d.npz"))
    npix = 41
    idx = otfm.sample_indices(z["data"].shape, z["element_pos"], z["tx_elements"],
                              float(z["c"]), float(z["fs"]), float(z["radius_m"]), npix,
                              float(z["half"]))
    rng = np.random.default_rng(7)
    for _ in range(6):
        i, j = int(rng.integers(0, idx.shape[1])), int(rng.integers(0, idx.shape[2]))
        k = int(idx[int(rng.integers(0, idx.shape[0])), i, j])
        ds = _Dataset(z)
        ds.data = np.zeros_like(z["data"])
        ds.data[i, k, j] = 1.0
        img_re, _ = tfm(ds, npix=npix, half_size=float(z["half"]), envelope=False)
        want = (idx[:, i, j] == k).astype(float).reshape(npix, npix)
        # the real part of the analytic signal is the data itself
        assert np.array_equal(img_re, want)


def test_tfm_focuses_the_point_scatterer_and_runs_as_plugin():
    from openusct_gb300.imaging import register, tfm
    z = np.load(os.path.join(GOLDEN, "tfm2d.npz"))
    ds = _Dataset(z)
    img, axes = tfm(ds, npix=81, half_size=0.018)
    ix, iy = np.unravel_index(int(np.argmax(img)), img.shape)
    peak = np.array([axes[0][ix], axes[1][iy]])
    assert float(np.hypot(*(peak - z["true_pos"]))) < 0.004

    class _Registry:
        def __init__(self):
            self.entries = {}

        def register(self, name, description="", output="image"):
            def deco(fn):
                self.entries[name] = fn
                return fn
            return deco

    reg = _Registry()
    register(reg)
    out = reg.entries["tfm"](ds, npix=41, half_size=0.018)
    assert out.shape == (41, 41)


@pytest.mark.parametrize("case,key", [("ring2d_point", "point"), ("parity2d", "parity")])
def test_p_window_weights_match_reference(case, key):
    """fwi.p_window_weights (fwi.py:663-699) on the device: the windows of the
    reference (pwindow2d fixture) on the same data.  The envelope is FP32 on
    the device, so an onset may move by a sample where the envelope crosses
    the threshold within FP32 rounding; every other window is equal to 1e-12."""
    from openusct_gb300.imaging import p_window_weights
    ref = np.load(os.path.join(GOLDEN, "pwindow2d.npz"))
    d = np.load(os.path.join(GOLDEN, f"{case}.npz"))["dobs"]
    W = np.asarray(p_window_weights(d, float(ref[f"dt_{key}"]), float(ref[f"f0_{key}"])))
    Wr = ref[f"W_{key}"]
    assert W.shape == Wr.shape
    same = np.all(np.abs(W - Wr) <= 1e-12, axis=1)          # per (transmit, receiver) trace
    assert same.mean() >= 0.98, same.mean()


def test_tfm_at_the_c1_acquisition_size_matches_the_oracle():
    """The C1 acquisition (64-element ring r = 16 mm, 64 x 1500 x 64 FMC,
    120 x 120 pixels) with seeded data: GPU image against the oracle's
    restatement of imaging.tfm (which equals the reference bit for bit)."""
    import oracle.tfm as otfm
    from openusct_gb300.geometry import RingGeometry
    from openusct_gb300.imaging import tfm
    h = 0.15e-3
    ring = RingGeometry(64, 0.016, 255 * h, h)
    dt = 0.3 * h / 1580.0
    rng = np.random.default_rng(0)
    data = rng.standard_normal((64, 1500, 64))
    pos = np.asarray(ring.element_positions, np.float64)

    class DS:
        pass
    ds = DS()
    ds.data = data
    ds.geometry = _Geom(pos, 0.016)
    ds.tx_elements = np.arange(64)
    ds.nominal_speed_m_s = 1500.0
    ds.sample_rate_hz = 1.0 / dt
    img, _ = tfm(ds, npix=120)
    ref, _ = otfm.tfm(data, pos, np.arange(64), 1500.0, 1.0 / dt, 0.016, 120)
    assert rel_l2(img, ref) < 1e-5


def test_tfm_with_more_receivers_than_one_distance_chunk():
    """Over 256 receivers the kernel holds the receiver distances in chunks of
    256 (each transmit's sum is then split at the chunk boundary, in FP32):
    the image still equals the oracle's restatement of imaging.tfm."""
    import oracle.tfm as otfm
    from openusct_gb300.imaging import tfm
    rng = np.random.default_rng(11)
    n_el, n_tx, nt, npix = 330, 3, 256, 20
    a = 2 * np.pi * np.arange(n_el) / n_el
    pos = np.stack([0.02 * np.cos(a), 0.02 * np.sin(a)], axis=1)
    data = rng.standard_normal((n_tx, nt, n_el))

    class DS:
        pass
    ds = DS()
    ds.data = data
    ds.geometry = _Geom(pos, 0.02)
    ds.tx_elements = np.array([0, 110, 220])
    ds.nominal_speed_m_s = 1500.0
    ds.sample_rate_hz = 4.0e6
    img, _ = tfm(ds, npix=npix)
    ref, _ = otfm.tfm(data, pos, ds.tx_elements, 1500.0, 4.0e6, 0.02, npix)
    assert rel_l2(img, ref) < 1e-5
