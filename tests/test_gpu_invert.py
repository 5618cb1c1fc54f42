"""The device-resident FWI loop (openusct_gb300.invert) and its update kernels.

* usct_smooth_dev == scipy.ndimage.gaussian_filter bit for bit; the
  elementwise update kernels == their NumPy expressions bit for bit; max|x|
  exact; dot/sum within a few ulps of NumPy;
* invert() on the device == the host restatement of fwi.invert
  (oracle/invert.py) driven by the same GB300 backend, for steepest descent
  (L2, GCN, windowed data) and Gauss-Newton: same accepted steps, the same
  history and model up to the last-bit differences of the device mean/dot;
* within the FP32 tolerance of the reference's own fwi.invert (invert2d
  fixture).
"""

import os

import numpy as np
import pytest

from golden_util import GOLDEN, load, rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from openusct_gb300 import build
    build.build()
    yield


def _ops(shape):
    from openusct_gb300.invert import ModelOps
    return ModelOps(shape, torch.device("cuda", 0))


@pytest.mark.parametrize("shape,sigma", [((61, 61), 1.0), ((24, 31, 19), 1.0), ((5, 40), 2.0),
                                         ((3, 4, 5), 1.5), ((33, 20, 7), 0.3)])
def test_smoothing_is_scipy_bit_for_bit(shape, sigma):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(11)
    x = rng.standard_normal(shape)
    ops = _ops(shape)
    xd = torch.from_numpy(x).cuda()
    out = ops.empty()
    ops.smooth(xd, out, sigma)
    assert np.array_equal(out.cpu().numpy(), gaussian_filter(x, sigma))


def test_update_kernels_match_numpy():
    rng = np.random.default_rng(12)
    shape = (37, 29, 23)
    m, d = rng.standard_normal(shape), rng.standard_normal(shape)
    mask = (rng.random(shape) > 0.3).astype(float)
    lo, hi = np.full(shape, -0.5), np.full(shape, 0.7)
    ops = _ops(shape)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()   # noqa: E731
    out = ops.empty()
    ops.mul(T(m), T(mask), out)
    assert np.array_equal(out.cpu().numpy(), m * mask)
    ops.axpy(T(m), 0.37, T(d), out)
    assert np.array_equal(out.cpu().numpy(), m + 0.37 * d)
    ops.axpy(None, -1.0, T(d), out)
    assert np.array_equal(out.cpu().numpy(), -d)
    step = 0.123
    ops.trial(T(m), -step, T(d), T(lo), T(hi), T(mask), out)
    mt = m + step * (-d)
    want = np.where(mask > 0, np.clip(mt, lo, hi), mt)
    assert np.array_equal(out.cpu().numpy(), want)
    ops.trial(T(m), step, T(d), T(lo), T(hi), None, out)
    assert np.array_equal(out.cpu().numpy(), np.clip(m + step * d, lo, hi))
    ops.trial(T(m), step, T(d), None, None, T(mask), out)
    assert np.array_equal(out.cpu().numpy(), m + step * d)
    assert ops.absmax(T(d)) == float(np.max(np.abs(d)))
    assert abs(ops.dot(T(m), T(d)) - float(m.ravel() @ d.ravel())) <= 1e-12 * np.abs(m * d).sum()
    assert abs(ops.mean(T(m)) - float(np.mean(m))) <= 1e-14 * np.abs(m).mean()
    # reproducible: a second reduction gives the same bits
    assert ops.dot(T(m), T(d)) == ops.dot(T(m), T(d))


RUNS = {"gd": dict(n_iter=3), "gcn": dict(n_iter=2, misfit_type="gcn"), "tw": dict(n_iter=2),
        "gn": dict(n_iter=1, optimizer="gauss-newton", n_cg=3)}


@pytest.mark.parametrize("key", sorted(RUNS))
def test_device_invert_equals_host_loop_and_reference(key):
    import openusct_gb300.backend as gb
    from openusct_gb300.invert import invert
    from oracle.invert import invert as host_invert
    c = load("invert2d")
    kw = dict(RUNS[key])
    if key == "tw":
        kw["time_weights"] = c["tw"]
    common = dict(src_list=c.src_list, update_mask=c["mask"],
                  m_bounds=(float(c["lo"]), float(c["hi"])), step_frac=0.03)
    m, hist = invert(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], **common, **kw)
    mh, hh = host_invert(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], backend=gb,
                         **common, **kw)
    assert len(hist) == len(hh)
    assert np.max(np.abs(np.asarray(hist) - hh) / np.asarray(hh)) < 1e-9
    assert rel_l2(m - c["m0"], mh - c["m0"]) < 1e-9
    # the reference's own inversion, within FP32 tolerance
    ref = c["hist_" + key]
    assert len(hist) == len(ref)
    assert np.max(np.abs(np.asarray(hist) - ref) / ref) < 1e-3
    assert rel_l2(m - c["m0"], c["m_" + key] - c["m0"]) < 1e-3


def test_evaluator_reuses_the_trial_forward_bit_exactly():
    """The inversion's evaluator: a trial misfit followed by the gradient at
    the same model (only the backward sweep runs) gives J and g bit-identical
    to backend.misfit_and_gradient -- L2 and GCN, one shot batch (the forward
    is kept) and several (it is not) -- and so does a gradient call without a
    trial before it."""
    import openusct_gb300.backend as gb
    from openusct_gb300.invert import _Evaluator
    c = load("invert2d")
    dev = torch.device("cuda", 0)
    m = torch.from_numpy(c["m0"]).to(dev)
    for batch, mt in ((None, "l2"), (None, "gcn"), (1, "l2")):
        ev = _Evaluator(gb, m, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], None, c.src_list,
                        mt, None, None, batch=batch)
        assert ev.single == (batch is None)
        Jr, gr = gb.misfit_and_gradient(m, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                        src_list=c.src_list, misfit_type=mt, batch=batch)
        Jt = ev.misfit(m)
        J, g = ev.misfit_and_gradient(m)
        assert Jt == Jr and J == Jr
        assert torch.equal(g, gr)
        J2, g2 = ev.misfit_and_gradient(m)
        assert J2 == Jr and torch.equal(g2, gr)
    # another call on the same (cached) plan between a trial and its gradient
    # leaves the kept state alone
    ev = _Evaluator(gb, m, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], None, c.src_list,
                    "l2", None, None)
    Jr, gr = gb.misfit_and_gradient(m, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                    src_list=c.src_list)
    ev.misfit(m)
    gb.misfit_and_gradient(m * 1.01, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                           src_list=c.src_list)
    J, g = ev.misfit_and_gradient(m)
    assert J == Jr and torch.equal(g, gr)


def test_device_invert_keeps_tensors_on_the_device():
    from openusct_gb300.invert import invert
    c = load("invert2d")
    m0 = torch.from_numpy(c["m0"]).cuda()
    m, hist = invert(m0, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], src_list=c.src_list,
                     n_iter=1, update_mask=torch.from_numpy(c["mask"]).cuda())
    assert isinstance(m, torch.Tensor) and m.is_cuda and m.dtype == torch.float64
    assert len(hist) == 2 and hist[1] < hist[0]


def test_gauss_newton_beats_gradient_descent():
    """simulation/tests/test_gauss_newton.py:54-75 on the device loop: after 4
    iterations Gauss-Newton (n_cg 8) reduces the misfit more than gradient
    descent, and below 5 %; the first iterations track the reference's."""
    from openusct_gb300.invert import invert
    c = load("gn_vs_gd2d")
    kw = dict(src_list=c.src_list, n_iter=4, update_mask=c["mask"])
    _, hist_gd = invert(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], **kw)
    _, hist_gn = invert(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                        optimizer="gauss-newton", n_cg=8, **kw)
    red_gd = hist_gd[-1] / hist_gd[0]
    red_gn = hist_gn[-1] / hist_gn[0]
    assert red_gn < red_gd
    assert red_gn < 0.05
    assert abs(hist_gd[1] / c["hist_gd"][1] - 1) < 1e-3
    assert abs(hist_gn[1] / c["hist_gn"][1] - 1) < 1e-2


def test_gcn_gradient_matches_finite_differences():
    """simulation/tests/test_gradient_gcn.py: the device GCN gradient against
    central differences of the FP64 GCN misfit at the reference's probes."""
    import oracle
    import openusct_gb300.backend as gb
    c = load("ring2d_point")
    m0 = c["m0"]
    _, g = gb.misfit_and_gradient(m0, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                  src_list=c.src_list, misfit_type="gcn")
    n = m0.shape[0]
    cc = n // 2
    for iy, ix in [(cc, cc), (cc + 5, cc), (cc, cc - 6)]:
        eps = 1e-3 * m0[iy, ix]
        mp = m0.copy()
        mp[iy, ix] += eps
        mm = m0.copy()
        mm[iy, ix] -= eps
        Jp = oracle.misfit(mp, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                           src_list=c.src_list, misfit_type="gcn")
        Jm = oracle.misfit(mm, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                           src_list=c.src_list, misfit_type="gcn")
        fd = (Jp - Jm) / (2 * eps)
        ad = g[iy, ix]
        assert abs(fd - ad) / max(abs(fd), abs(ad), 1e-30) < 0.05


def test_time_weights_unit_window_is_identity_and_mute_reduces_misfit():
    """simulation/tests/test_time_weights.py on the device: unit windows give
    the unwindowed misfit and gradient bit for bit; a real mute lowers the
    misfit and changes the gradient."""
    import openusct_gb300.backend as gb
    c = load("ring2d_window")
    args = (c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"])
    J0, g0 = gb.misfit_and_gradient(*args, src_list=c.src_list)
    ones = [np.ones((c.nt, len(c["idx"]))) for _ in c.src_list]
    J1, g1 = gb.misfit_and_gradient(*args, src_list=c.src_list, time_weights=ones)
    assert J1 == J0 and np.array_equal(g1, g0)
    J2, g2 = gb.misfit_and_gradient(*args, src_list=c.src_list, time_weights=list(c["tw"]))
    assert np.isfinite(J2) and np.isfinite(g2).all()
    assert J2 < J0
    assert rel_l2(g2, g0) > 1e-2     # (the gradient entries are far below allclose's atol)


def test_pipeline_simulate_then_fwi_plugin(tmp_path):
    """simulation/tests/test_pipeline.py:23-59: simulate the acquisition with
    openusct_gb300.acquire, round-trip it through the portable HDF5 file
    (openusct_gb300.dataset_io; FP32 traces on disk), reconstruct it through
    the "fwi" plugin entry (openusct_gb300.invert.fwi_from_dataset) from the
    flaw-free background; the misfit halves and the flaw is recovered slower
    than the background, as the reference's run does (pipeline2d)."""
    from openusct_gb300.acquire import simulate_dataset
    from openusct_gb300.geometry import IndexGeometry
    from openusct_gb300.invert import fwi_from_dataset, register
    z = np.load(os.path.join(GOLDEN, "pipeline2d.npz"))

    class Ring(IndexGeometry):
        pass

    ring = Ring([tuple(int(v) for v in r) for r in z["idx"]])
    ring.h = float(z["h"])
    ring.radius_m = float(z["radius_m"])
    ring.element_positions = z["element_pos"]
    ds = simulate_dataset(z["c_true"], ring, z["wavelet"], float(z["dt"]),
                          nominal_speed_m_s=3000.0)
    assert rel_l2(ds.data, z["data"]) < 1e-5
    path = str(tmp_path / "acq.h5")
    ds.save(path)
    loaded = type(ds).load(path)
    assert np.array_equal(loaded.data, ds.data.astype(np.float32))
    res = fwi_from_dataset(loaded, start_c=z["c_bg"], m_bounds=(float(z["lo"]), float(z["hi"])),
                           n_iter=6, step_frac=0.04)
    hist = res["history"]
    assert hist[-1] < 0.5 * hist[0]
    n = res["c"].shape[0]
    ix, iy = int(round(0.60 * (n - 1))), int(round(0.50 * (n - 1)))
    assert res["c"][iy, ix] < 2900.0
    ref = z["history"]
    assert len(hist) == len(ref)
    assert abs(hist[0] / ref[0] - 1) < 1e-4
    assert np.max(np.abs(np.asarray(hist) / ref - 1)) < 1e-2

    class _Registry:
        entries = {}

        def register(self, name, description="", output="image"):
            def deco(fn):
                self.entries[name] = (fn, output)
                return fn
            return deco

    reg = _Registry()
    register(reg)
    assert reg.entries["fwi"] == (fwi_from_dataset, "model")


def test_readme_quick_start_runs():
    """The README's quick start, as written there (n_iter shortened)."""
    from openusct_gb300 import backend as gb, problems
    from openusct_gb300.invert import invert
    p = problems.ring2d(seed=0)
    d = gb.forward_fmc(p.m_true, p.geom, p.wavelet, p.dt, p.h, p.nt)
    assert d.shape == (64, 1500, 64)
    J, g = gb.misfit_and_gradient(p.m0, p.geom, p.wavelet, p.dt, p.h, p.nt, d)
    assert J > 0 and g.shape == p.m0.shape
    m, hist = invert(p.m0, p.geom, p.wavelet, p.dt, p.h, p.nt, d, n_iter=2)
    assert hist[-1] < hist[0] and m.shape == p.m0.shape
