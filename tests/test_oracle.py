"""The oracle (oracle/usct_oracle.c) pinned against the reference.

* FP64 restatement == the reference's C++ core (software/core/libuap.hpp),
  bit for bit, on every point-element golden fixture;
* FP64 restatement ~= the reference's Python package (fwi.py) to 1e-12..1e-10
  (the two reference implementations sum the Laplacian in different orders);
* checkpointed recompute == full history, bit for bit;
* the FP32 kernel-order restatement stays within the FP32 tolerances of FP64;
* the reference's own finite-difference gradient checks (test_gradient.py,
  test_gradient_misfits.py patterns) hold for the oracle.
"""

import os

import numpy as np
import pytest

import oracle
from golden_util import CASES, GOLDEN, grad_tol, load, rel_l2, rel_max, trace_tol

POINT_CPP = ["ring2d_point", "cyl3d_point", "odd2d", "odd3d", "parity2d", "parity3d", "gpu3d"]


@pytest.mark.parametrize("name", CASES)
def test_forward_matches_reference_python(name):
    c = load(name)
    a = c.args()
    d = oracle.forward_fmc(c["m_true"], c.geom, a["wavelet"], c.dt, c.h, c.nt, a["sponge"],
                           a["src_list"], a["footprints"])
    assert rel_max(d, c["dobs"]) < 1e-12


@pytest.mark.parametrize("name", POINT_CPP)
def test_forward_bit_identical_to_reference_cpp(name):
    c = load(name)
    d = oracle.forward_fmc(c["m_true"], c.geom, c.wavelet, c.dt, c.h, c.nt, None, c.src_list)
    assert np.array_equal(d, c["dobs_cpp"])


@pytest.mark.parametrize("name", CASES)
def test_gradient_matches_reference_python(name):
    c = load(name)
    a = c.args()
    J, g = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                      a["sponge"], a["src_list"], a["footprints"])
    assert abs(J - float(c["J"])) <= 1e-12 * abs(float(c["J"]))
    assert rel_max(g, c["g"]) < 1e-10


@pytest.mark.parametrize("name", POINT_CPP)
def test_gradient_bit_identical_to_reference_cpp(name):
    c = load(name)
    J, g = oracle.misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                      None, c.src_list)
    assert J == float(c["J_cpp"])
    assert np.array_equal(g, c["g_cpp"])


@pytest.mark.parametrize("name", ["ring2d_point", "ring2d_sponge", "cyl3d_aperture", "odd3d"])
@pytest.mark.parametrize("k", [2, 7, 16])
def test_checkpoint_recompute_is_bit_exact(name, k):
    c = load(name)
    a = c.args()
    J0, g0 = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                        a["sponge"], a["src_list"], a["footprints"], k=0)
    Jk, gk = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                        a["sponge"], a["src_list"], a["footprints"], k=k)
    assert J0 == Jk
    assert np.array_equal(g0, gk)


def test_gauss_newton_matches_reference_python():
    c = load("gn2d")
    hv = oracle.gn_hessian_vector(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["v"],
                                  src_list=c.src_list, k=16)
    assert rel_max(hv, c["Hv"]) < 1e-10


@pytest.mark.parametrize("name", CASES)
def test_fp32_restatement_within_fp32_tolerance(name):
    c = load(name)
    a = c.args()
    d32 = oracle.forward_fmc32(c["m_true"], c.geom, a["wavelet"], c.dt, c.h, c.nt, a["sponge"],
                               a["src_list"], a["footprints"])
    assert rel_l2(d32, c["dobs"]) < trace_tol(name)
    J32, g32 = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                            c["dobs"], a["sponge"], a["src_list"],
                                            a["footprints"], C=2)
    assert abs(J32.sum() - float(c["J"])) <= 1e-4 * abs(float(c["J"]))
    assert rel_l2(g32, c["g"]) < grad_tol(name)


def test_fp32_gauss_newton_within_tolerance():
    c = load("gn2d")
    hv, born = oracle.gn_hessian_vector32(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["v"],
                                          src_list=c.src_list, C=2)
    assert rel_l2(hv, c["Hv"]) < 1e-4


def test_adjoint_matches_finite_difference():
    """simulation/tests/test_gradient.py:43-71 applied to the oracle."""
    c = load("ring2d_point")
    _, g = oracle.misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                      None, c.src_list)
    n = c["m0"].shape[0]
    cc = n // 2
    for p in [(cc, cc), (cc + 5, cc)]:
        eps = 1e-3 * c["m0"][p]
        mp = c["m0"].copy(); mp[p] += eps
        mm = c["m0"].copy(); mm[p] -= eps
        Jp = oracle.misfit(mp, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], src_list=c.src_list)
        Jm = oracle.misfit(mm, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], src_list=c.src_list)
        fd = (Jp - Jm) / (2 * eps)
        assert abs(fd - g[p]) / max(abs(fd), abs(g[p])) < 0.05


def test_directional_derivative_matches():
    """Seeded random direction, border zeroed (test_gradient_misfits.py:38-59)."""
    c = load("odd2d")
    m0 = c["m0"]
    J0, g = oracle.misfit_and_gradient(m0, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                       None, c.src_list)
    rng = np.random.default_rng(1)
    dm = rng.standard_normal(m0.shape)
    dm[:5, :] = dm[-5:, :] = dm[:, :5] = dm[:, -5:] = 0.0
    dm *= float(np.mean(m0))
    eps = 1e-6
    Jp = oracle.misfit(m0 + eps * dm, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                       src_list=c.src_list)
    Jm = oracle.misfit(m0 - eps * dm, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                       src_list=c.src_list)
    fd = (Jp - Jm) / (2 * eps)
    assert abs(float(np.sum(g * dm)) - fd) / abs(fd) < 1e-4


@pytest.mark.skipif(not oracle.ref_available(), reason="reference core not built (oracle/_ref)")
def test_bit_identical_to_reference_cpp_on_fresh_inputs():
    rng = np.random.default_rng(11)
    shape = (19, 23, 17)
    m = 1.0 / (1500.0 + 40.0 * rng.standard_normal(shape)) ** 2
    idx = [tuple(int(rng.integers(1, s - 1)) for s in shape) for _ in range(6)]
    wav = np.sin(np.arange(90) * 0.3) * np.exp(-0.002 * (np.arange(90) - 20.0) ** 2)
    d_ref = oracle.ref_forward_fmc(m, idx, wav, 1e-7, 1e-3, 90, [1, 4])
    d_or = oracle.forward_fmc(m, idx, wav, 1e-7, 1e-3, 90, None, [1, 4])
    assert np.array_equal(d_ref, d_or)
    m0 = np.full(shape, 1.0 / 1500.0 ** 2)
    Jr, gr = oracle.ref_misfit_and_gradient(m0, idx, wav, 1e-7, 1e-3, 90, d_ref, [1, 4])
    Jo, go = oracle.misfit_and_gradient(m0, idx, wav, 1e-7, 1e-3, 90, d_ref, None, [1, 4], k=5)
    assert Jr == Jo and np.array_equal(gr, go)


GCN_CASES = ["ring2d_point", "ring2d_sponge", "cyl3d_point", "odd2d", "odd3d", "parity2d",
             "parity3d", "gpu3d"]


@pytest.mark.parametrize("name", GCN_CASES)
def test_gcn_gradient_matches_reference(name):
    """The GCN misfit (fwi.py:158-167, libuap.hpp:133-162): FP64 restatement
    against the reference's Python, bit for bit against its C++ core."""
    c = load(name)
    a = c.args()
    J, g = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                      a["sponge"], a["src_list"], None, k=9, misfit_type="gcn")
    assert abs(J - float(c["J_gcn"])) <= 1e-12 * abs(float(c["J_gcn"]))
    assert rel_max(g, c["g_gcn"]) < 1e-10
    if "J_gcn_cpp" in c:
        J0, g0 = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                            c["dobs"], None, a["src_list"], misfit_type="gcn")
        assert J0 == float(c["J_gcn_cpp"]) and np.array_equal(g0, c["g_gcn_cpp"])


@pytest.mark.parametrize("name", ["ring2d_point", "cyl3d_point", "parity2d"])
def test_gcn_fp32_restatement_within_tolerance(name):
    c = load(name)
    a = c.args()
    J, g = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                        a["sponge"], a["src_list"], None, C=4, misfit_type="gcn")
    assert abs(J.sum() - float(c["J_gcn"])) <= 1e-5 * abs(float(c["J_gcn"]))
    assert rel_l2(g, c["g_gcn"]) < 1e-4


WINDOW_CASES = ["ring2d_window", "cyl3d_window"]


@pytest.mark.parametrize("name", WINDOW_CASES)
@pytest.mark.parametrize("mt", ["l2", "gcn"])
def test_time_weights_match_reference(name, mt):
    """Per-transmit data windows (fwi.py:247-301 time_weights): misfit and
    gradient of the FP64 restatement against the reference's Python, the
    checkpointed form bit-identical to the full history, the misfit-only call
    equal to fwi.misfit."""
    c = load(name)
    a = c.args()
    sfx = "" if mt == "l2" else "_gcn"
    W = c["tw"]
    J, g = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                      None, a["src_list"], misfit_type=mt, time_weights=list(W))
    assert abs(J - float(c["J" + sfx])) <= 1e-12 * abs(float(c["J" + sfx]))
    assert rel_max(g, c["g" + sfx]) < 1e-9
    Jk, gk = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                        c["dobs"], None, a["src_list"], k=7, misfit_type=mt,
                                        time_weights=W)
    assert Jk == J and np.array_equal(gk, g)
    Jm = oracle.misfit(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"], None,
                       a["src_list"], misfit_type=mt, time_weights=W)
    assert abs(Jm - float(c["Jm" + sfx])) <= 1e-12 * abs(float(c["Jm" + sfx]))
    # the window matters: without it the gradient is a different vector
    _, g0 = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                       None, a["src_list"], misfit_type=mt)
    assert rel_l2(g0, g) > 1e-3


@pytest.mark.parametrize("name", WINDOW_CASES)
@pytest.mark.parametrize("mt", ["l2", "gcn"])
def test_time_weights_fp32_restatement_within_tolerance(name, mt):
    c = load(name)
    a = c.args()
    sfx = "" if mt == "l2" else "_gcn"
    J, g = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                        None, a["src_list"], None, C=2, misfit_type=mt,
                                        time_weights=c["tw"])
    assert abs(J.sum() - float(c["J" + sfx])) <= 1e-5 * abs(float(c["J" + sfx]))
    assert rel_l2(g, c["g" + sfx]) < grad_tol(name)


def test_time_weights_with_a_unit_window_change_nothing():
    c = load("ring2d_point")
    a = c.args()
    W = np.ones((len(a["src_list"]), c.nt, len(c["idx"])))
    J, g = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                      None, a["src_list"], time_weights=W)
    J0, g0 = oracle.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                        None, a["src_list"])
    assert J == J0 and np.array_equal(g, g0)
    J32, g32 = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                            c["dobs"], None, a["src_list"], C=2, time_weights=W)
    J320, g320 = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                              c["dobs"], None, a["src_list"], C=2)
    assert np.array_equal(J32, J320) and np.array_equal(g32, g320)


INVERT_RUNS = {"gd": dict(n_iter=3), "gcn": dict(n_iter=2, misfit_type="gcn"),
               "tw": dict(n_iter=2), "gn": dict(n_iter=1, optimizer="gauss-newton", n_cg=3)}


@pytest.mark.parametrize("key", sorted(INVERT_RUNS))
def test_invert_restatement_matches_reference(key):
    """oracle.invert (the host restatement of fwi.invert / _invert_gauss_newton
    that checks the device-resident loop) driven by the FP64 oracle reproduces
    the reference's own inversion: same accepted steps, same history."""
    from oracle.invert import FP64Backend, invert
    c = load("invert2d")
    kw = dict(INVERT_RUNS[key])
    if key == "tw":
        kw["time_weights"] = c["tw"]
    m, hist = invert(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                     src_list=c.src_list, update_mask=c["mask"],
                     m_bounds=(float(c["lo"]), float(c["hi"])), step_frac=0.03,
                     backend=FP64Backend(), **kw)
    ref = c["hist_" + key]
    assert len(hist) == len(ref)
    assert np.max(np.abs(np.asarray(hist) - ref) / ref) < 1e-12
    assert rel_l2(m - c["m0"], c["m_" + key] - c["m0"]) < 1e-10


@pytest.mark.parametrize("name", ["tfm2d", "tfm3d"])
def test_tfm_restatement_is_the_reference(name):
    """oracle.tfm (imaging.py:27-74 restated) reproduces the reference's TFM
    images bit for bit (envelope and real part)."""
    from oracle.tfm import tfm
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    args = (z["data"], z["element_pos"], z["tx_elements"], float(z["c"]), float(z["fs"]),
            float(z["radius_m"]), int(z["npix"]), float(z["half"]))
    img, axes = tfm(*args)
    assert np.array_equal(img, z["image"])
    assert np.array_equal(np.stack(axes), z["axes"])
    img_re, _ = tfm(*args, envelope=False)
    assert np.array_equal(img_re, z["image_re"])
