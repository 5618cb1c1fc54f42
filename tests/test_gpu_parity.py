"""GPU parity: the CUDA path against the oracle on the committed goldens.

* bit for bit against the FP32 kernel-order restatement (oracle o32_*), for
  several shot-batch widths and launch shapes -- this pins indexing, halos,
  the shot-innermost layout, source/receiver entries and the shot reduction;
* within the FP32 tolerances (golden_util.TRACE_TOL / GRAD_TOL) of the
  reference's FP64 outputs;
* checkpoint recompute bit-identical to no recompute;
* batched shots bit-identical to one shot per launch.
All calls go through the C ABI (libusct_gb300.so) via the backend module.
"""

import ctypes

import numpy as np
import pytest

import oracle
from golden_util import CASES, grad_tol, load, rel_l2, trace_tol

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from openusct_gb300 import build
    build.build()
    yield


def gb():
    import openusct_gb300.backend as backend
    return backend


def _tiles(ndim):
    """(tile_x, tile_y, zchunk, variant): variant 1 = TMA ring, 0 = register queue; the
    TMA ring needs 4*tile_x >= 4*C (the plan reports an error otherwise, so such
    combinations are skipped)."""
    if ndim == 3:
        return [(32, 4, 0, 1), (32, 8, 3, 1), (64, 2, 5, 1), (64, 4, 0, 1), (32, 8, 3, 0),
                (64, 4, 0, 0)]
    return [(64, 1, 0, 1), (128, 1, 7, 1), (64, 1, 0, 0), (128, 1, 7, 0)]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("C", [1, 2, 4])
def test_forward_bit_exact_vs_fp32_restatement(name, C):
    c = load(name)
    a = c.args()
    ref = oracle.forward_fmc32(c["m_true"], c.geom, a["wavelet"], c.dt, c.h, c.nt, a["sponge"],
                               a["src_list"], a["footprints"])
    for tile in _tiles(c["m_true"].ndim):
        if tile[3] == 1 and C < 4 and (c["m_true"].ndim == 2 or tile[0] != 32):
            continue   # outside the TMA ring's box constraints
        d = gb().forward_fmc(torch.from_numpy(c["m_true"]).cuda(), c.geom, a["wavelet"], c.dt,
                             c.h, c.nt, a["sponge"], a["src_list"], a["footprints"], batch=C,
                             tile=tile)
        d = d.cpu().numpy()
        assert d.dtype == np.float32
        assert np.array_equal(d, ref), f"tile {tile}: max diff {np.abs(d - ref).max()}"


@pytest.mark.parametrize("name", CASES)
def test_forward_vs_reference_fp64(name):
    c = load(name)
    a = c.args()
    d = gb().forward_fmc(c["m_true"], c.geom, a["wavelet"], c.dt, c.h, c.nt, a["sponge"],
                         a["src_list"], a["footprints"])
    assert d.dtype == np.float64 and d.shape == c["dobs"].shape
    assert rel_l2(d, c["dobs"]) < trace_tol(name)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("C", [1, 4, 16])
@pytest.mark.parametrize("variant", [0, 1])
def test_gradient_bit_exact_vs_fp32_restatement(name, C, variant):
    c = load(name)
    a = c.args()
    ndim = c["m0"].ndim
    if variant == 1 and C < 4 and ndim == 2:
        pytest.skip("the TMA ring needs C >= 4 in 2D")
    tile = (32, 8, 0, variant) if ndim == 3 else (128, 1, 0, variant)
    Jr, gr = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                          c["dobs"], a["sponge"], a["src_list"], a["footprints"],
                                          C=C)
    J, g, Js = gb().misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                        c["dobs"], a["sponge"], a["src_list"],
                                        footprints=a["footprints"], batch=C, ckpt_k=5,
                                        tile=tile, return_per_shot=True)
    assert np.allclose(Js, Jr, rtol=1e-12, atol=0)
    assert np.array_equal(g, gr), f"max diff {np.abs(g - gr).max()} of {np.abs(gr).max()}"


@pytest.mark.parametrize("name", CASES)
def test_gradient_vs_reference_fp64(name):
    c = load(name)
    a = c.args()
    J, g = gb().misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"],
                                    a["sponge"], a["src_list"], footprints=a["footprints"])
    assert g.dtype == np.float64 and g.shape == c["m0"].shape
    assert abs(J - float(c["J"])) <= 1e-4 * abs(float(c["J"]))
    assert rel_l2(g, c["g"]) < grad_tol(name)


@pytest.mark.parametrize("name", ["ring2d_point", "cyl3d_aperture", "parity3d", "ring2d_sponge"])
def test_checkpoint_recompute_bit_exact(name):
    """k = nt-1: one segment, the stash is filled by the forward sweep itself
    (no recompute); smaller k recompute every earlier segment from stored
    levels -- the gradients must agree bit for bit."""
    c = load(name)
    a = c.args()
    res = []
    for k in (c.nt - 1, 2, 3, 16):
        _, g = gb().misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                        c["dobs"], a["sponge"], a["src_list"],
                                        footprints=a["footprints"], batch=2, ckpt_k=k)
        res.append(g)
    for g in res[1:]:
        assert np.array_equal(g, res[0])


@pytest.mark.parametrize("name", ["parity2d", "gpu3d"])
def test_batched_equals_one_shot_per_launch(name):
    c = load(name)
    a = c.args()
    m = torch.from_numpy(c["m_true"]).cuda()
    ds = [gb().forward_fmc(m, c.geom, a["wavelet"], c.dt, c.h, c.nt, None, a["src_list"],
                           batch=C).cpu().numpy() for C in (1, 4, 16)]
    assert np.array_equal(ds[0], ds[1]) and np.array_equal(ds[0], ds[2])


@pytest.mark.parametrize("C,variant", [(2, 0), (4, 1)])
def test_gauss_newton_hessian_vector(C, variant):
    c = load("gn2d")
    hv32, born32 = oracle.gn_hessian_vector32(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["v"],
                                              src_list=c.src_list, C=C)
    hv, born = gb().gn_hessian_vector(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["v"],
                                      src_list=c.src_list, batch=C, ckpt_k=7,
                                      tile=(128, 1, 0, variant), return_born=True)
    assert np.array_equal(born.astype(np.float32), born32)
    assert np.array_equal(hv, hv32)
    assert rel_l2(hv, c["Hv"]) < 1e-4


@pytest.mark.parametrize("variant", [0, 1])
def test_gauss_newton_3d_bit_exact(variant):
    c = load("gpu3d")
    rng = np.random.default_rng(3)
    v = rng.standard_normal(c["m0"].shape) * float(np.mean(c["m0"])) * 0.01
    sl = c.src_list[:4]
    hv32, born32 = oracle.gn_hessian_vector32(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, v,
                                              src_list=sl, C=4)
    hv, born = gb().gn_hessian_vector(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, v,
                                      src_list=sl, batch=4, ckpt_k=9,
                                      tile=(32, 8, 0, variant), return_born=True)
    assert np.array_equal(born.astype(np.float32), born32)
    assert np.array_equal(hv, hv32)


def test_gauss_newton_3d_vs_fp64_oracle():
    c = load("parity3d")
    rng = np.random.default_rng(5)
    v = rng.standard_normal(c["m0"].shape)
    v[:3] = v[-3:] = v[:, :3] = v[:, -3:] = v[:, :, :3] = v[:, :, -3:] = 0.0
    v *= float(np.mean(c["m0"])) * 0.01
    sl = c.src_list[:3]
    ref = oracle.gn_hessian_vector(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, v, src_list=sl)
    hv = gb().gn_hessian_vector(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, v, src_list=sl)
    assert rel_l2(hv, ref) < 1e-4


@pytest.mark.parametrize("name", ["parity2d", "gpu3d", "odd3d"])
def test_plain_one_shot_form(name):
    c = load(name)
    d = gb().plain_forward_fmc(c["m_true"], c.geom, c.wavelet, c.dt, c.h, c.nt, c.src_list)
    assert rel_l2(d, c["dobs"]) < trace_tol(name)
    J, g = gb().plain_misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                          c.src_list)
    assert abs(J - float(c["J"])) <= 1e-4 * abs(float(c["J"]))
    assert rel_l2(g, c["g"]) < grad_tol(name)


def test_host_pointer_abi_matches_reference_core():
    """usct_forward_fmc / usct_misfit_and_gradient take the arguments of
    uap::forward_fmc / uap::misfit_and_gradient (libuap.hpp:109,169)."""
    from openusct_gb300 import _lib
    from openusct_gb300.geometry import linear_indices
    lib = _lib.load()
    c = load("parity3d")
    m = np.ascontiguousarray(c["m_true"])
    dims = (ctypes.c_int * 3)(*m.shape)
    rec = linear_indices(c.geom.idx, m.shape).astype(np.int32)
    tx = np.ascontiguousarray(rec[c.src_list])
    data = np.zeros((len(tx), c.nt, len(rec)))
    _lib.check(lib.usct_forward_fmc(m.ctypes.data_as(_lib._dp), dims, 3, c.h, c.dt, c.nt,
                                    tx.ctypes.data_as(_lib._ip), len(tx),
                                    rec.ctypes.data_as(_lib._ip), len(rec),
                                    c.wavelet.ctypes.data_as(_lib._dp),
                                    data.ctypes.data_as(_lib._dp)))
    assert rel_l2(data, c["dobs_cpp"]) < 1e-5
    g = np.zeros(m.shape)
    J = ctypes.c_double()
    m0 = np.ascontiguousarray(c["m0"])
    dobs = np.ascontiguousarray(c["dobs"])
    _lib.check(lib.usct_misfit_and_gradient(m0.ctypes.data_as(_lib._dp), dims, 3, c.h, c.dt, c.nt,
                                            tx.ctypes.data_as(_lib._ip), len(tx),
                                            rec.ctypes.data_as(_lib._ip), len(rec),
                                            c.wavelet.ctypes.data_as(_lib._dp),
                                            dobs.ctypes.data_as(_lib._dp),
                                            g.ctypes.data_as(_lib._dp), ctypes.byref(J)))
    assert abs(J.value - float(c["J_cpp"])) <= 1e-4 * float(c["J_cpp"])
    assert rel_l2(g, c["g_cpp"]) < 1e-4
    _lib.check(lib.usct_misfit_and_gradient_mt(m0.ctypes.data_as(_lib._dp), dims, 3, c.h, c.dt,
                                               c.nt, tx.ctypes.data_as(_lib._ip), len(tx),
                                               rec.ctypes.data_as(_lib._ip), len(rec),
                                               c.wavelet.ctypes.data_as(_lib._dp),
                                               dobs.ctypes.data_as(_lib._dp),
                                               g.ctypes.data_as(_lib._dp), 1, ctypes.byref(J)))
    assert abs(J.value - float(c["J_gcn_cpp"])) <= 1e-5 * float(c["J_gcn_cpp"])
    assert rel_l2(g, c["g_gcn_cpp"]) < 1e-4


def test_directional_derivatives_eight_seeded_directions():
    """GPU gradient . dm against a central difference of the FP64 misfit along
    8 seeded directions (the reference's test_gradient_misfits.py pattern)."""
    c = load("parity3d")
    sl = c.src_list[:3]
    m0 = c["m0"]
    _, g = gb().misfit_and_gradient(m0, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"][:3],
                                    src_list=sl)
    rng = np.random.default_rng(1)
    for _ in range(8):
        dm = rng.standard_normal(m0.shape)
        dm[:3] = dm[-3:] = dm[:, :3] = dm[:, -3:] = dm[:, :, :3] = dm[:, :, -3:] = 0.0
        dm *= float(np.mean(m0))
        eps = 1e-6
        Jp = oracle.misfit(m0 + eps * dm, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"][:3],
                           src_list=sl)
        Jm = oracle.misfit(m0 - eps * dm, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"][:3],
                           src_list=sl)
        fd = (Jp - Jm) / (2 * eps)
        assert abs(float(np.sum(g * dm)) - fd) <= 1e-4 * abs(fd)


GCN_CASES = ["ring2d_point", "ring2d_sponge", "cyl3d_point", "odd2d", "odd3d", "parity2d",
             "parity3d", "gpu3d"]


@pytest.mark.parametrize("name", GCN_CASES)
@pytest.mark.parametrize("C", [1, 4])
def test_gcn_gradient_bit_exact_and_vs_reference(name, C):
    """The GCN misfit (libuap.hpp misfit_type=1): GPU == FP32 restatement bit
    for bit; within tolerance of the reference's FP64 result."""
    c = load(name)
    a = c.args()
    Jr, gr = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                          c["dobs"], a["sponge"], a["src_list"], None, C=C,
                                          misfit_type="gcn")
    J, g, Js = gb().misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                        c["dobs"], a["sponge"], a["src_list"], misfit_type="gcn",
                                        batch=C, ckpt_k=6, return_per_shot=True)
    assert np.array_equal(Js, Jr)
    assert np.array_equal(g, gr)
    assert abs(J - float(c["J_gcn"])) <= 1e-5 * abs(float(c["J_gcn"]))
    assert rel_l2(g, c["g_gcn"]) < 1e-4
    Jm = gb().misfit(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"], a["sponge"],
                     a["src_list"], misfit_type="gcn")
    assert abs(Jm - float(c["J_gcn"])) <= 1e-5 * abs(float(c["J_gcn"]))


def test_error_conventions():
    c = load("ring2d_point")
    with pytest.raises(NotImplementedError):
        gb().misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                 src_list=c.src_list, misfit_type="envelope")
    with pytest.raises(ValueError):
        gb().misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                 src_list=c.src_list, misfit_type="nope")
    with pytest.raises(ValueError):
        gb().misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"][:1],
                                 src_list=c.src_list)


def test_backend_protocol_as_invert_calls_it():
    """fwi.invert calls a backend positionally (fwi.py:598-603):
    misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list,
    misfit_type=...) and misfit(same...)."""
    c = load("parity2d")
    mg = gb().misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], None,
                                  c.src_list, misfit_type="l2")
    mf = gb().misfit(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], None, c.src_list,
                     misfit_type="l2")
    assert isinstance(mg[0], float) and mg[1].shape == c["m0"].shape
    assert abs(mf - mg[0]) <= 1e-9 * mg[0]


def test_simulate_dataset_on_the_gpu():
    from openusct_gb300 import acquire
    from openusct_gb300.geometry import RingGeometry
    c = load("ring2d_point")
    ring = RingGeometry(8, 0.024, 0.06, 1e-3)
    ds = acquire.simulate_dataset(1.0 / np.sqrt(c["m_true"]), ring, c.wavelet, c.dt, 1480.0,
                                  src_list=c.src_list)
    assert ds.data.shape == c["dobs"].shape
    assert rel_l2(ds.data, c["dobs"]) < 1e-5


@pytest.mark.parametrize("name", ["ring2d_window", "cyl3d_window"])
@pytest.mark.parametrize("mt", ["l2", "gcn"])
@pytest.mark.parametrize("C", [1, 2])
def test_time_weights_bit_exact_and_vs_reference(name, mt, C):
    """Data windows (fwi.py:247-301 time_weights) on the device: misfit and
    gradient bit-identical to the FP32 restatement, within tolerance of the
    reference's FP64 result; the misfit-only call agrees; a list of windows
    and one stacked array give the same answer."""
    c = load(name)
    a = c.args()
    sfx = "" if mt == "l2" else "_gcn"
    W = c["tw"]
    Jr, gr = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                          c["dobs"], None, a["src_list"], None, C=C,
                                          misfit_type=mt, time_weights=W)
    J, g, Js = gb().misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                        c["dobs"], None, a["src_list"], misfit_type=mt,
                                        time_weights=list(W), batch=C, ckpt_k=6,
                                        return_per_shot=True)
    # the L2 sum over samples is a device tree (FP64, order differs from the
    # restatement's loop); the GCN sums run in the same order on both sides
    if mt == "l2":
        assert np.allclose(Js, Jr, rtol=1e-12, atol=0)
    else:
        assert np.array_equal(Js, Jr)
    assert np.array_equal(g, gr)
    assert abs(J - float(c["J" + sfx])) <= 1e-5 * abs(float(c["J" + sfx]))
    assert rel_l2(g, c["g" + sfx]) < grad_tol(name)
    Jm = gb().misfit(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt, c["dobs"], None,
                     a["src_list"], misfit_type=mt, time_weights=W, batch=C)
    assert abs(Jm - float(np.sum(Jr))) <= 1e-12 * abs(float(np.sum(Jr)))
    assert abs(Jm - float(c["Jm" + sfx])) <= 1e-5 * abs(float(c["Jm" + sfx]))


def test_time_weights_shape_is_checked():
    c = load("ring2d_window")
    with pytest.raises(ValueError, match="time_weights"):
        gb().misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"], None,
                                 c.src_list, time_weights=c["tw"][:, :-1])


def test_cpp_example_against_the_oracle(tmp_path):
    """Run the plain C++ example (host-pointer C ABI) and check its checksums
    against the FP64 oracle on the same inputs."""
    import subprocess
    from example_inputs import example_problem
    from openusct_gb300 import build
    exe = build.build_example(str(tmp_path / "usct_example"))
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    vals = dict(line.split("=") for line in out.splitlines() if "=" in line)
    vals = {k: float(v) for k, v in vals.items()}
    assert "usct_example OK" in out
    p = example_problem()
    args = (p["wavelet"], p["dt"], p["h"], p["nt"])
    d = oracle.forward_fmc(p["m_true"], p["idx"], *args)
    assert abs(vals["forward_sum_abs"] / np.abs(d).sum() - 1) < 1e-5
    J, g = oracle.misfit_and_gradient(p["m0"], p["idx"], p["wavelet"], p["dt"], p["h"], p["nt"], d)
    assert abs(vals["l2_J"] / J - 1) < 1e-4
    assert abs(vals["l2_grad_sum_abs"] / np.abs(g).sum() - 1) < 1e-4
    Jg, gg = oracle.misfit_and_gradient(p["m0"], p["idx"], p["wavelet"], p["dt"], p["h"],
                                        p["nt"], d, misfit_type="gcn")
    assert abs(vals["gcn_J"] / Jg - 1) < 1e-4
    assert abs(vals["gcn_grad_sum_abs"] / np.abs(gg).sum() - 1) < 1e-4


@pytest.mark.parametrize("mt", ["l2", "gcn"])
def test_windows_with_footprints_and_sponge_bit_exact(mt):
    """Data windows combined with finite-aperture elements (and, in 2D, the
    sponge): the device equals the FP32 restatement bit for bit."""
    for name in ("ring2d_aperture", "cyl3d_aperture", "ring2d_sponge"):
        c = load(name)
        a = c.args()
        rng = np.random.default_rng(21)
        W = rng.uniform(0.0, 1.0, (len(a["src_list"]), c.nt, len(c["idx"])))
        Jr, gr = oracle.misfit_and_gradient32(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                              c["dobs"], a["sponge"], a["src_list"],
                                              a["footprints"], C=2, misfit_type=mt,
                                              time_weights=W)
        J, g, Js = gb().misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                            c["dobs"], a["sponge"], a["src_list"], misfit_type=mt,
                                            footprints=a["footprints"], time_weights=W, batch=2,
                                            ckpt_k=7, return_per_shot=True)
        assert np.array_equal(g, gr), name
        assert np.allclose(Js, Jr, rtol=1e-12, atol=0), name


def test_sphere_array_with_disc_apertures_vs_fp64():
    """A spherical-shell array (SphereArray semantics) with disc apertures
    built by geometry.build_footprints: traces and gradient against the FP64
    oracle, and bit for bit against the FP32 restatement."""
    from openusct_gb300.geometry import ShellGeometry, build_footprints, ricker
    h = 8.0e-4
    shell = ShellGeometry(24, 0.012, 0.032, h)
    fps = build_footprints(shell, width_m=0.003, shape="disc", height_m=0.003)
    n = shell.n
    rng = np.random.default_rng(4)
    c0 = 1500.0 + 40.0 * rng.standard_normal((n, n, n))
    m_true = 1.0 / (c0 * c0)
    m0 = np.full((n, n, n), 1.0 / 1500.0 ** 2)
    dt, nt = 0.3 * h / 1700.0, 160
    wav = ricker(nt, dt, 0.6e6)
    sl = [0, 7, 15]
    d64 = oracle.forward_fmc(m_true, shell.idx, wav, dt, h, nt, None, sl, fps)
    d32 = gb().forward_fmc(m_true, shell, wav, dt, h, nt, None, sl, fps)
    assert rel_l2(d32, d64) < 1e-4
    Jr, gr = oracle.misfit_and_gradient32(m0, shell.idx, wav, dt, h, nt, d64, None, sl, fps, C=4)
    J, g, Js = gb().misfit_and_gradient(m0, shell, wav, dt, h, nt, d64, None, sl,
                                        footprints=fps, batch=4, return_per_shot=True)
    assert np.array_equal(g, gr)
    J64, g64 = oracle.misfit_and_gradient(m0, shell.idx, wav, dt, h, nt, d64, None, sl, fps, k=20)
    assert abs(J - J64) <= 1e-4 * J64
    assert rel_l2(g, g64) < 1e-4
