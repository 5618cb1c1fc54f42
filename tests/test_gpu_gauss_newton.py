"""Gauss-Newton Hessian-vector products on the GPU.

* Against a central difference of the FP64 gradient at a zero-residual point,
  where the finite difference of the gradient is the exact Gauss-Newton
  Hessian: the reference's own check (simulation/tests/test_gauss_newton.py:
  30-51, its setup; rel. max error) with the GPU's FP32 product held to 1e-4.
* At the Gauss-Newton configuration's grid (224^3, dx = 0.18 mm, 8 x 32
  elements, seeded smooth perturbation) on a 2-shot subset and a shortened
  time axis, against the FP64 oracle.
"""

import numpy as np
import pytest

import oracle
from golden_util import load, rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gb():
    assert torch.cuda.is_available()
    from openusct_gb300 import build
    build.build()
    import openusct_gb300.backend as backend
    return backend


def _rel_max(a, b):
    return float(np.max(np.abs(a - b)) / (np.max(np.abs(b)) + 1e-30))


def _fd_of_gradient(m0, geom, wav, dt, h, nt, v, sl, eps):
    d0 = oracle.forward_fmc(m0, geom, wav, dt, h, nt, None, sl)   # r = 0 at m0
    _, gp = oracle.misfit_and_gradient(m0 + eps * v, geom, wav, dt, h, nt, d0, None, sl)
    _, gm = oracle.misfit_and_gradient(m0 - eps * v, geom, wav, dt, h, nt, d0, None, sl)
    return (gp - gm) / (2.0 * eps)


def test_hessian_vector_matches_fd_of_fp64_gradient(gb):
    """The reference's setup (8-element ring, 61^2, nt = 300, shots 0 and 4,
    seeded v): GPU Hv against the FP64 gradient's central difference."""
    c = load("gn2d")
    v = c["v"]
    fd = _fd_of_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, v, c.src_list, 1e-4)
    hv = gb.gn_hessian_vector(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, v,
                              src_list=c.src_list)
    assert _rel_max(hv, fd) < 1e-4
    # and the reference's own FP64 product agrees with the same difference
    assert _rel_max(c["Hv"], fd) < 1e-5


def test_hessian_vector_matches_fd_of_fp64_gradient_3d(gb):
    """The same check on a 3D cylinder problem (a non-homogeneous m0)."""
    c = load("gpu3d")
    rng = np.random.default_rng(7)
    v = rng.standard_normal(c["m0"].shape)
    v[:3] = v[-3:] = v[:, :3] = v[:, -3:] = v[:, :, :3] = v[:, :, -3:] = 0.0
    v *= float(np.mean(c["m0"]))
    sl = c.src_list[:3]
    fd = _fd_of_gradient(c["m_true"], c.geom, c.wavelet, c.dt, c.h, c.nt, v, sl, 1e-4)
    hv = gb.gn_hessian_vector(c["m_true"], c.geom, c.wavelet, c.dt, c.h, c.nt, v, src_list=sl)
    assert _rel_max(hv, fd) < 1e-4


@pytest.mark.slow
def test_gauss_newton_224_grid_vs_fp64(gb):
    """224^3, dx = 0.18 mm, two seeded shots over 400 steps: Hv against the
    FP64 oracle's product (rel. L2 1e-4)."""
    from openusct_gb300 import problems
    p = problems.gn3d(seed=0, nt=400)
    rng = np.random.default_rng(224)
    sl = sorted(int(s) for s in rng.choice(p.n_shots, size=2, replace=False))
    args = (p.geom, p.wavelet, p.dt, p.h, p.nt, p.v)
    ref = oracle.gn_hessian_vector(p.m0, *args, src_list=sl, k=40)
    hv = gb.gn_hessian_vector(p.m0, *args, src_list=sl)
    assert np.abs(ref).max() > 0.0
    assert rel_l2(hv, ref) < 1e-4


@pytest.mark.slow
def test_gauss_newton_224_full_time_axis_vs_fp64(gb):
    """The Gauss-Newton configuration's full time axis (224^3, nt = 2500), one
    seeded shot: Hv and the Born traces against the FP64 oracle (rel. L2
    1e-4 and 1e-5)."""
    from openusct_gb300 import problems
    p = problems.gn3d(seed=0)
    sl = [int(np.random.default_rng(2240).integers(p.n_shots))]
    args = (p.geom, p.wavelet, p.dt, p.h, p.nt, p.v)
    ref, born64 = oracle.gn_hessian_vector(p.m0, *args, src_list=sl, k=64, return_born=True)
    hv, born = gb.gn_hessian_vector(p.m0, *args, src_list=sl, return_born=True)
    assert rel_l2(born, born64) < 1e-5
    assert rel_l2(hv, ref) < 1e-4
