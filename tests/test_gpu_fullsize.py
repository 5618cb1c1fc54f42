"""GPU parity at the benchmark's full grid size (192^3, dx = 0.2 mm, 8x32
cylinder, seeded random-field model).

The FP64 oracle cannot run the full 256-shot x 2000-step workload in a test,
so parity against it uses a 2-shot subset and a shortened time axis on the
full grid; the full time axis is covered by size-independent properties
(batched shots bit-identical to one shot per launch, reciprocity of the
point-to-point traces).
"""

import numpy as np
import pytest

import oracle
from golden_util import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def prob():
    assert torch.cuda.is_available()
    from openusct_gb300 import build, problems
    build.build()
    return problems.cylinder3d(seed=0)


def _sub(p, nt):
    return p.wavelet[:nt]


def test_fullsize_traces_and_gradient_vs_fp64(prob):
    import openusct_gb300.backend as gb
    nt = 240
    wav = _sub(prob, nt)
    sl = [0, 40]
    d64 = oracle.forward_fmc(prob.m_true, prob.geom, wav, prob.dt, prob.h, nt, None, sl)
    d32 = gb.forward_fmc(prob.m_true, prob.geom, wav, prob.dt, prob.h, nt, None, sl)
    assert rel_l2(d32, d64) < 1e-5
    J64, g64 = oracle.misfit_and_gradient(prob.m0, prob.geom, wav, prob.dt, prob.h, nt, d64, None,
                                          sl, k=24)
    J32, g32 = gb.misfit_and_gradient(prob.m0, prob.geom, wav, prob.dt, prob.h, nt, d64,
                                      src_list=sl, ckpt_k=24)
    assert abs(J32 - J64) <= 1e-4 * J64
    assert rel_l2(g32, g64) < 1e-4
    # 8 seeded directions: GPU gradient . dm against a central difference of the FP64 misfit
    rng = np.random.default_rng(8)
    for _ in range(8):
        dm = rng.standard_normal(prob.m0.shape).astype(np.float64)
        dm[:5] = dm[-5:] = dm[:, :5] = dm[:, -5:] = dm[:, :, :5] = dm[:, :, -5:] = 0.0
        dm *= float(np.mean(prob.m0))
        eps = 1e-6
        Jp = oracle.misfit(prob.m0 + eps * dm, prob.geom, wav, prob.dt, prob.h, nt, d64,
                           src_list=sl)
        Jm = oracle.misfit(prob.m0 - eps * dm, prob.geom, wav, prob.dt, prob.h, nt, d64,
                           src_list=sl)
        fd = (Jp - Jm) / (2 * eps)
        assert abs(float(np.sum(g32 * dm)) - fd) <= 1e-4 * abs(fd)


def test_fullsize_batched_equals_one_shot_and_reciprocity(prob):
    import openusct_gb300.backend as gb
    sl = [0, 37, 101, 200]
    m = torch.from_numpy(prob.m_true).cuda()
    d4 = gb.forward_fmc(m, prob.geom, prob.wavelet, prob.dt, prob.h, prob.nt, None, sl,
                        batch=4).cpu().numpy()
    d1 = gb.forward_fmc(m, prob.geom, prob.wavelet, prob.dt, prob.h, prob.nt, None, sl,
                        batch=1).cpu().numpy()
    assert np.array_equal(d4, d1)
    # reciprocity of point-to-point traces (the scheme is symmetric in space)
    for a in range(len(sl)):
        for b in range(a + 1, len(sl)):
            tab = d4[a, :, sl[b]]
            tba = d4[b, :, sl[a]]
            assert rel_l2(tab, tba) < 1e-4


def test_fullsize_checkpoint_interval_is_bit_exact(prob):
    """The checkpoint interval k (16, 32, 64 as the gradient configuration
    sweeps it, and k = nt-1: no recompute at all) changes only what is stored
    and recomputed, never the result: bit-identical gradients at 192^3."""
    import openusct_gb300.backend as gb
    nt = 240
    wav = _sub(prob, nt)
    sl = [5, 133]
    d = gb.forward_fmc(prob.m_true, prob.geom, wav, prob.dt, prob.h, nt, None, sl)
    ref = None
    for k in (16, 32, 64, nt - 1):
        J, g = gb.misfit_and_gradient(prob.m0, prob.geom, wav, prob.dt, prob.h, nt, d,
                                      src_list=sl, ckpt_k=k)
        if ref is None:
            ref = (J, g)
        else:
            assert J == ref[0] and np.array_equal(g, ref[1]), k


def test_320_grid_traces_and_gradient_vs_fp64():
    """The large gradient configuration's grid (320^3, dx = 0.12 mm, 16 x 32
    elements) on a 2-shot subset and a shortened time axis, against the FP64
    oracle."""
    import openusct_gb300.backend as gb
    from openusct_gb300 import problems
    p = problems.cylinder3d_large(seed=0)
    nt = 100
    wav = p.wavelet[:nt]
    sl = [0, 300]
    d64 = oracle.forward_fmc(p.m_true, p.geom, wav, p.dt, p.h, nt, None, sl)
    d32 = gb.forward_fmc(p.m_true, p.geom, wav, p.dt, p.h, nt, None, sl)
    assert rel_l2(d32, d64) < 1e-5
    J64, g64 = oracle.misfit_and_gradient(p.m0, p.geom, wav, p.dt, p.h, nt, d64, None, sl, k=20)
    J32, g32 = gb.misfit_and_gradient(p.m0, p.geom, wav, p.dt, p.h, nt, d64, src_list=sl)
    assert abs(J32 - J64) <= 1e-4 * J64
    # after 100 steps the residual is only 4.3e-4 of the data, so the FP32
    # trace rounding (1.6e-7 of the data, measured with the FP32 restatement)
    # is 3.6e-4 of the residual: that, not the kernels, bounds the gradient
    # here (the 192^3 test above holds 1e-4 on a longer time axis)
    assert rel_l2(g32, g64) < 5e-4


# ---- the configurations' full time axes against the FP64 oracle -------------
# The FP32 rounding of the wavefields accumulates over the time steps, so the
# long axes are the cases that matter.  Shot subsets keep the FP64 runs to a
# minute or two on the host cores (shots are independent and the gradient is
# a sum over shots); the oracle checkpoints so its memory stays bounded.

@pytest.mark.slow
def test_192_full_time_axis_vs_fp64(prob):
    """192^3, two seeded shots over all nt = 2000 levels: traces <= 1e-5,
    gradient and misfit <= 1e-4 against the FP64 oracle."""
    import openusct_gb300.backend as gb
    rng = np.random.default_rng(1920)
    sl = sorted(int(s) for s in rng.choice(prob.n_shots, size=2, replace=False))
    args = (prob.geom, prob.wavelet, prob.dt, prob.h, prob.nt)
    d64 = oracle.forward_fmc(prob.m_true, *args, None, sl)
    d32 = gb.forward_fmc(prob.m_true, *args, None, sl)
    assert rel_l2(d32, d64) < 1e-5
    J64, g64 = oracle.misfit_and_gradient(prob.m0, *args, d64, None, sl, k=64)
    J32, g32 = gb.misfit_and_gradient(prob.m0, *args, d64, src_list=sl)
    assert abs(J32 - J64) <= 1e-4 * J64
    assert rel_l2(g32, g64) < 1e-4


@pytest.mark.slow
def test_ring2d_full_acquisition_vs_fp64():
    """The 2D ring configuration in full: 256^2, two seeded discs, all 64
    shots x 64 receivers over nt = 1500: traces <= 1e-5, gradient and misfit
    <= 1e-4 against the FP64 oracle."""
    import openusct_gb300.backend as gb
    from openusct_gb300 import problems
    p = problems.ring2d(seed=0)
    args = (p.geom, p.wavelet, p.dt, p.h, p.nt)
    d64 = oracle.forward_fmc(p.m_true, *args)
    d32 = gb.forward_fmc(p.m_true, *args)
    assert d32.shape == (64, 1500, 64)
    assert rel_l2(d32, d64) < 1e-5
    J64, g64 = oracle.misfit_and_gradient(p.m0, *args, d64, k=0)
    J32, g32 = gb.misfit_and_gradient(p.m0, *args, d64)
    assert abs(J32 - J64) <= 1e-4 * J64
    assert rel_l2(g32, g64) < 1e-4


@pytest.mark.slow
def test_320_full_time_axis_vs_fp64():
    """320^3 (dx = 0.12 mm, 16 x 32 elements), one seeded shot over all
    nt = 3000 levels: traces <= 1e-5, gradient and misfit <= 1e-4 against the
    FP64 oracle."""
    import openusct_gb300.backend as gb
    from openusct_gb300 import problems
    p = problems.cylinder3d_large(seed=0)
    sl = [int(np.random.default_rng(320).integers(p.n_shots))]
    args = (p.geom, p.wavelet, p.dt, p.h, p.nt)
    d64 = oracle.forward_fmc(p.m_true, *args, None, sl)
    d32 = gb.forward_fmc(p.m_true, *args, None, sl)
    assert rel_l2(d32, d64) < 1e-5
    J64, g64 = oracle.misfit_and_gradient(p.m0, *args, d64, None, sl, k=64)
    J32, g32 = gb.misfit_and_gradient(p.m0, *args, d64, src_list=sl)
    assert abs(J32 - J64) <= 1e-4 * J64
    assert rel_l2(g32, g64) < 1e-4
