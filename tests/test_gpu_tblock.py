"""Two time levels per forward launch (usct_tma2.cuh, USCT_SET_TBLOCK).

The two-step kernel computes the first level on the tile grown by one cell
and one row with the single-step kernel's arithmetic and op order, so every
level it writes -- traces, checkpoints, the d2p stash of the forward sweep and
of the segment recompute -- and hence the gradient must be bit-identical to
the single-step sweeps and to the FP32 oracle, for every tile, z-chunk, ring
depth, odd and even level counts (an odd last level takes one single-step
launch), checkpoint intervals whose segments have odd and even lengths,
sources on the grid border and a sponge.
"""

import ctypes

import numpy as np
import pytest

import oracle
from golden_util import load

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def eng():
    assert torch.cuda.is_available()
    from openusct_gb300 import build
    build.build()
    from openusct_gb300 import _lib, backend
    return _lib, backend


def _run(eng, c, m, sl, C, k, tblock, sponge=None, nt=None, stages=0, zchunk=0, tile=(0, 0, 0)):
    """(traces, J per shot, gradient) of one plan through the engine's
    whole-acquisition entry points."""
    _lib, gb = eng
    from openusct_gb300.geometry import element_csr
    nt = nt or c.nt
    shape = m.shape
    tx, rx = element_csr(c.geom, shape, sl, c.footprints)
    plan = gb.Plan(shape, c.h, c.dt, nt, tx, rx, batch=C, ckpt_k=k, tile_x=tile[0],
                   tile_y=tile[1], zchunk=tile[2])
    if stages:
        plan.set("tblock_stages", stages)
    if zchunk:
        plan.set("tblock_zchunk", zchunk)
    if tblock:
        plan.set("tblock", tblock)
        assert plan.info("tblock") == (tblock if tblock > 1 else plan.info("tblock"))
    dev = torch.device("cuda", 0)
    P = lambda t: ctypes.c_void_p(0 if t is None else t.data_ptr())  # noqa: E731
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib = _lib.load()
    md = torch.from_numpy(m).to(dev)
    wd = torch.from_numpy(np.ascontiguousarray(c.wavelet[:nt])).to(dev)
    sd = torch.from_numpy(sponge).to(dev) if sponge is not None else None
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    bws = torch.empty(plan.batch_bytes(_lib.MODE_GRADIENT), dtype=torch.uint8, device=dev)
    d = torch.empty((plan.n_tx, nt, plan.n_rx), dtype=torch.float32, device=dev)
    _lib.check(lib.usct_forward_fmc_dev(plan.handle, P(md), P(sd), P(wd), P(d), P(mws), P(bws),
                                        s))
    m0 = torch.from_numpy(np.ascontiguousarray(c["m0"])).to(dev)
    J = torch.zeros(plan.n_tx, dtype=torch.float64, device=dev)
    g = torch.empty(shape, dtype=torch.float64, device=dev)
    _lib.check(lib.usct_misfit_and_gradient_dev(plan.handle, P(m0), P(sd), P(wd), P(d), P(J),
                                                P(g), P(mws), P(bws), s))
    plan.check()
    out = (d.cpu().numpy(), J.cpu().numpy(), g.cpu().numpy())
    plan.close()
    return out


@pytest.mark.parametrize("name,C,tblock,k", [
    ("gpu3d", 8, 1608, 9), ("gpu3d", 16, 808, 8), ("gpu3d", 32, 808, 7),
    ("odd3d", 8, 804, 5), ("odd3d", 16, 1604, 6), ("parity3d", 32, 408, 10),
    ("parity3d", 64, 408, 11), ("cyl3d_point", 8, 1608, 0), ("gpu3d", 32, 1608, 8),
    ("gpu3d", 8, 1608, 249)])
def test_two_step_sweeps_equal_single_steps(eng, name, C, tblock, k):
    c = load(name)
    sl = c.src_list
    base = _run(eng, c, c["m_true"], sl, C, k, 0)
    two = _run(eng, c, c["m_true"], sl, C, k, tblock)
    for a, b in zip(base, two):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("nt_cut", [0, 1])
def test_two_step_sweeps_equal_the_fp32_oracle(eng, nt_cut):
    """Against the FP32 restatement directly, with an even and an odd number
    of levels to produce."""
    c = load("gpu3d")
    nt = c.nt - nt_cut
    sl = c.src_list[:8]
    d, J, g = _run(eng, c, c["m_true"], sl, 8, 12, 1, nt=nt)
    d32 = oracle.forward_fmc32(c["m_true"], c.geom, c.wavelet[:nt], c.dt, c.h, nt, None, sl)
    assert np.array_equal(d, d32)
    Jr, gr = oracle.misfit_and_gradient32(c["m0"], c.geom, c.wavelet[:nt], c.dt, c.h, nt,
                                          d.astype(np.float64), src_list=sl, C=8)
    assert np.array_equal(g, gr)


def test_two_step_sweeps_with_sponge_zchunks_and_rings(eng):
    from openusct_gb300.geometry import make_sponge
    c = load("gpu3d")
    sp = np.ascontiguousarray(make_sponge(c["m_true"].shape, width=4, strength=0.1))
    sl = c.src_list
    base = _run(eng, c, c["m_true"], sl, 16, 6, 0, sponge=sp)
    for zc, st in ((3, 43), (7, 32), (0, 65)):
        two = _run(eng, c, c["m_true"], sl, 16, 6, 808, sponge=sp, zchunk=zc, stages=st)
        for a, b in zip(base, two):
            assert np.array_equal(a, b), (zc, st)


def test_two_step_setting_is_refused_after_a_sweep(eng):
    _lib, gb = eng
    from openusct_gb300.geometry import element_csr
    c = load("gpu3d")
    tx, rx = element_csr(c.geom, c["m_true"].shape, c.src_list, None)
    plan = gb.Plan(c["m_true"].shape, c.h, c.dt, c.nt, tx, rx, batch=8)
    dev = torch.device("cuda", 0)
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    bws = torch.empty(plan.batch_bytes(_lib.MODE_FORWARD), dtype=torch.uint8, device=dev)
    d = torch.empty((plan.n_tx, c.nt, plan.n_rx), dtype=torch.float32, device=dev)
    md = torch.from_numpy(c["m_true"]).to(dev)
    wd = torch.from_numpy(c.wavelet).to(dev)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    lib = _lib.load()
    _lib.check(lib.usct_forward_fmc_dev(plan.handle, P(md), None, P(wd), P(d), P(mws), P(bws),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    with pytest.raises(_lib.USCTError, match="before the plan's first sweep"):
        plan.set("tblock", 1)
    plan.close()
