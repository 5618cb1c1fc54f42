"""Shots on different models in one launch (usct_plan_set_channel_models).

Forward requests of the same grid, spacing, time axis and wavelet share one
plan whose shot channels carry their own models, one per group of four
channels (each request padded to whole groups with transmits that inject
nothing).  The model operand is the same FP32 value per cell that the
one-model plan broadcasts, so every request's traces must be bit-identical to
its own plan's -- in 2D and 3D, with the group's transmits spread over several
batches -- and a served group must give each request exactly what it gets
when served alone.
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


def _group_traces(eng, models, geoms, src_lists, c, C):
    """Traces of several requests through one plan with per-channel models."""
    _lib, gb = eng
    from openusct_gb300.geometry import element_csr
    from openusct_gb300.serve import _concat_csr, _pad_rows, _union_rows
    shape = models[0].shape
    parts = [element_csr(g, shape, sl, None) for g, sl in zip(geoms, src_lists)]
    padded = [_pad_rows(t, 4) for t, _ in parts]
    tx = _concat_csr(padded)
    rx, rx_of = _union_rows([r for _, r in parts])
    plan = gb.Plan(shape, c.h, c.dt, c.nt, tx, rx, batch=C)
    owner = np.concatenate([np.full(t.rows, i, np.int32) for i, t in enumerate(padded)])
    lib = _lib.load()
    _lib.check(lib.usct_plan_set_channel_models(plan.handle, len(models),
                                                owner.ctypes.data_as(_lib._ip)))
    dev = torch.device("cuda", 0)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    md = torch.from_numpy(np.stack(models)).to(dev)
    wd = torch.from_numpy(c.wavelet).to(dev)
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    bws = torch.empty(plan.batch_bytes(_lib.MODE_FORWARD), dtype=torch.uint8, device=dev)
    d = torch.empty((plan.n_tx, c.nt, plan.n_rx), dtype=torch.float32, device=dev)
    _lib.check(lib.usct_model_prepare_channels(plan.handle, P(mws), P(md), P(wd), s))
    for b in range(plan.nbatch):
        _lib.check(lib.usct_batch_forward(plan.handle, P(mws), P(bws), b, _lib.MODE_FORWARD, P(d),
                                          s))
    plan.check()
    host = d.cpu().numpy()
    out, t0 = [], 0
    for (t, _), tp, ix in zip(parts, padded, rx_of):
        out.append(host[t0:t0 + t.rows][:, :, ix])
        t0 += tp.rows
    plan.close()
    return out


@pytest.mark.parametrize("name,C", [("parity2d", 8), ("gpu3d", 16), ("gpu3d", 4)])
def test_per_channel_models_equal_each_models_own_plan(eng, name, C):
    _lib, gb = eng
    c = load(name)
    rng = np.random.default_rng(3)
    models = [c["m_true"], c["m0"], c["m_true"] * (1.0 + 0.01 * rng.standard_normal(c["m0"].shape))]
    src = [c.src_list[:3], c.src_list[1:6], c.src_list[:5]]   # 13 transmits: several batches
    got = _group_traces(eng, [np.ascontiguousarray(m) for m in models], [c.geom] * 3, src, c, C)
    for m, sl, g in zip(models, src, got):
        alone = gb.forward_fmc(m, c.geom, c.wavelet, c.dt, c.h, c.nt, None, sl, batch=C)
        assert np.array_equal(g, alone)
        assert np.array_equal(g, oracle.forward_fmc32(m, c.geom, c.wavelet, c.dt, c.h, c.nt,
                                                      None, sl))


def test_per_channel_models_are_refused_for_gradients(eng):
    _lib, gb = eng
    from openusct_gb300.geometry import element_csr
    c = load("parity2d")
    tx, rx = element_csr(c.geom, c["m0"].shape, c.src_list, None)
    plan = gb.Plan(c["m0"].shape, c.h, c.dt, c.nt, tx, rx, batch=8)
    owner = np.zeros(tx.rows, np.int32)
    lib = _lib.load()
    _lib.check(lib.usct_plan_set_channel_models(plan.handle, 1, owner.ctypes.data_as(_lib._ip)))
    dev = torch.device("cuda", 0)
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    bws = torch.empty(plan.batch_bytes(_lib.MODE_GRADIENT), dtype=torch.uint8, device=dev)
    rc = lib.usct_batch_forward(plan.handle, ctypes.c_void_p(mws.data_ptr()),
                                ctypes.c_void_p(bws.data_ptr()), 0, _lib.MODE_GRADIENT, None,
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.USCT_ERR_ARG and b"forward sweeps only" in lib.usct_last_error()
    bad = np.full(tx.rows, 3, np.int32)
    assert lib.usct_plan_set_channel_models(plan.handle, 2, bad.ctypes.data_as(_lib._ip)) \
        == _lib.USCT_ERR_ARG
    mixed = np.zeros(tx.rows, np.int32)
    mixed[5] = 1                      # transmits 4..7 would need two models
    assert lib.usct_plan_set_channel_models(plan.handle, 2, mixed.ctypes.data_as(_lib._ip)) \
        == _lib.USCT_ERR_ARG and b"group of four" in lib.usct_last_error()
    plan.close()


def test_served_forward_requests_share_launches_and_match_alone(eng):
    """Compatible small forward requests waiting together are served in one
    launch group; each result equals the same request served alone."""
    from openusct_gb300.geometry import RingGeometry, ricker
    from openusct_gb300.serve import Engine, GpuExecutor, Request

    n, h = 96, 0.15e-3
    ring = RingGeometry(16, 0.8 * (n - 1) * h / 2, (n - 1) * h, h)
    dt = 0.3 * h / 1580.0
    nt = 400
    wav = ricker(nt, dt, 1e6)
    rng = np.random.default_rng(9)
    reqs = []
    for k in range(5):
        c = np.full((n, n), 1500.0)
        cx, cy = rng.uniform(35, 60, size=2)
        yy, xx = np.mgrid[0:n, 0:n]
        c[(yy - cy) ** 2 + (xx - cx) ** 2 <= 64] = 1580.0
        reqs.append(Request(kind="forward", m=1.0 / c ** 2, geom=ring, wavelet=wav, dt=dt, h=h,
                            nt=nt, src_list=list(range(k, k + 5)), arrival=0.001 * k))
    ex = GpuExecutor()                 # shared launches are the default
    mixed = Engine(ex, budget_bytes=20 << 30, max_active=1).run_stream(reqs, realtime=False)
    assert all(r.ok for r in mixed), [r.error for r in mixed]
    assert max(r.group for r in mixed) > 1
    alone = [Engine(GpuExecutor(merge=False), budget_bytes=20 << 30, max_active=1).run_stream(
        [Request(kind="forward", m=q.m, geom=q.geom, wavelet=q.wavelet, dt=q.dt, h=q.h, nt=q.nt,
                 src_list=q.src_list)], realtime=False)[0] for q in reqs]
    for a, b in zip(mixed, alone):
        assert b.ok and b.group == 1
        assert np.array_equal(a.traces, b.traces)
