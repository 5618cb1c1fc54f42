"""GPU: the autograd operator, CUDA-graph replay and the serving engine."""

import numpy as np
import pytest

import oracle
from golden_util import load, rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def cuda():
    assert torch.cuda.is_available()
    from openusct_gb300 import build
    build.build()


def test_autograd_l2_gradient_equals_misfit_and_gradient():
    import openusct_gb300.backend as gb
    from openusct_gb300.autograd import FMCProblem, fmc
    c = load("gpu3d")
    sl = c.src_list[:6]
    dobs = torch.from_numpy(c["dobs"][:6]).float().cuda()
    for keep in (None, 0):   # checkpoints kept from the forward / recomputed in backward
        prob = FMCProblem(c["m0"].shape, c.geom, c.wavelet, c.dt, c.h, c.nt, src_list=sl,
                          batch=4, ckpt_k=16, keep_bytes=keep)
        m = torch.from_numpy(c["m0"]).cuda().requires_grad_(True)
        tr = fmc(m, prob)
        loss = 0.5 * ((tr - dobs).double() ** 2).sum()
        loss.backward()
        J, g = gb.misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"][:6],
                                      src_list=sl, batch=4, ckpt_k=16)
        assert np.array_equal(m.grad.cpu().numpy(), g)
        assert abs(loss.item() - J) <= 1e-9 * J


def test_autograd_slowness_parametrisation_matches_fd():
    from openusct_gb300.autograd import FMCProblem, fmc
    c = load("parity3d")
    sl = c.src_list[:2]
    dobs = c["dobs"][:2]
    s0 = np.sqrt(c["m0"])
    prob = FMCProblem(s0.shape, c.geom, c.wavelet, c.dt, c.h, c.nt, src_list=sl, batch=2)
    s = torch.from_numpy(s0).cuda().requires_grad_(True)
    tr = fmc(s, prob, param="slowness")
    loss = 0.5 * ((tr - torch.from_numpy(dobs).float().cuda()) ** 2).double().sum()
    loss.backward()
    gs = s.grad.cpu().numpy()
    rng = np.random.default_rng(4)
    for _ in range(3):
        ds = rng.standard_normal(s0.shape)
        ds[:3] = ds[-3:] = ds[:, :3] = ds[:, -3:] = ds[:, :, :3] = ds[:, :, -3:] = 0.0
        ds *= float(np.mean(s0))
        eps = 1e-6
        Jp = oracle.misfit((s0 + eps * ds) ** 2, c.geom, c.wavelet, c.dt, c.h, c.nt, dobs,
                           src_list=sl)
        Jm = oracle.misfit((s0 - eps * ds) ** 2, c.geom, c.wavelet, c.dt, c.h, c.nt, dobs,
                           src_list=sl)
        fd = (Jp - Jm) / (2 * eps)
        assert abs(float(np.sum(gs * ds)) - fd) <= 1e-4 * abs(fd)


def test_graph_replay_is_bit_identical():
    import openusct_gb300.backend as gb
    c = load("parity2d")
    base = dict(src_list=c.src_list, batch=8, ckpt_k=20)
    J0, g0 = gb.misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                    tile=(128, 1, 0, 1), **base)
    plan = gb._PLANS[next(reversed(gb._PLANS))]
    plan.set("graphs", 1)
    outs = [gb.misfit_and_gradient(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                   tile=(128, 1, 0, 1), **base) for _ in range(3)]
    for J, g in outs:
        assert J == J0 and np.array_equal(g, g0)
    # a different model through the same captured graphs
    m1 = c["m0"] * 1.01
    J1, g1 = gb.misfit_and_gradient(m1, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                    tile=(128, 1, 0, 1), **base)
    plan.set("graphs", 0)
    J2, g2 = gb.misfit_and_gradient(m1, c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                                    tile=(128, 1, 0, 1), **base)
    assert J1 == J2 and np.array_equal(g1, g2)


def test_each_result_is_the_same_alone_and_in_the_mix():
    import openusct_gb300.backend as gb
    from openusct_gb300.serve import Engine, GpuExecutor, make_stream, summarize

    def dobs_fn(m, geom, wav, dt, h, nt):
        return gb.forward_fmc(m, geom, wav, dt, h, nt)

    reqs = make_stream(8, rate_hz=40.0, seed=3, sizes_2d=(96, 160), sizes_3d=(40, 56),
                       elements_2d=(16, 32), elements_3d=(16, 32), frac_gradient=0.5,
                       nt_cap=300, dobs_fn=dobs_fn)
    eng = Engine(GpuExecutor(), budget_bytes=40 << 30, max_active=4)
    mixed = eng.run_stream(reqs)
    st = summarize(mixed, eng)
    assert st.ok == len(reqs)
    assert eng.max_concurrent >= 2
    alone = Engine(GpuExecutor(), budget_bytes=40 << 30, max_active=1).run_stream(
        reqs, realtime=False)
    for a, b in zip(mixed, alone):
        assert a.ok and b.ok
        if a.kind == "forward":
            assert np.array_equal(a.traces, b.traces)
        else:
            assert a.J == b.J and np.array_equal(a.g, b.g)
    # and agree with the backend's own call (its batch width may differ, which
    # only re-associates the FP32 shot sum of the imaging condition)
    for r, q in zip(mixed, reqs):
        if q.kind == "gradient":
            J, g = gb.misfit_and_gradient(q.m, q.geom, q.wavelet, q.dt, q.h, q.nt, q.dobs)
            assert rel_l2(r.g, g) < 1e-5 and abs(r.J - J) <= 1e-9 * abs(J)


def test_gauss_newton_request_is_the_same_alone_in_the_mix_and_as_invert():
    """Four Gauss-Newton iterations served as one long-lived request (the
    reference's GN-beats-GD setup, test_gauss_newton.py:54-75) give the same
    final model and misfit history when served alone, when served among
    overlapping forward and gradient requests, and when run by
    ``invert(optimizer="gauss-newton")`` through the backend with the same
    batch width; and the misfit falls as the reference's test demands."""
    import openusct_gb300.backend as gb
    from openusct_gb300.invert import invert
    from openusct_gb300.serve import Engine, GpuExecutor, Request, make_stream

    c = load("gn_vs_gd2d")

    def gn_request(arrival):
        return Request(kind="gauss-newton", m=c["m0"].copy(), geom=c.geom, wavelet=c.wavelet,
                       dt=c.dt, h=c.h, nt=c.nt, dobs=c["dobs"], src_list=list(c.src_list),
                       update_mask=c["mask"], n_iter=4, n_cg=8, arrival=arrival, batch=4)

    def dobs_fn(m, geom, wav, dt, h, nt):
        return gb.forward_fmc(m, geom, wav, dt, h, nt)

    others = make_stream(5, rate_hz=40.0, seed=5, sizes_2d=(96, 160), sizes_3d=(40, 56),
                         elements_2d=(16, 32), elements_3d=(16, 32), frac_gradient=0.5,
                         nt_cap=300, dobs_fn=dobs_fn)
    mix = others[:2] + [gn_request(others[1].arrival + 0.01)] + others[2:]
    eng = Engine(GpuExecutor(), budget_bytes=40 << 30, max_active=4)
    mixed = eng.run_stream(mix)
    assert all(r.ok for r in mixed), [r.error for r in mixed]
    assert eng.max_concurrent >= 2
    served = mixed[2]
    alone = Engine(GpuExecutor(), budget_bytes=40 << 30, max_active=1).run_stream(
        [gn_request(0.0)], realtime=False)[0]
    assert alone.ok
    assert np.array_equal(served.m, alone.m) and served.history == alone.history
    m_inv, hist = invert(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"],
                         src_list=c.src_list, n_iter=4, update_mask=c["mask"],
                         optimizer="gauss-newton", n_cg=8, engine_options={"batch": 4})
    assert np.array_equal(served.m, m_inv) and served.history == [float(v) for v in hist]
    assert served.history[-1] / served.history[0] < 0.05


def test_bounded_wait_reports_and_recovers():
    """A TMA stage whose bytes never all arrive: the kernel's bounded wait gives
    up, the error is reported on the host, later launches skip their work, and
    the context stays usable for a correct run afterwards."""
    import openusct_gb300.backend as gb
    from openusct_gb300._lib import USCTError
    c = load("cyl3d_point")
    args = (c["m_true"], c.geom, c.wavelet, c.dt, c.h, c.nt, None, c.src_list)
    ref = gb.forward_fmc(*args, batch=4, tile=(32, 8, 0, 1))
    plan = gb._PLANS[next(reversed(gb._PLANS))]
    assert plan.info("variant") == 1
    plan.set("wait_test", 1)
    with pytest.raises(USCTError, match="gave up waiting"):
        gb.forward_fmc(*args, batch=4, tile=(32, 8, 0, 1))
    plan.set("wait_test", 0)
    again = gb.forward_fmc(*args, batch=4, tile=(32, 8, 0, 1))
    assert np.array_equal(again, ref)


def test_cancel_mid_flight_then_serve_normally():
    """A request cancelled while it runs stops at a shot-batch boundary (one
    shot per batch here, 64 batches), releases its budget and slot, and the
    next request on the same device is computed exactly as when served alone."""
    import threading
    import openusct_gb300.backend as gb
    from openusct_gb300.geometry import RingGeometry, ricker
    from openusct_gb300.serve import Engine, GpuExecutor, Request
    h = 2e-4
    geom = RingGeometry(64, 0.4 * 127 * h, 127 * h, h)
    n = geom.n
    m = np.full((n, n), 1.0 / 1500.0 ** 2)
    dt = 0.3 * h / 1500.0
    nt = 1500      # one shot per batch: about a second for all 64 batches
    wav = ricker(nt, dt, 1e6)
    dobs = gb.forward_fmc(m * 0.98, geom, wav, dt, h, nt)
    long_req = Request(kind="gradient", m=m, geom=geom, wavelet=wav, dt=dt, h=h, nt=nt,
                       dobs=dobs, batch=1)
    short = Request(kind="gradient", m=m, geom=geom, wavelet=wav, dt=dt, h=h, nt=nt,
                    dobs=dobs[[3, 9]], src_list=[3, 9], batch=2, arrival=0.0)
    eng = Engine(GpuExecutor(), budget_bytes=40 << 30, max_active=1)
    threading.Timer(0.25, long_req.cancel).start()
    res = eng.run_stream([long_req], realtime=False)
    assert not res[0].ok and res[0].error.startswith("Cancelled")
    k = int(res[0].error.split("after ")[1].split(" of")[0])
    assert 0 < k < 64
    assert eng.reserved == 0 and eng.active == 0
    after = eng.run_stream([short], realtime=False)[0]
    alone = Engine(GpuExecutor(), budget_bytes=40 << 30, max_active=1).run_stream(
        [Request(kind="gradient", m=m, geom=geom, wavelet=wav, dt=dt, h=h, nt=nt,
                 dobs=dobs[[3, 9]], src_list=[3, 9], batch=2)], realtime=False)[0]
    assert after.ok and after.J == alone.J and np.array_equal(after.g, alone.g)


def test_concurrent_backend_calls_on_one_plan_are_exact():
    """Four threads calling the backend with the same problem share one cached
    plan and its workspaces; the plan lock serialises them, so every result
    equals the single-threaded one bit for bit (the reference's C++ core is
    reentrant; so is this backend)."""
    import threading
    import openusct_gb300.backend as gb
    c = load("ring2d_point")
    args = (c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, c["dobs"])
    J0, g0 = gb.misfit_and_gradient(*args, src_list=c.src_list)
    d0 = gb.forward_fmc(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt, src_list=c.src_list)
    out, errs = [], []

    def work():
        try:
            for _ in range(3):
                J, g = gb.misfit_and_gradient(*args, src_list=c.src_list)
                d = gb.forward_fmc(c["m0"], c.geom, c.wavelet, c.dt, c.h, c.nt,
                                   src_list=c.src_list)
                out.append((J, g, d))
        except Exception as exc:     # reported below
            errs.append(exc)

    ts = [threading.Thread(target=work) for _ in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs, errs
    assert len(out) == 12
    for J, g, d in out:
        assert J == J0 and np.array_equal(g, g0) and np.array_equal(d, d0)


def test_served_gcn_and_windowed_gradients_match_the_backend():
    """Gradient requests may carry the GCN misfit and data windows; the served
    result equals the backend's own call bit for bit (same batch width)."""
    import openusct_gb300.backend as gb
    from openusct_gb300.serve import Engine, GpuExecutor, Request
    c = load("ring2d_window")
    reqs = [Request(kind="gradient", m=c["m0"], geom=c.geom, wavelet=c.wavelet, dt=c.dt, h=c.h,
                    nt=c.nt, dobs=c["dobs"], src_list=c.src_list, batch=2, misfit_type=mt,
                    time_weights=tw)
            for mt, tw in (("gcn", None), ("l2", c["tw"]), ("gcn", c["tw"]))]
    res = Engine(GpuExecutor(), budget_bytes=8 << 30, max_active=2).run_stream(reqs,
                                                                              realtime=False)
    for r, q in zip(res, reqs):
        assert r.ok, r.error
        J, g = gb.misfit_and_gradient(q.m, q.geom, q.wavelet, q.dt, q.h, q.nt, q.dobs,
                                      src_list=q.src_list, misfit_type=q.misfit_type,
                                      time_weights=q.time_weights, batch=2)
        assert np.array_equal(r.g, g) and r.J == J
