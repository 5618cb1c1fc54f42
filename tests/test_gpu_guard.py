"""Canary guard bands: every device buffer the library writes is followed by
1 MiB of a known byte pattern, and the pattern must survive a full gradient
(and forward, Born and TFM) run -- an overrun check that needs no memory
sanitizer."""

import ctypes

import numpy as np
import pytest

from golden_util import load

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GUARD = 1 << 20
PATTERN = 0xA5


@pytest.fixture(scope="module", autouse=True)
def cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from openusct_gb300 import build
    build.build()
    yield


def _guarded(nbytes):
    t = torch.full((int(nbytes) + GUARD,), PATTERN, dtype=torch.uint8, device="cuda")
    return t


def _intact(t, nbytes):
    tail = t[int(nbytes):].cpu().numpy()
    return bool(np.all(tail == PATTERN))


@pytest.mark.parametrize("name,C,mode", [("cyl3d_point", 2, 1), ("cyl3d_aperture", 4, 1),
                                         ("ring2d_sponge", 2, 1), ("odd3d", 4, 2),
                                         ("odd2d", 4, 2)])
def test_no_write_past_any_buffer(name, C, mode):
    from openusct_gb300 import _lib
    from openusct_gb300.backend import Plan
    from openusct_gb300.geometry import element_csr
    c = load(name)
    a = c.args()
    shape = c["m0"].shape
    tx, rx = element_csr(c.geom, shape, a["src_list"], a["footprints"])
    plan = Plan(shape, c.h, c.dt, c.nt, tx, rx, batch=C, ckpt_k=5)
    lib = _lib.load()
    P = lambda t: ctypes.c_void_p(t.data_ptr())   # noqa: E731
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    N = int(np.prod(shape))
    mb, bb = plan.model_bytes(), plan.batch_bytes(mode)
    nd = plan.n_tx * plan.nt * plan.n_rx
    mws, bws = _guarded(mb), _guarded(bb)
    traces, grad = _guarded(4 * nd), _guarded(8 * N)
    J = _guarded(8 * plan.n_tx)
    m = torch.from_numpy(c["m0"]).cuda()
    wav = torch.from_numpy(np.ascontiguousarray(c.wavelet[:c.nt])).cuda()
    sp = torch.from_numpy(a["sponge"]).cuda() if a["sponge"] is not None else None
    dobs = torch.from_numpy(np.ascontiguousarray(c["dobs"], np.float32)).cuda()
    v = torch.from_numpy(np.ascontiguousarray(c["m0"] * 0.01)).cuda() if mode == 2 else None
    _lib.check(lib.usct_model_prepare(plan.handle, P(mws), P(m), P(sp) if sp is not None else None,
                                      P(v) if v is not None else None, P(wav), s))
    for b in range(plan.nbatch):
        _lib.check(lib.usct_batch_forward(plan.handle, P(mws), P(bws), b, mode, P(traces), s))
        if mode == 1:
            _lib.check(lib.usct_batch_misfit(plan.handle, P(bws), b, P(dobs), P(J), s))
        _lib.check(lib.usct_batch_backward(plan.handle, P(mws), P(bws), b, s))
    _lib.check(lib.usct_model_gradient(plan.handle, P(mws), P(m), P(grad), s))
    plan.check()
    for t, n in ((mws, mb), (bws, bb), (traces, 4 * nd), (grad, 8 * N), (J, 8 * plan.n_tx)):
        assert _intact(t, n)
    plan.close()


def test_tfm_buffers_have_no_overrun():
    import os
    from golden_util import GOLDEN
    from openusct_gb300 import _lib
    from openusct_gb300.imaging import hilbert_taps
    z = np.load(os.path.join(GOLDEN, "tfm3d.npz"))
    lib = _lib.load()
    P = lambda t: ctypes.c_void_p(t.data_ptr())   # noqa: E731
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    data = torch.from_numpy(z["data"]).cuda()
    n_tx, nt, n_rx = z["data"].shape
    taps = torch.from_numpy(hilbert_taps(nt).astype(np.float32)).cuda()
    A = _guarded(8 * n_tx * n_rx * nt)
    _lib.check(lib.usct_analytic_dev(P(data), P(A), n_tx, nt, n_rx, P(taps), s))
    npix = 9
    pos = torch.from_numpy(np.ascontiguousarray(z["element_pos"])).cuda()
    axes = torch.from_numpy(np.stack([np.linspace(-0.008, 0.008, npix)] * 3)).cuda()
    re, im = _guarded(8 * npix ** 3), _guarded(8 * npix ** 3)
    _lib.check(lib.usct_tfm_dev(P(A), n_tx, n_rx, nt, P(pos), P(pos), 3, P(axes), npix,
                                ctypes.c_double(float(z["c"])), ctypes.c_double(float(z["fs"])),
                                P(re), P(im), s))
    W = _guarded(8 * n_tx * nt * n_rx)
    _lib.check(lib.usct_pwindow_dev(P(A), n_tx, nt, n_rx, ctypes.c_double(0.2),
                                    ctypes.c_double(40.0), ctypes.c_double(10.0), P(W), s))
    torch.cuda.synchronize()
    assert _intact(A, 8 * n_tx * n_rx * nt)
    assert _intact(re, 8 * npix ** 3) and _intact(im, 8 * npix ** 3)
    assert _intact(W, 8 * n_tx * nt * n_rx)


def test_uploads_cast_on_the_device_equal_numpy_casts():
    """Host arrays go up as they are and are cast on the device: the device
    values equal NumPy's astype bit for bit (FP64 -> FP32 rounding with
    overflow and subnormals, FP32 -> FP64 widening, ints, Fortran order), from
    concurrent threads too."""
    import threading
    from openusct_gb300 import backend
    rng = np.random.default_rng(3)
    dev = torch.device("cuda", 0)
    cases = [(rng.standard_normal((37, 129, 61)) * 10.0 ** rng.integers(-30, 30, (37, 129, 61)),
              torch.float32, np.float32),
             (rng.standard_normal(600001).astype(np.float32), torch.float64, np.float64),
             (rng.integers(-1000, 1000, (700, 500)), torch.float32, np.float32),
             (np.asfortranarray(rng.standard_normal((513, 1031))), torch.float32, np.float32)]
    for a, td, nd in cases:
        got = backend._to_dev(a, td, dev).cpu().numpy()
        with np.errstate(over="ignore"):
            want = np.ascontiguousarray(a, dtype=nd)
        assert got.shape == want.shape
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    errs = []

    def up(seed):
        b = np.random.default_rng(seed).standard_normal((300, 1000))
        for _ in range(5):
            if not np.array_equal(backend._to_dev(b, torch.float32, dev).cpu().numpy(),
                                  b.astype(np.float32)):
                errs.append(seed)
    ts = [threading.Thread(target=up, args=(s,)) for s in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs


def test_cached_plans_hold_at_most_their_share_of_memory(monkeypatch):
    """Workspaces kept with cached plans are capped in total: past the cap a
    call still runs (its workspace is allocated for the call) and gives the
    same result, and the held bytes stay under the cap."""
    from openusct_gb300 import backend as gb
    c = load("ring2d_point")
    a = c.args()
    gb.release()
    total = torch.cuda.get_device_properties(0).total_memory
    res = {}
    for cap_div in (4, total):   # the default cap, then one that keeps nothing
        monkeypatch.setattr(gb, "WS_HOLD_DIV", cap_div)
        gb.release()
        for shots in ([0], [1], [0, 1]):
            J, g = gb.misfit_and_gradient(c["m0"], c.geom, a["wavelet"], c.dt, c.h, c.nt,
                                          c["dobs"][shots], src_list=shots)
            res.setdefault(tuple(shots), []).append((J, g))
            assert gb._held_workspace_bytes() <= total // cap_div
    for runs in res.values():
        (J0, g0), (J1, g1) = runs
        assert J0 == J1 and np.array_equal(g0, g1)
    gb.release()
