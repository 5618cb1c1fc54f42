"""Host-side logic: element placement, CSR construction, batching arithmetic."""

import numpy as np
import pytest

from golden_util import load
from openusct_gb300 import geometry
from openusct_gb300.backend import batch_bytes_estimate, choose_batch


def test_ring_geometry_matches_reference_placement():
    # the golden ring was made by ringfwi.geometry.RingArray(8, 0.024, 0.06, 1e-3)
    c = load("ring2d_point")
    ring = geometry.RingGeometry(8, 0.024, 0.06, 1e-3)
    assert ring.n == c["m0"].shape[0]
    assert [tuple(t) for t in ring.idx] == [tuple(int(v) for v in r) for r in c["idx"]]


def test_cylinder_geometry_matches_reference_placement():
    c = load("cyl3d_point")
    cyl = geometry.CylinderGeometry(2, 6, 0.010, 0.012, 0.03, 1.5e-3)
    assert cyl.n == c["m0"].shape[0]
    assert [tuple(t) for t in cyl.idx] == [tuple(int(v) for v in r) for r in c["idx"]]


def test_ricker_matches_reference_wavelet():
    c = load("ring2d_point")
    w = geometry.ricker(c.nt, c.dt, 0.4e6)
    assert np.array_equal(w, c.wavelet)


def test_linear_indices_row_major():
    shape = (5, 7, 11)
    idx = [(0, 0, 0), (4, 6, 10), (2, 3, 4)]
    lin = geometry.linear_indices(idx, shape)
    assert list(lin) == [int(np.ravel_multi_index(t, shape)) for t in idx]
    with pytest.raises(ValueError):
        geometry.linear_indices([(5, 0, 0)], shape)


def test_element_csr_points_and_src_list():
    g = geometry.IndexGeometry([(1, 2), (3, 4), (5, 6)])
    tx, rx = geometry.element_csr(g, (8, 9), src_list=[2, 0])
    assert list(tx.ptr) == [0, 1, 2] and list(tx.cell) == [5 * 9 + 6, 1 * 9 + 2]
    assert list(rx.ptr) == [0, 1, 2, 3] and np.all(rx.w == 1.0)
    with pytest.raises(ValueError):
        geometry.element_csr(g, (8, 9), src_list=[3])


def test_element_csr_footprints():
    c = load("ring2d_aperture")
    tx, rx = geometry.element_csr(c.geom, c["m0"].shape, c.src_list, c.footprints)
    assert rx.rows == len(c.footprints)
    assert tx.rows == len(c.src_list)
    for j, (cells, w) in enumerate(c.footprints):
        a, b = rx.ptr[j], rx.ptr[j + 1]
        assert b - a == len(cells)
        assert np.isclose(rx.w[a:b].sum(), 1.0)
        assert list(rx.cell[a:b]) == list(geometry.linear_indices(cells, c["m0"].shape))


def test_element_csr_rows_are_the_elements_rows():
    """Transmit row i is receiver row src_list[i] (cells, weights, dtypes), for
    point elements and footprints, repeated and reordered transmits, 2D and 3D."""
    c = load("ring2d_aperture")
    g3 = geometry.IndexGeometry([(1, 2, 3), (4, 4, 4), (0, 5, 6)])
    cases = [(c.geom, c["m0"].shape, [3, 1, 3, 0], None),
             (c.geom, c["m0"].shape, c.src_list[::-1] + c.src_list[:2], c.footprints),
             (c.geom, c["m0"].shape, [], c.footprints),
             (g3, (5, 6, 7), None, None)]
    for geom, shape, src, fp in cases:
        tx, rx = geometry.element_csr(geom, shape, src, fp)
        src = list(range(rx.rows)) if src is None else src
        assert tx.ptr.dtype == np.int32 and tx.cell.dtype == np.int64 and tx.w.dtype == np.float64
        assert tx.rows == len(src) and tx.ptr[0] == 0
        for i, s in enumerate(src):
            a, b = tx.ptr[i], tx.ptr[i + 1]
            ra, rb = rx.ptr[s], rx.ptr[s + 1]
            assert np.array_equal(tx.cell[a:b], rx.cell[ra:rb])
            assert np.array_equal(tx.w[a:b], rx.w[ra:rb])


def test_batch_choice_respects_budget():
    shape, nt = (192, 192, 192), 2000
    full = batch_bytes_estimate(shape, nt, 256, 256, 32, 64, 1)
    # 32 shots x (4 + 2*32 + 64) levels of 28.3 MB
    assert 110e9 < full < 125e9
    assert choose_batch(shape, nt, 256, 256, 256, 64, 1, full) == 32
    assert choose_batch(shape, nt, 256, 256, 256, 64, 1, full - 1) == 16
    assert choose_batch((61, 61), 350, 2, 8, 8, 0, 1, 1 << 40) == 2


def test_smoothing_taps_are_scipys_gaussian_kernel():
    """The taps handed to usct_smooth_dev are exactly scipy's: filtering a unit
    impulse with gaussian_filter1d returns the kernel itself."""
    from scipy.ndimage import gaussian_filter1d
    from openusct_gb300.invert import smoothing_taps
    for sigma in (0.3, 1.0, 1.7, 3.0):
        t = smoothing_taps(sigma)
        r = len(t) - 1
        delta = np.zeros(4 * r + 9)
        delta[2 * r + 4] = 1.0
        k = gaussian_filter1d(delta, sigma)
        assert np.array_equal(k[2 * r + 4:3 * r + 5], t)
        assert np.array_equal(k[r + 4:2 * r + 5][::-1], t)


def test_smoothing_order_reproduces_scipy_bit_for_bit():
    """The order usct_smooth_dev adds taps in (centre first, then the pairs from
    the outermost in, 'reflect' extension with period 2n, axes in order)
    reproduces scipy.ndimage.gaussian_filter exactly, including a radius larger
    than an axis."""
    from scipy.ndimage import gaussian_filter
    from openusct_gb300.invert import smoothing_taps

    def refl(i, n):
        k = i % (2 * n)
        return 2 * n - 1 - k if k >= n else k

    def pass_axis(x, axis, t):
        r = len(t) - 1
        xm = np.moveaxis(x, axis, -1)
        out = np.empty_like(xm)
        n = xm.shape[-1]
        for i in range(n):
            acc = xm[..., i] * t[0]
            for j in range(r, 0, -1):
                acc = acc + (xm[..., refl(i - j, n)] + xm[..., refl(i + j, n)]) * t[j]
            out[..., i] = acc
        return np.moveaxis(out, -1, axis)

    rng = np.random.default_rng(3)
    for shape, sigma in (((9, 13, 11), 1.0), ((3, 5), 2.0), ((17,), 1.3)):
        x = rng.standard_normal(shape)
        t = smoothing_taps(sigma)
        y = x
        for ax in range(x.ndim):
            y = pass_axis(y, ax, t)
        assert np.array_equal(y, gaussian_filter(x, sigma))


def test_hilbert_taps_reproduce_scipy_hilbert():
    """x + i (x circularly convolved with hilbert_taps) == scipy.signal.hilbert,
    for even and odd lengths (the identity usct_analytic_dev computes)."""
    from scipy.signal import hilbert
    from openusct_gb300.imaging import hilbert_taps
    rng = np.random.default_rng(5)
    for nt in (64, 97, 320, 1501):
        x = rng.standard_normal(nt)
        g = hilbert_taps(nt)
        idx = (np.arange(nt)[:, None] - np.arange(nt)[None, :]) % nt
        y = (g[idx] * x[None, :]).sum(axis=1)
        a = hilbert(x)
        assert np.allclose(a.real, x, atol=1e-12)
        assert np.allclose(a.imag, y, atol=1e-12 * np.abs(x).max() * nt)


def test_tfm_fp32_index_margin_holds():
    """k_tfm decides a sample index in FP32, (d_tx + d_rx) * (fs / c), and
    falls back to the reference's FP64 expression within 1e-6 * v + 1e-5 of a
    half-integer.  On ring geometries the FP32 value stays within 2e-7 * v of
    the FP64 one, so outside the margin both round to the same index."""
    rng = np.random.default_rng(1)
    for c, dt, R, npix in ((1480.0, 1.5e-7, 0.02, 61), (1500.0, 0.3 * 0.15e-3 / 1580, 0.016, 80)):
        fs = 1.0 / dt
        ang = rng.uniform(0, 2 * np.pi, 48)
        epos = np.stack([R * np.cos(ang), R * np.sin(ang)], 1)
        ax = np.linspace(-0.95 * R, 0.95 * R, npix)
        X, Y = np.meshgrid(ax, ax, indexing="ij")
        pts = np.stack([X.ravel(), Y.ravel()], 1)
        d = np.sqrt(((pts[:, None, :] - epos[None, :, :]) ** 2).sum(axis=2))
        d32 = d.astype(np.float32)
        rate = np.float32(fs / c)
        for i in range(0, 48, 5):
            v64 = ((d[:, i][:, None] + d) / c) * fs
            v = (d32[:, i][:, None] + d32) * rate
            assert np.all(np.abs(v.astype(np.float64) - v64) <= 2e-7 * v64 + 1e-9)
            fr = v - np.floor(v)
            outside = np.abs(fr - np.float32(0.5)) > np.float32(1e-6) * v + np.float32(1e-5)
            assert np.array_equal(np.rint(v)[outside].astype(np.float64), np.round(v64)[outside])


def test_backend_validates_what_the_kernels_would_read():
    """Arrays the kernels index by the plan's sizes are checked on the host
    before anything is launched: the wavelet needs nt-1 samples (the last one
    may be missing, as in the reference), the sponge and v the model's shape,
    nt >= 2; an empty transmit list returns the reference's empty results."""
    import torch
    from openusct_gb300 import backend as gb
    dev = torch.device("cpu")
    w = gb._wavelet(np.arange(9.0), 10, dev)
    assert w.shape == (10,) and float(w[9]) == 0.0 and float(w[8]) == 8.0
    assert gb._wavelet(np.arange(12.0), 10, dev).shape == (10,)
    with pytest.raises(ValueError, match="wavelet"):
        gb._wavelet(np.arange(8.0), 10, dev)
    with pytest.raises(ValueError, match="sponge"):
        gb._grid_array(np.ones((4, 5)), (5, 4), "sponge", dev)
    assert gb._grid_array(None, (5, 4), "sponge", dev) is None

    class G:
        idx = [(1, 1), (2, 2), (3, 1)]
    m = np.ones((6, 6))
    d = gb.forward_fmc(m, G(), np.zeros(5), 1e-7, 1e-3, 5, src_list=[])
    assert d.shape == (0, 5, 3)
    J, g = gb.misfit_and_gradient(m, G(), np.zeros(5), 1e-7, 1e-3, 5, np.zeros((0, 5, 3)),
                                  src_list=[])
    assert J == 0.0 and np.array_equal(g, np.zeros((6, 6)))
    assert gb.misfit(m, G(), np.zeros(5), 1e-7, 1e-3, 5, np.zeros((0, 5, 3)), src_list=[]) == 0.0
    hv = gb.gn_hessian_vector(m, G(), np.zeros(5), 1e-7, 1e-3, 5, np.ones((6, 6)), src_list=[])
    assert np.array_equal(hv, np.zeros((6, 6)))


def test_backend_calls_hold_the_plan_lock():
    """Concurrent calls that hit one cached plan are serialised on its lock
    (the plan's workspaces are shared); the cache itself is guarded."""
    import inspect
    from openusct_gb300 import backend as gb
    for fn in (gb.forward_fmc, gb.misfit_and_gradient, gb.misfit, gb.gn_hessian_vector):
        src = inspect.getsource(fn)
        assert "with plan.lock:" in src, fn.__name__
    assert "_PLANS_LOCK" in inspect.getsource(gb.get_plan)


def _fp_csr(footprints):
    ptr, cells, w = [0], [], []
    for idxs, ws in footprints:
        for c, wi in zip(idxs, ws):
            cells.append(tuple(int(a) for a in c))
            w.append(float(wi))
        ptr.append(len(cells))
    return np.asarray(ptr, np.int32), np.asarray(cells, np.int32), np.asarray(w)


def test_geometry_and_footprints_equal_the_references():
    """Element placement of rings, cylinders, spheres and hemispheres and the
    finite-aperture footprints of every shape equal the reference's
    (footprints fixture) exactly: the same cells in the same order, the same
    weights."""
    import os
    from golden_util import GOLDEN
    from openusct_gb300.geometry import (CylinderGeometry, RingGeometry, ShellGeometry,
                                         build_footprints)
    z = np.load(os.path.join(GOLDEN, "footprints.npz"))
    gs = {"ring": RingGeometry(12, 0.02, 0.05, 1.0e-3),
          "cyl": CylinderGeometry(3, 10, 0.012, 0.012, 0.032, 8.0e-4),
          "sphere": ShellGeometry(20, 0.012, 0.032, 8.0e-4),
          "hemi": ShellGeometry(16, 0.012, 0.032, 8.0e-4, hemisphere=True)}
    cases = [("flat", 0.004, None), ("rect", 0.005, 0.003), ("disc", 0.005, 0.004),
             ("point", 0.004, None), ("rect", 0.0005, 0.0005), ("disc", 0.02, 0.02)]
    for gname, g in gs.items():
        assert np.array_equal(np.asarray(g.idx, np.int32), z[f"{gname}_idx"]), gname
        for ci, (shp, w, hgt) in enumerate(cases):
            p, c, wt = _fp_csr(build_footprints(g, width_m=w, shape=shp, height_m=hgt))
            assert np.array_equal(p, z[f"{gname}_{ci}_ptr"]), (gname, ci)
            assert np.array_equal(c, z[f"{gname}_{ci}_idx"]), (gname, ci)
            assert np.array_equal(wt, z[f"{gname}_{ci}_w"]), (gname, ci)


def test_autotune_cache_roundtrip(tmp_path, monkeypatch):
    """The autotuner's cache: a stored best launch shape is found again by
    (dimension, grid, batch width), other keys miss, a corrupt file is
    ignored."""
    from openusct_gb300 import autotune
    path = tmp_path / "tune.json"
    monkeypatch.setenv("OPENUSCT_GB300_CACHE", str(path))
    assert autotune.lookup((64, 64, 64), 16) is None
    autotune._save_cache({autotune.key((64, 64, 64), 16): {"tile": [32, 8, 0, 1], "results": []}})
    assert autotune.lookup((64, 64, 64), 16) == (32, 8, 0, 1)
    assert autotune.lookup((64, 64, 64), 32) is None
    assert autotune.lookup((64, 64), 16) is None
    path.write_text("{not json")
    assert autotune.lookup((64, 64, 64), 16) is None
    assert autotune._parse_tiles("64x4x0x1x6x4,32x8") == [(64, 4, 0, 1, 6, 4), (32, 8, 0)]


def test_make_sponge_matches_the_reference_and_extends_to_3d():
    import os
    import sys
    from openusct_gb300.geometry import make_sponge
    m = make_sponge((64, 80), width=10, strength=0.1)
    assert m.shape == (64, 80) and m[32, 40] == 1.0
    assert np.allclose(m, m[::-1, ::-1]) and m.min() > 0.0 and m.max() == 1.0
    assert m[0, 40] == np.exp(-((0.1 * 10) ** 2))
    m3 = make_sponge((40, 64, 80), width=10, strength=0.1)
    assert np.array_equal(m3[20], m) and m3.shape == (40, 64, 80)
    assert np.array_equal(m3[:, 32, 40], make_sponge((40, 30), 10, 0.1)[:, 15])
    for bad in ((8, 80), (64, 80, 5)):
        with pytest.raises(ValueError):
            make_sponge(bad, width=10)
    ref = os.path.join(os.environ.get("USCT_REFERENCE", ""), "simulation")
    if os.environ.get("USCT_REFERENCE") and os.path.isdir(ref):
        sys.path.insert(0, ref)
        try:
            from ringfwi.solver import make_sponge as ref_sponge
        finally:
            sys.path.remove(ref)
        for shape, w, s in (((64, 80), 10, 0.1), ((101, 101), 25, 0.08), ((50, 200), 20, 0.05)):
            assert np.array_equal(make_sponge(shape, w, s), ref_sponge(shape, w, s))


def test_bench_schedule_bytes_and_tail_interval():
    """The pipeline byte count bench.py reports: forward and adjoint on every
    level, the stash on the last segment, the recompute on the others; one
    segment is 32 C + 24 B per cell-step.  The backend's HBM-sized interval
    maximises the never-recomputed last segment within the budget."""
    import importlib.util
    import os
    from openusct_gb300 import _lib
    from openusct_gb300.backend import batch_bytes_estimate, tail_ckpt_k
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    cells, C, nt = 1000, 32, 2000
    one, rec, tail = bench.schedule_bytes(cells, C, nt, nt - 1, "grad")
    assert (rec, tail) == (0, nt - 1) and one == cells * (nt - 1) * (32 * C + 24)
    b64, rec, tail = bench.schedule_bytes(cells, C, nt, 64, "grad")
    assert (rec, tail) == (31 * 64, 1999 - 31 * 64)
    assert b64 == cells * (1999 * (12 * C + 4 + 16 * C + 20) + tail * 4 * C + rec * (16 * C + 4))
    gn, _, _ = bench.schedule_bytes(cells, C, nt, 64, "gn")
    assert gn - b64 == cells * 1999 * (12 * C + 4)
    shape, n_rx = (192, 192, 192), 256
    budget = int(0.7 * 284208 * 2 ** 20)
    k = tail_ckpt_k(shape, nt, n_rx, n_rx, C, _lib.MODE_GRADIENT, budget)
    assert batch_bytes_estimate(shape, nt, n_rx, n_rx, C, k, _lib.MODE_GRADIENT) <= budget
    _, _, tail_k = bench.schedule_bytes(1, C, nt, k, "grad")
    for kk in range(2, nt):
        if batch_bytes_estimate(shape, nt, n_rx, n_rx, C, kk, _lib.MODE_GRADIENT) <= budget:
            assert bench.schedule_bytes(1, C, nt, kk, "grad")[2] <= tail_k
    assert k == 200 and tail_k == 199


def test_default_checkpoint_interval_policy():
    """The public API's interval when none is given: one segment when the whole
    stash fits the workspace share, else the longest never-recomputed last
    segment that fits (192^3 / 32 shots: k = 200 within 70 % of a GB300), 0
    (the engine's memory-saving interval) when nothing fits; chosen once per
    problem, so a later call under memory pressure keeps the same plan; the
    fraction can be lowered."""
    from openusct_gb300 import _lib
    import openusct_gb300.backend as gb
    total = 284208 * 2 ** 20
    G = _lib.MODE_GRADIENT
    gb._DEFAULT_K.clear()
    try:
        assert gb.default_ckpt_k((256, 256), 1500, 64, 64, 64, G, avail=total, total=total) == 1499
        assert gb.default_ckpt_k((192, 192, 192), 2000, 256, 256, 32, G, avail=total,
                                 total=total) == 200
        assert gb.default_ckpt_k((192, 192, 192), 2000, 256, 256, 32, G, avail=10, total=total) == 0
        assert gb.default_ckpt_k((192, 192, 192), 2000, 256, 256, 32, _lib.MODE_FORWARD) == 0
        # what the device reported is remembered: a later call under memory
        # pressure keeps the same interval (and plan)
        free = [total, total]
        real = gb._available_bytes
        gb._available_bytes = lambda: tuple(free)
        try:
            assert gb.default_ckpt_k((192, 192, 192), 2000, 256, 256, 32, G) == 200
            free[0] = 1 << 30
            assert gb.default_ckpt_k((192, 192, 192), 2000, 256, 256, 32, G) == 200
        finally:
            gb._available_bytes = real
        small = gb.default_ckpt_k((192, 192, 192), 2000, 256, 256, 32, G, avail=total, total=total,
                                  budget_bytes=150 << 30)
        assert 0 < small < 200
        assert gb.batch_bytes_estimate((192, 192, 192), 2000, 256, 256, 32, small, G) <= 150 << 30
        gb.set_workspace_fraction(0.5)
        k5 = gb.default_ckpt_k((192, 192, 192), 2000, 256, 256, 32, G, avail=total, total=total)
        assert 0 < k5 < 200
        assert gb.batch_bytes_estimate((192, 192, 192), 2000, 256, 256, 32, k5, G) <= 0.5 * total
        with pytest.raises(ValueError):
            gb.set_workspace_fraction(1.5)
    finally:
        gb.set_workspace_fraction(0.7)


def test_plan_cache_builds_plans_without_deadlock(monkeypatch):
    """get_plan builds a plan while it holds the cache lock, and a plan
    registers itself as live on construction: the two must not share a lock
    (a stand-in plan runs the same registration, under a thread timeout)."""
    import threading
    import openusct_gb300.backend as gb

    class Key:
        def key(self):
            return ("k",)

    class StandIn:
        def __init__(self, *a, **k):
            self._ws = {}
            gb._register_live(self)

    monkeypatch.setattr(gb, "Plan", StandIn)
    monkeypatch.setattr(gb, "_PLANS", gb.OrderedDict())
    monkeypatch.setattr(gb.torch.cuda, "current_device", lambda: 0)
    out = []
    th = threading.Thread(target=lambda: out.append(gb.get_plan((8, 8), 1e-3, 1e-7, 10, Key(),
                                                                Key())), daemon=True)
    th.start()
    th.join(timeout=10)
    assert not th.is_alive(), "get_plan deadlocked"
    assert isinstance(out[0], StandIn) and out[0] in gb._LIVE_PLANS
    assert gb._held_workspace_bytes() >= 0


def test_cpu_arm_memory_plan():
    """The CPU arms keep the reference core's full-history plan (k = 0) when
    the FP64 history fits 65 % of the host's available memory, else the
    longest checkpoint interval whose checkpoints and segment fit; the
    Gauss-Newton restatement always checkpoints."""
    import importlib.util
    import os
    import types
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod2", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    prob = types.SimpleNamespace(shape=(192, 192, 192), nt=2000)
    N = 192 ** 3
    hist = 2000 * N * 8
    bench.host_available_bytes = lambda: 197 << 30
    assert bench.cpu_shot_interval(prob, "grad") == (0, hist)
    bench.host_available_bytes = lambda: 100 << 30
    k, need = bench.cpu_shot_interval(prob, "grad")
    assert 2 <= k < 1999 and need <= 0.65 * (100 << 30)
    nseg = (1999 + k - 1) // k
    assert need == (2 * nseg + k + 2) * N * 8
    # the next longer interval would not fit
    k2 = k + 1
    nseg2 = (1999 + k2 - 1) // k2
    assert (2 * nseg2 + k2 + 2) * N * 8 > 0.65 * (100 << 30)
    bench.host_available_bytes = lambda: 197 << 30
    kg, _ = bench.cpu_shot_interval(prob, "gn")
    assert kg > 0


def test_workspace_allocation_falls_back_to_releasing_caches(monkeypatch):
    """A workspace that does not fit first releases torch's cached blocks, and
    then the workspaces other plans keep between calls, before giving up."""
    import torch
    import openusct_gb300.backend as gb

    class StandIn:
        def __init__(self):
            self._ws = {"grad": "held"}
            gb._register_live(self)

    other = StandIn()
    calls = {"empty": 0, "cache": 0}

    def fake_empty(n, dtype=None, device=None):
        calls["empty"] += 1
        if calls["empty"] < 3:
            raise torch.cuda.OutOfMemoryError("out of memory")
        return torch.zeros(n, dtype=dtype)

    monkeypatch.setattr(gb.torch, "empty", fake_empty)
    monkeypatch.setattr(gb.torch.cuda, "empty_cache",
                        lambda: calls.__setitem__("cache", calls["cache"] + 1))
    t = gb._alloc_bytes(1000, "cpu")
    assert t.numel() == 1000 and calls == {"empty": 3, "cache": 2}
    assert other._ws == {}
