"""GB300 backend with the reference's backend protocol.

Use it wherever the reference accepts a ``backend=`` module::

    from ringfwi import fwi
    import openusct_gb300.backend as gb300
    m, hist = fwi.invert(m0, geom, wavelet, dt, h, nt, dobs, backend=gb300)
    plugins.run("fwi", dataset, backend=gb300)

Signatures follow ``simulation/ringfwi/fwi.py`` (forward_fmc :102, misfit :246,
misfit_and_gradient :266, gn_hessian_vector :410), which is the superset of the
reference's C++ (software/python/uap.py:34-67) and CuPy
(software/python/uap_gpu.py:166-233) backends; inputs are NumPy arrays (or CUDA
tensors), outputs are FP64 NumPy arrays like the reference's.  The misfits are
those of the reference C++ core, ``l2`` and ``gcn`` (uap.py:41); the Python-only
robust misfits raise NotImplementedError as the reference GPU backend does for
non-L2 (uap_gpu.py:191-192), an unknown one ValueError (fwi.py:243).

Everything runs on the CUDA kernels of ``libusct_gb300.so``; a missing library
or device raises instead of falling back to the CPU.
"""

from __future__ import annotations

import ctypes
import threading
import weakref
from collections import OrderedDict

import numpy as np
import torch

from . import _lib
from .geometry import CSR, element_csr

_KNOWN_MISFITS = ("l2", "gcn", "envelope", "egcn", "gsot", "traveltime")


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


_EXEC_STREAMS = {}


class _on_exec_stream:
    """Run the engine on a private per-device stream (capturable, so batch
    sweeps can be CUDA graphs) ordered after the caller's current stream."""

    def __enter__(self):
        dev = torch.cuda.current_device()
        st = _EXEC_STREAMS.get(dev)
        if st is None:
            st = _EXEC_STREAMS[dev] = torch.cuda.Stream(device=dev)
        st.wait_stream(torch.cuda.current_stream())
        self.stream = st
        return st

    def __exit__(self, *exc):
        torch.cuda.current_stream().wait_stream(self.stream)


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("openusct_gb300 needs a CUDA device (there is no CPU fallback)")


def _to_dev(x, dtype, device):
    """A host array or tensor as a contiguous device tensor of dtype.  Host
    data go up as they are and are cast on the device (the same round to
    nearest even as NumPy's astype): the GPU reads pageable host memory
    directly over the CPU link at ~150 GB/s, faster than any host-side pass
    over the data (an FP64 -> FP32 astype, or a copy into page-locked memory,
    takes 2-9 ms for the 49-131 MB FMCs of the benchmarked acquisitions)."""
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    a = np.asarray(x)
    if a.dtype not in (np.float64, np.float32):
        a = a.astype(np.float64)
    t = torch.from_numpy(np.ascontiguousarray(a)).to(device)
    return t if t.dtype == dtype else t.to(dtype)


class Plan:
    """A ``usct_plan``: grid, time axis, elements and batching on one device."""

    def __init__(self, shape, h, dt, nt, tx: CSR, rx: CSR, batch=0, ckpt_k=0, tile_x=0,
                 tile_y=0, zchunk=0, variant=None, stages=None):
        _require_cuda()
        lib = _lib.load()
        self.shape = tuple(int(s) for s in shape)
        self.h, self.dt, self.nt = float(h), float(dt), int(nt)
        self.tx, self.rx = tx, rx
        self.n_tx, self.n_rx = tx.rows, rx.rows
        dims = (ctypes.c_int * len(self.shape))(*self.shape)
        self._keep = (tx, rx)
        ptr = ctypes.c_void_p()
        _lib.check(lib.usct_plan_create(
            ctypes.byref(ptr), len(self.shape), dims, self.h, self.dt, self.nt,
            tx.rows, tx.ptr.ctypes.data_as(_lib._ip), tx.cell.ctypes.data_as(_lib._lp),
            tx.w.ctypes.data_as(_lib._dp), rx.rows, rx.ptr.ctypes.data_as(_lib._ip),
            rx.cell.ctypes.data_as(_lib._lp), rx.w.ctypes.data_as(_lib._dp), int(batch),
            int(ckpt_k), int(tile_x), int(tile_y), int(zchunk)))
        self._p = ptr
        self._lib = lib
        if variant is not None:
            self.set("variant", int(variant))
        if stages is not None:
            self.set("stages", int(stages))
        self._ws = {}
        self.lock = threading.RLock()
        _register_live(self)
        # launch-bound sizes replay whole batch sweeps as CUDA graphs
        level = int(np.prod(self.shape)) * max(1, self.batch)
        if level <= (1 << 22):
            self.set("graphs", 1)

    def workspace(self, kind, nbytes, device):
        """A workspace kept with the plan (stable buffers let captured graphs
        replay).  One larger than an eighth of the device, or one that would
        take the workspaces all cached plans hold past a quarter of it, is not
        kept: memory a plan does not hold goes back to torch's allocator for
        the caller's own tensors."""
        t = self._ws.get(kind)
        if t is not None and t.numel() >= nbytes:
            return t
        t = _alloc_bytes(nbytes, device)
        total = torch.cuda.get_device_properties(device).total_memory
        if nbytes <= total // 8 and \
                _held_workspace_bytes(self, kind) + nbytes <= total // WS_HOLD_DIV:
            self._ws[kind] = t
        return t

    def release(self):
        self._ws.clear()

    def set(self, key, value):
        _lib.check(self._lib.usct_plan_set(self._p, _lib.SET[key], int(value)))

    def check(self, stream=None):
        """Synchronise and raise if a pipelined kernel gave up waiting."""
        _lib.check(self._lib.usct_plan_check(self._p, _stream(stream)))

    @property
    def handle(self):
        return self._p

    def info(self, key):
        v = ctypes.c_int64()
        _lib.check(self._lib.usct_plan_info(self._p, _lib.INFO[key], ctypes.byref(v)))
        return int(v.value)

    @property
    def batch(self):
        return self.info("batch")

    @property
    def nbatch(self):
        return self.info("nbatch")

    def model_bytes(self):
        return int(self._lib.usct_model_bytes(self._p))

    def batch_bytes(self, mode):
        return int(self._lib.usct_batch_bytes(self._p, int(mode)))

    def plain_bytes(self, gradient):
        return int(self._lib.usct_plain_bytes(self._p, int(bool(gradient))))

    def close(self):
        self._ws = {}
        if getattr(self, "_p", None) is not None and self._p.value:
            self._lib.usct_plan_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_bytes_estimate(shape, nt, n_rx, nslot, C, ckpt_k, mode):
    """Bytes of one batch workspace (mirrors usct_batch_bytes)."""
    al = lambda x: (x + 255) // 256 * 256  # noqa: E731
    nx = shape[-1]
    nxs = (nx + 3) // 4 * 4
    rows = int(np.prod(shape[:-1]))
    lv = al(rows * nxs * C * 4)
    k = ckpt_k if ckpt_k else max(2, int(round((2.0 * (nt - 1)) ** 0.5)))
    k = min(k, max(2, nt - 1))
    nseg = (nt - 1 + k - 1) // k
    b = (2 * lv + al(nt * nslot * C * 4) + al(nt * n_rx * C * 4) + al(64 * C * 8) +
         al(n_rx * C * 8))
    if mode >= _lib.MODE_GRADIENT:
        b += (2 + 2 * nseg + k) * lv
    if mode == _lib.MODE_BORN:
        b += 2 * lv
    return b


def _available_bytes():
    """(bytes the allocator can still hand out, device total): the driver's
    free memory plus the blocks torch has cached but not in use."""
    free, total = torch.cuda.mem_get_info()
    return free + torch.cuda.memory_reserved() - torch.cuda.memory_allocated(), total


# Share of the device one gradient workspace may take when the caller gives no
# checkpoint interval; set_workspace_fraction lowers (or raises) it.
_WORKSPACE_FRACTION = 0.7
_DEFAULT_K = {}
_DEFAULT_K_LOCK = threading.Lock()


def set_workspace_fraction(fraction):
    """Cap, as a share of the device's memory, the batch workspace a gradient
    or Gauss-Newton call sizes for itself when it is given no checkpoint
    interval (default 0.7).  Intervals already chosen are forgotten."""
    global _WORKSPACE_FRACTION
    f = float(fraction)
    if not 0.0 < f <= 0.95:
        raise ValueError(f"workspace fraction must be in (0, 0.95], got {fraction}")
    with _DEFAULT_K_LOCK:
        _WORKSPACE_FRACTION = f
        _DEFAULT_K.clear()


def tail_ckpt_k(shape, nt, n_rx, nslot, C, mode, budget_bytes):
    """The checkpoint interval whose last segment -- the levels the forward
    sweep stashes itself, so the backward sweep never recomputes them -- is the
    longest while the batch workspace fits ``budget_bytes`` (ties: the smaller
    workspace); k = nt - 1 (one segment, nothing recomputed) when everything
    fits, 0 when not even the smallest workspace does."""
    nt = int(nt)
    best = None
    for k in range(2, nt):
        need = batch_bytes_estimate(shape, nt, n_rx, nslot, C, k, mode)
        if need > budget_bytes:
            continue
        nseg = (nt - 1 + k - 1) // k
        tail = nt - 1 - (nseg - 1) * k
        if best is None or (tail, -need) > best[:2]:
            best = (tail, -need, k)
    return best[2] if best else 0


def default_ckpt_k(shape, nt, n_rx, nslot, C, mode, avail=None, total=None, budget_bytes=None):
    """The checkpoint interval when the caller gives none: the one whose last
    segment (stashed by the forward sweep itself, never recomputed) is the
    longest while the batch workspace fits ``budget_bytes`` -- by default the
    workspace fraction (0.7) of the device, and never more than 90 % of what
    is available.  One segment (k = nt - 1, nothing recomputed: 32 C + 24
    instead of 44 C + 28 bytes per cell-step) when the whole stash fits, as for
    2D acquisitions; at the 192^3 / 32-shot gradient k = 200 (a 203 GB
    workspace: only the last 199 of 1999 levels are not recomputed).  0 (the
    engine's memory-saving k = sqrt(2 (nt - 1))) when nothing fits.  The
    gradient is bit-identical for every k.  The choice is made once per problem
    and device and then kept, so plans do not change with memory pressure."""
    if mode < _lib.MODE_GRADIENT or int(nt) < 3:
        return 0
    dev = torch.cuda.current_device() if torch.cuda.is_available() else -1
    key = (tuple(int(s) for s in shape), int(nt), int(n_rx), int(nslot), int(C), int(mode), dev,
           None if budget_bytes is None else int(budget_bytes), _WORKSPACE_FRACTION)
    measured = avail is None or total is None
    if measured:
        with _DEFAULT_K_LOCK:
            if key in _DEFAULT_K:
                return _DEFAULT_K[key]
        avail, total = _available_bytes()
    cap = _WORKSPACE_FRACTION * total if budget_bytes is None else budget_bytes
    k = tail_ckpt_k(shape, nt, n_rx, nslot, C, mode, int(min(cap, 0.9 * avail)))
    if measured:   # only what the device itself said is remembered
        with _DEFAULT_K_LOCK:
            _DEFAULT_K[key] = k
    return k


def choose_batch(shape, nt, n_tx, n_rx, nslot, ckpt_k, mode, budget):
    """Widest power-of-two shot batch (<= 64) whose workspace fits ``budget``."""
    C = 1
    while C < n_tx and C < 64:
        C *= 2
    while C > 1 and batch_bytes_estimate(shape, nt, n_rx, nslot, C, ckpt_k, mode) > budget:
        C //= 2
    return C


# cached plans together hold at most total memory // WS_HOLD_DIV of workspaces
WS_HOLD_DIV = 4


def _held_workspace_bytes(plan=None, kind=None):
    """Bytes of the workspaces every live plan holds (cached ones, and ones
    evicted from the cache that a caller still uses), not counting ``plan``'s
    workspace of ``kind`` (the one a new allocation replaces)."""
    with _LIVE_LOCK:
        plans = list(_LIVE_PLANS)
    if plan is not None and plan not in plans:
        plans.append(plan)
    held = 0
    for p in plans:
        for k, t in list(p._ws.items()):   # a copy made under the GIL
            if not (p is plan and k == kind):
                held += t.numel()
    return held


_PLANS: "OrderedDict[tuple, Plan]" = OrderedDict()
_LIVE_PLANS: "weakref.WeakSet[Plan]" = weakref.WeakSet()
_LIVE_LOCK = threading.Lock()


def _register_live(plan):
    """Count ``plan``'s workspaces against the cap while it is alive.  Its own
    lock: plans are built while get_plan holds _PLANS_LOCK."""
    with _LIVE_LOCK:
        _LIVE_PLANS.add(plan)
_MAX_PLANS = 8
_PLANS_LOCK = threading.Lock()


def get_plan(shape, h, dt, nt, tx, rx, batch=0, ckpt_k=0, tile_x=0, tile_y=0, zchunk=0,
             variant=None, stages=None):
    key = (tuple(shape), float(h), float(dt), int(nt), tx.key(), rx.key(), int(batch),
           int(ckpt_k), int(tile_x), int(tile_y), int(zchunk), variant, stages,
           torch.cuda.current_device())
    with _PLANS_LOCK:
        p = _PLANS.get(key)
        if p is None:
            p = Plan(shape, h, dt, nt, tx, rx, batch, ckpt_k, tile_x, tile_y, zchunk, variant,
                     stages)
            _PLANS[key] = p
            while len(_PLANS) > _MAX_PLANS:
                # dropped from the cache only: a call still holding it keeps it
                # alive, and it is destroyed when the last reference goes
                _PLANS.popitem(last=False)
        else:
            _PLANS.move_to_end(key)
        return p


def _setup(m, geom, h, dt, nt, src_list, footprints, mode, batch, ckpt_k, tile):
    _require_cuda()
    shape = tuple(np.shape(m))
    if len(shape) not in (2, 3):
        raise ValueError(f"model must be 2D or 3D, got shape {shape}")
    if int(nt) < 2:
        raise ValueError(f"nt must be >= 2 (got {nt}): the scheme has no step to take")
    tx, rx = element_csr(geom, shape, src_list, footprints)
    if not batch:
        free, _total = torch.cuda.mem_get_info()
        budget = int(0.7 * free)
        batch = choose_batch(shape, nt, tx.rows, rx.rows, len(rx.cell), ckpt_k or 0, mode,
                             budget)
    if not ckpt_k and mode >= _lib.MODE_GRADIENT:
        ckpt_k = default_ckpt_k(shape, nt, rx.rows, len(rx.cell), batch, mode)
    tile = tuple(tile) if tile else ()
    if len(tile) < 3:
        from .autotune import lookup
        tuned = lookup(shape, batch)
        tile = tuple(tuned) if tuned else (0, 0, 0)
    tile = tile + (None,) * (5 - len(tile))
    return get_plan(shape, h, dt, nt, tx, rx, batch, ckpt_k or 0, *tile)


def _drop_cached_workspaces():
    """Let go of the workspaces plans keep between calls (a call in flight
    holds its own references, so it is unaffected; later calls allocate
    again)."""
    with _LIVE_LOCK:
        plans = list(_LIVE_PLANS)
    for p in plans:
        p._ws = {}


def _alloc_bytes(nbytes, device):
    """A byte buffer on the device.  The interval a gradient sizes for itself
    counts the blocks torch has cached but not in use as available; one large
    workspace may not be carved from them, so on running out they are handed
    back to the driver and the allocation is tried again, and then once more
    after the workspaces other plans keep cached are let go as well."""
    n = max(int(nbytes), 256)
    try:
        return torch.empty(n, dtype=torch.uint8, device=device)
    except torch.cuda.OutOfMemoryError:
        torch.cuda.empty_cache()
    try:
        return torch.empty(n, dtype=torch.uint8, device=device)
    except torch.cuda.OutOfMemoryError:
        _drop_cached_workspaces()
        torch.cuda.empty_cache()
    return torch.empty(n, dtype=torch.uint8, device=device)


def _workspace(nbytes, device):
    return _alloc_bytes(nbytes, device)


def _out(x, like):
    """Host FP64 NumPy output unless the caller passed CUDA tensors."""
    if isinstance(like, torch.Tensor) and like.is_cuda:
        return x
    # widened on the device (exact), so the host only receives the bytes
    return x.detach().to(torch.float64).cpu().numpy()


_MISFIT_CODES = {"l2": 0, "gcn": 1}


def _check_misfit(misfit_type):
    """Returns the engine's code for misfit_type (l2 = 0, gcn = 1, as uap.py:41)."""
    if misfit_type not in _KNOWN_MISFITS:
        raise ValueError(f"unknown misfit_type {misfit_type!r}")
    if misfit_type not in _MISFIT_CODES:
        raise NotImplementedError("the GB300 backend implements the l2 and gcn misfits")
    return _MISFIT_CODES[misfit_type]


def _time_weights(time_weights, plan, dev):
    """The per-transmit data windows of fwi.py:250-259 as one device FP32
    (n_tx, nt, n_rx) array: entry i windows the i-th transmit of src_list.
    Accepts a list of (nt, n_rx) arrays or one stacked array/tensor."""
    if time_weights is None:
        return None
    if torch.is_tensor(time_weights):
        w = time_weights.to(device=dev, dtype=torch.float32)
    else:
        if isinstance(time_weights, (list, tuple)):
            time_weights = np.stack([np.asarray(t, dtype=np.float64) for t in time_weights])
        w = torch.from_numpy(np.ascontiguousarray(time_weights, dtype=np.float32)).to(dev)
    want = (plan.n_tx, plan.nt, plan.n_rx)
    if tuple(w.shape) != want:
        raise ValueError(f"time_weights have shape {tuple(w.shape)}, expected {want} "
                         "(one (nt, n_rx) window per transmit)")
    return w.contiguous()


def _wavelet(wavelet, nt, dev):
    """The source series as exactly nt FP64 device samples.  The scheme reads
    samples 0..nt-2 (fwi.py:65-66 injects series[n-1] for n < nt): fewer than
    nt-1 is an error, as in the reference; the unused last sample may be
    missing, extra samples are ignored."""
    w = _to_dev(wavelet, torch.float64, dev).reshape(-1)
    nt = int(nt)
    if w.numel() < nt - 1:
        raise ValueError(f"the wavelet has {w.numel()} samples; nt = {nt} needs at least {nt - 1}")
    if w.numel() < nt:
        w = torch.cat([w, w.new_zeros(nt - w.numel())])
    return w[:nt].contiguous()


def _grid_array(x, shape, name, dev):
    """A model-shaped FP64 device array (sponge, v), shape-checked."""
    if x is None:
        return None
    t = _to_dev(x, torch.float64, dev)
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, the model {tuple(shape)}")
    return t


def _no_shots(src_list):
    """An explicitly empty transmit list: the reference's loops run zero times
    (fwi.py:113-118, 294-331), so there is nothing to launch."""
    return src_list is not None and len(list(src_list)) == 0


def _zeros(shape, like):
    if isinstance(like, torch.Tensor) and like.is_cuda:
        return torch.zeros(shape, dtype=torch.float64, device=like.device)
    return np.zeros(shape)


def _n_receivers(geom, shape, footprints):
    return len(footprints) if footprints is not None else len(geom.idx)


# ---------------------------------------------------------------------------
# public API (signature-compatible with ringfwi.fwi)
# ---------------------------------------------------------------------------
def forward_fmc(m, geom, wavelet, dt, h, nt, sponge=None, src_list=None, footprints=None, *,
                batch=None, tile=None):
    """Full-matrix capture: data[i, n, j] = receiver j at level n for transmit i."""
    if _no_shots(src_list):
        return _zeros((0, int(nt), _n_receivers(geom, np.shape(m), footprints)), m)
    plan = _setup(m, geom, h, dt, nt, src_list, footprints, _lib.MODE_FORWARD, batch, None, tile)
    with plan.lock:   # one call at a time per plan: its workspaces are shared
        dev = torch.device("cuda", torch.cuda.current_device())
        md = _to_dev(m, torch.float64, dev)
        wd = _wavelet(wavelet, nt, dev)
        sd = _grid_array(sponge, np.shape(m), "sponge", dev)
        nd = plan.n_tx * plan.nt * plan.n_rx
        # a buffer kept with the plan, so a captured sweep replays into the same place
        dbuf = plan.workspace("traces", 4 * nd, dev)[: 4 * nd].view(torch.float32)
        mws = plan.workspace("model", plan.model_bytes(), dev)
        bws = plan.workspace(_lib.MODE_FORWARD, plan.batch_bytes(_lib.MODE_FORWARD), dev)
        with _on_exec_stream() as st:
            _lib.check(plan._lib.usct_forward_fmc_dev(plan.handle, _ptr(md), _ptr(sd), _ptr(wd),
                                                      _ptr(dbuf), _ptr(mws), _ptr(bws), _stream(st)))
            plan.check(st)
            with torch.cuda.stream(st):   # copied out before the next call may reuse the buffer
                data = dbuf.view(plan.n_tx, plan.nt, plan.n_rx).clone()
        return _out(data, m)


def misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None,
                        misfit_type="l2", footprints=None, time_weights=None, *, batch=None,
                        ckpt_k=None, tile=None, return_per_shot=False):
    """Waveform misfit (l2 or gcn) and its exact discrete-adjoint gradient in m (FP64).

    ``time_weights`` windows the data per transmit (fwi.py:298-301): the misfit
    compares dsyn*W with dobs*W and the adjoint source is multiplied by W.
    """
    mt = _check_misfit(misfit_type)
    if _no_shots(src_list):
        z = _zeros(np.shape(m), m)
        return (0.0, z, np.zeros(0)) if return_per_shot else (0.0, z)
    plan = _setup(m, geom, h, dt, nt, src_list, footprints, _lib.MODE_GRADIENT, batch, ckpt_k,
                  tile)
    with plan.lock:   # one call at a time per plan: its workspaces are shared
        dev = torch.device("cuda", torch.cuda.current_device())
        md = _to_dev(m, torch.float64, dev)
        wd = _wavelet(wavelet, nt, dev)
        sd = _grid_array(sponge, np.shape(m), "sponge", dev)
        od = _to_dev(dobs, torch.float32, dev)
        if tuple(od.shape) != (plan.n_tx, plan.nt, plan.n_rx):
            raise ValueError(f"dobs has shape {tuple(od.shape)}, expected "
                             f"{(plan.n_tx, plan.nt, plan.n_rx)}")
        tw = _time_weights(time_weights, plan, dev)
        J = torch.zeros(plan.n_tx, dtype=torch.float64, device=dev)
        g = torch.empty(plan.shape, dtype=torch.float64, device=dev)
        mws = plan.workspace("model", plan.model_bytes(), dev)
        bws = plan.workspace(_lib.MODE_GRADIENT, plan.batch_bytes(_lib.MODE_GRADIENT), dev)
        with _on_exec_stream() as st:
            _lib.check(plan._lib.usct_misfit_and_gradient_tw_dev(
                plan.handle, _ptr(md), _ptr(sd), _ptr(wd), _ptr(od), _ptr(tw), mt, _ptr(J), _ptr(g),
                _ptr(mws), _ptr(bws), _stream(st)))
            plan.check(st)
        Jh = J.cpu().numpy()
        Jv = float(np.sum(Jh))
        if return_per_shot:
            return Jv, _out(g, m), Jh
        return Jv, _out(g, m)


def misfit(m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None, misfit_type="l2",
           footprints=None, time_weights=None, *, batch=None, tile=None):
    """Waveform misfit (l2 or gcn) only: one forward sweep per batch (``time_weights``
    as in :func:`misfit_and_gradient`)."""
    mt = _check_misfit(misfit_type)
    if _no_shots(src_list):
        return 0.0
    plan = _setup(m, geom, h, dt, nt, src_list, footprints, _lib.MODE_FORWARD, batch, None, tile)
    with plan.lock:   # one call at a time per plan: its workspaces are shared
        dev = torch.device("cuda", torch.cuda.current_device())
        md = _to_dev(m, torch.float64, dev)
        wd = _wavelet(wavelet, nt, dev)
        sd = _grid_array(sponge, np.shape(m), "sponge", dev)
        od = _to_dev(dobs, torch.float32, dev)
        if tuple(od.shape) != (plan.n_tx, plan.nt, plan.n_rx):
            raise ValueError("dobs shape does not match the acquisition")
        tw = _time_weights(time_weights, plan, dev)
        J = torch.zeros(plan.n_tx, dtype=torch.float64, device=dev)
        mws = plan.workspace("model", plan.model_bytes(), dev)
        bws = plan.workspace(_lib.MODE_FORWARD, plan.batch_bytes(_lib.MODE_FORWARD), dev)
        lib = plan._lib
        with _on_exec_stream() as st:
            s = _stream(st)
            _lib.check(lib.usct_model_prepare(plan.handle, _ptr(mws), _ptr(md), _ptr(sd), None,
                                              _ptr(wd), s))
            for b in range(plan.nbatch):
                _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), b,
                                                  _lib.MODE_FORWARD, None, s))
                _lib.check(lib.usct_batch_misfit_tw(plan.handle, _ptr(bws), b, _ptr(od), _ptr(tw),
                                                    mt, _ptr(J), s))
            plan.check(st)
        return float(np.sum(J.cpu().numpy()))


def gn_hessian_vector(m, geom, wavelet, dt, h, nt, v, sponge=None, src_list=None,
                      footprints=None, wavefields=None, *, batch=None, ckpt_k=None, tile=None,
                      return_born=False):
    """Gauss-Newton product sum_s J_s^T J_s v (exact Born + exact adjoint).

    ``wavefields`` is accepted for signature compatibility and ignored: the
    background is recomputed from checkpoints on the device.
    """
    del wavefields
    if _no_shots(src_list):
        z = _zeros(np.shape(m), m)
        if return_born:
            return z, _zeros((0, int(nt), _n_receivers(geom, np.shape(m), footprints)), m)
        return z
    plan = _setup(m, geom, h, dt, nt, src_list, footprints, _lib.MODE_BORN, batch, ckpt_k, tile)
    with plan.lock:   # one call at a time per plan: its workspaces are shared
        dev = torch.device("cuda", torch.cuda.current_device())
        md = _to_dev(m, torch.float64, dev)
        wd = _wavelet(wavelet, nt, dev)
        sd = _grid_array(sponge, np.shape(m), "sponge", dev)
        vd = _grid_array(v, np.shape(m), "v", dev)
        hv = torch.empty(plan.shape, dtype=torch.float64, device=dev)
        born = torch.empty((plan.n_tx, plan.nt, plan.n_rx), dtype=torch.float32, device=dev) \
            if return_born else None
        mws = plan.workspace("model", plan.model_bytes(), dev)
        bws = plan.workspace(_lib.MODE_BORN, plan.batch_bytes(_lib.MODE_BORN), dev)
        with _on_exec_stream() as st:
            _lib.check(plan._lib.usct_gn_hessian_vector_dev(
                plan.handle, _ptr(md), _ptr(sd), _ptr(wd), _ptr(vd), _ptr(hv), _ptr(born), _ptr(mws),
                _ptr(bws), _stream(st)))
            plan.check(st)
        if return_born:
            return _out(hv, m), _out(born, m)
        return _out(hv, m)


def release():
    """Free every cached plan and workspace (waiting for calls in flight)."""
    with _PLANS_LOCK:
        plans = list(_PLANS.values())
        _PLANS.clear()
    for p in plans:
        with p.lock:
            p.close()
    torch.cuda.empty_cache()


# ---------------------------------------------------------------------------
# the plain one-shot-per-launch GPU form (comparison baseline)
# ---------------------------------------------------------------------------
def plain_forward_fmc(m, geom, wavelet, dt, h, nt, src_list=None):
    plan = _setup(m, geom, h, dt, nt, src_list, None, _lib.MODE_FORWARD, 1, None, None)
    with plan.lock:   # one call at a time per plan: its workspaces are shared
        dev = torch.device("cuda", torch.cuda.current_device())
        md = _to_dev(m, torch.float64, dev)
        wd = _wavelet(wavelet, nt, dev)
        data = torch.empty((plan.n_tx, plan.nt, plan.n_rx), dtype=torch.float32, device=dev)
        ws = _workspace(plan.plain_bytes(False), dev)
        _lib.check(plan._lib.usct_plain_forward_fmc_dev(plan.handle, _ptr(md), _ptr(wd), _ptr(data),
                                                        _ptr(ws), _stream()))
        return _out(data, m)


def plain_misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, src_list=None):
    plan = _setup(m, geom, h, dt, nt, src_list, None, _lib.MODE_FORWARD, 1, None, None)
    with plan.lock:   # one call at a time per plan: its workspaces are shared
        dev = torch.device("cuda", torch.cuda.current_device())
        md = _to_dev(m, torch.float64, dev)
        wd = _wavelet(wavelet, nt, dev)
        od = _to_dev(dobs, torch.float32, dev)
        if tuple(od.shape) != (plan.n_tx, plan.nt, plan.n_rx):
            raise ValueError("dobs shape does not match the acquisition")
        J = torch.zeros(plan.n_tx, dtype=torch.float64, device=dev)
        g = torch.empty(plan.shape, dtype=torch.float64, device=dev)
        ws = _workspace(plan.plain_bytes(True), dev)
        _lib.check(plan._lib.usct_plain_misfit_and_gradient_dev(
            plan.handle, _ptr(md), _ptr(wd), _ptr(od), _ptr(J), _ptr(g), _ptr(ws), _stream()))
        return float(np.sum(J.cpu().numpy())), _out(g, m)
