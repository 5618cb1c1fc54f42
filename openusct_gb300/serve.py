"""Continuous-batching service for forward, gradient and Gauss-Newton FMC requests.

Requests of different grids, element counts and kinds (forward-only, L2/GCN
gradient, or a Gauss-Newton inversion of ``n_iter`` outer iterations served as
one long-lived request) arrive over time.  The scheduler admits a request as soon as a slot
is free and its device footprint (model + batch workspaces + its data, from
the engine's own size queries) fits the HBM budget; requests that do not fit
wait while later, smaller ones may go ahead; a request larger than the whole
budget is rejected at once.  Each admitted request gets its own plan, its own
workspaces and its own CUDA stream, so the batch sweeps of co-admitted
requests overlap on the device; the request's shots advance C at a time in one
launch per time step.  Wavefields and checkpoints stay on the device; only the
request's inputs and its result cross PCIe/C2C.

A Gauss-Newton request runs the device-resident ``invert(optimizer=
"gauss-newton")`` (fwi.py:434-532) on its own plan, workspace and stream: the
model, the observed data and every wavefield stay on the device across its
iterations, and only scalars (misfits, CG dot products) reach the host until
the final model.

Forward requests that share grid, spacing, time axis and wavelet (and have
no sponge or footprints) are put in shared launches when more of them wait
than there are free slots (``GpuExecutor(merge=False)`` turns this off): when one is
admitted, compatible requests already waiting join it (up to a batch of
shots), and the group runs on one plan whose shot channels each carry their
own model (``usct_plan_set_channel_models``).  Every request of a group gets
exactly the traces it would get alone.

Latency is measured from a request's arrival to its result being on the host;
``Stats`` gives p50/p99 and shots/s.  The scheduling logic is independent of
the executor (``GpuExecutor`` here), so it is tested on the CPU with a fake.
"""

from __future__ import annotations

import heapq
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib


@dataclass
class Request:
    kind: str                      # "forward" | "gradient" | "gauss-newton"
    m: np.ndarray                  # squared slowness on the grid
    geom: object                   # .idx of grid-index tuples
    wavelet: np.ndarray
    dt: float
    h: float
    nt: int
    dobs: np.ndarray | None = None
    src_list: list | None = None
    footprints: list | None = None
    sponge: np.ndarray | None = None
    misfit_type: str = "l2"        # gradient requests: "l2" or "gcn"
    time_weights: object = None    # gradient requests: one (nt, n_rx) window per transmit
    n_iter: int = 4                # gauss-newton requests: outer iterations
    n_cg: int = 8                  # gauss-newton requests: CG steps per iteration
    update_mask: np.ndarray | None = None   # gauss-newton requests
    m_bounds: tuple | None = None           # gauss-newton requests
    arrival: float = 0.0           # seconds after the stream starts
    rid: int = -1
    batch: int | None = None
    cancelled: threading.Event = field(default_factory=threading.Event, repr=False)

    @property
    def n_shots(self):
        return len(self.src_list) if self.src_list is not None else len(self.geom.idx)

    def cancel(self):
        """Withdraw the request: if it is still queued it is never admitted;
        if it is running it stops at the next shot-batch boundary (the device
        finishes the batch in flight) and its slot and budget are released."""
        self.cancelled.set()


class Cancelled(Exception):
    """Raised by an executor that stopped a request because it was cancelled."""


@dataclass
class Result:
    rid: int
    kind: str
    ok: bool
    error: str | None = None
    traces: np.ndarray | None = None
    J: float | None = None
    g: np.ndarray | None = None
    m: np.ndarray | None = None          # gauss-newton: the final model
    history: list | None = None          # gauss-newton: the misfit history
    shots: int = 0
    footprint: int = 0
    t_arrival: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    waited_for_budget: bool = False      # a slot was free but its footprint did not fit
    group: int = 1                       # requests that shared its launches

    @property
    def latency(self):
        return self.t_done - self.t_arrival

    def record(self):
        """The per-request JSON record (times in seconds from the stream start)."""
        return {"rid": self.rid, "kind": self.kind, "ok": self.ok, "error": self.error,
                "shots": self.shots, "device_bytes": self.footprint,
                "t_arrival": self.t_arrival, "t_admit": self.t_admit, "t_done": self.t_done,
                "queue_s": max(0.0, self.t_admit - self.t_arrival),
                "waited_for_budget": self.waited_for_budget, "group": self.group,
                "latency_s": self.latency if self.ok else None}


@dataclass
class Stats:
    n: int
    ok: int
    rejected: int
    p50_s: float
    p99_s: float
    mean_s: float
    makespan_s: float
    shots: int
    shots_per_s: float
    max_concurrent: int
    peak_reserved_bytes: int
    waited_for_budget: int = 0
    merged: int = 0                      # requests served in a shared launch group

    def as_dict(self):
        return dict(self.__dict__)


def percentile(xs, q):
    if not xs:
        return float("nan")
    xs = sorted(xs)
    k = (len(xs) - 1) * q / 100.0
    lo, hi = int(np.floor(k)), int(np.ceil(k))
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


_MODES = {"forward": _lib.MODE_FORWARD, "gradient": _lib.MODE_GRADIENT,
          "gauss-newton": _lib.MODE_BORN}


class _PlanBackend:
    """The backend protocol of ``invert`` (misfit, misfit_and_gradient,
    gn_hessian_vector on CUDA tensors) bound to one request's plan, model and
    batch workspaces (the batch workspace sized for the Born mode, of which the
    gradient and forward layouts are prefixes), its wavelet, sponge and
    observed data on the device, and its stream."""

    def __init__(self, plan, mws, bws, wavelet, sponge, dobs, stream):
        from .backend import _ptr, _stream
        self.plan, self.P = plan, _ptr
        self.mws, self.bws, self.w, self.sp, self.dobs = mws, bws, wavelet, sponge, dobs
        self.stream, self.s = stream, _stream(stream)
        self.lib = plan._lib

    def _J(self):
        import torch
        return torch.zeros(self.plan.n_tx, dtype=torch.float64, device=self.dobs.device)

    def misfit(self, m, *args, **kw):
        P, p, J = self.P, self.plan, self._J()
        _lib.check(self.lib.usct_model_prepare(p.handle, P(self.mws), P(m), P(self.sp), None,
                                               P(self.w), self.s))
        for b in range(p.nbatch):
            _lib.check(self.lib.usct_batch_forward(p.handle, P(self.mws), P(self.bws), b,
                                                   _lib.MODE_FORWARD, None, self.s))
            _lib.check(self.lib.usct_batch_misfit_tw(p.handle, P(self.bws), b, P(self.dobs),
                                                     None, 0, P(J), self.s))
        p.check(self.stream)
        return float(J.sum().item())

    def misfit_and_gradient(self, m, *args, **kw):
        import torch
        P, p, J = self.P, self.plan, self._J()
        g = torch.empty(p.shape, dtype=torch.float64, device=m.device)
        _lib.check(self.lib.usct_misfit_and_gradient_dev(
            p.handle, P(m), P(self.sp), P(self.w), P(self.dobs), P(J), P(g), P(self.mws),
            P(self.bws), self.s))
        p.check(self.stream)
        return float(J.sum().item()), g

    def gn_hessian_vector(self, m, geom, wavelet, dt, h, nt, v, *args, **kw):
        import torch
        P, p = self.P, self.plan
        hv = torch.empty(p.shape, dtype=torch.float64, device=m.device)
        _lib.check(self.lib.usct_gn_hessian_vector_dev(
            p.handle, P(m), P(self.sp), P(self.w), P(v.contiguous()), P(hv), None, P(self.mws),
            P(self.bws), self.s))
        p.check(self.stream)
        return hv


def _concat_csr(parts):
    """Rows of several element CSR lists, one after the other."""
    from .geometry import CSR
    ptr = [0]
    for c in parts:
        base = ptr[-1]
        ptr.extend(int(v) + base for v in c.ptr[1:])
    return CSR(np.asarray(ptr, np.int32), np.concatenate([c.cell for c in parts]),
               np.concatenate([c.w for c in parts]))


def _pad_rows(c, quantum):
    """``c`` with empty rows (no entries) appended up to a multiple of
    ``quantum`` rows: transmits that inject nothing, so their fields stay 0."""
    from .geometry import CSR
    extra = -c.rows % quantum
    if not extra:
        return c
    ptr = np.concatenate([np.asarray(c.ptr, np.int32), np.full(extra, c.ptr[-1], np.int32)])
    return CSR(ptr, c.cell, c.w)


def _union_rows(parts):
    """One CSR holding each distinct row of several element CSR lists once (a
    row is its cells and weights), and per list the union row of each of its
    rows: requests on the same elements share their receivers' traces."""
    from .geometry import CSR
    where, ptr, cells, ws, idx = {}, [0], [], [], []
    for c in parts:
        rows = []
        for j in range(c.rows):
            a, b = int(c.ptr[j]), int(c.ptr[j + 1])
            cj, wj = np.asarray(c.cell[a:b]), np.asarray(c.w[a:b])
            key = (cj.tobytes(), wj.tobytes())
            if key not in where:
                where[key] = len(ptr) - 1
                ptr.append(ptr[-1] + (b - a))
                cells.append(cj)
                ws.append(wj)
            rows.append(where[key])
        idx.append(np.asarray(rows, np.int64))
    cell = np.concatenate(cells) if cells else np.zeros(0, parts[0].cell.dtype)
    w = np.concatenate(ws) if ws else np.zeros(0, parts[0].w.dtype)
    return CSR(np.asarray(ptr, np.int32), cell, w), idx


class GpuExecutor:
    """Runs one request on the GB300 engine on its own stream."""

    merge_width = 32   # shots of one launch group (a batch)
    merge_quantum = 4  # a request's shots fill whole groups of four channels (one model each)

    def __init__(self, device=None, graphs=False, workspace_bytes=None, merge=True):
        import torch
        self.torch = torch
        # compatible forward requests may share launches when they outnumber
        # the free slots (one launch stream instead of several, each launch
        # over up to a batch of shots)
        self.merge = merge
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.graphs = graphs
        # the batch workspace one request may size its checkpoint interval for
        # (default an eighth of the device, so several requests run at once)
        self.workspace_bytes = (int(workspace_bytes) if workspace_bytes else
                                torch.cuda.get_device_properties(self.device).total_memory // 8)

    def plan_for(self, req):
        from .backend import Plan, choose_batch, default_ckpt_k
        from .geometry import element_csr
        shape = tuple(req.m.shape)
        if req.kind not in _MODES:
            raise ValueError(f"unknown request kind {req.kind!r}")
        tx, rx = element_csr(req.geom, shape, req.src_list, req.footprints)
        mode = _MODES[req.kind]
        # the widest batch (<= 32 shots) whose least-memory workspace fits
        # this request's workspace share
        C = req.batch or min(32, choose_batch(shape, req.nt, tx.rows, rx.rows, len(rx.cell), 0,
                                              mode, self.workspace_bytes))
        # the backend's default interval within this request's workspace share
        # (one segment when its stash fits); the footprint used for admission
        # is this plan's workspace
        k = default_ckpt_k(shape, req.nt, rx.rows, len(rx.cell), C, mode,
                           budget_bytes=self.workspace_bytes)
        plan = Plan(shape, req.h, req.dt, req.nt, tx, rx, batch=C, ckpt_k=k)
        if not self.graphs:
            plan.set("graphs", 0)
        return plan

    def footprint(self, req, plan):
        mode = _MODES[req.kind]
        data = 4 * plan.n_tx * plan.nt * plan.n_rx
        cells = int(np.prod(plan.shape))
        # model-sized FP64 arrays beside the workspaces: the model and gradient;
        # a Gauss-Newton request's loop holds 13 more (CG vectors, trial model,
        # mask, bounds)
        models = 2 if req.kind != "gauss-newton" else 15
        return plan.model_bytes() + plan.batch_bytes(mode) + data + 8 * models * cells + (1 << 20)

    def run(self, req, plan):
        torch = self.torch
        from .backend import (_check_misfit, _grid_array, _ptr, _stream, _time_weights,
                              _to_dev, _wavelet)
        lib = plan._lib
        dev = self.device
        st = torch.cuda.Stream(device=dev)
        with torch.cuda.stream(st):
            m = torch.from_numpy(np.ascontiguousarray(req.m, np.float64)).to(dev, non_blocking=True)
            w = _wavelet(req.wavelet, req.nt, dev)
            sp = _grid_array(req.sponge, np.shape(req.m), "sponge", dev)
            mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
            s = _stream(st)
            # shot batches in order, one queued on the device behind the one
            # running (so the device never waits for the host to enqueue the
            # next), the request's cancellation checked between them; the same
            # calls in the same order as the whole-acquisition entry points, so
            # results are identical
            def batches():
                prev = None
                for b in range(plan.nbatch):
                    if req.cancelled.is_set():
                        raise Cancelled(f"cancelled after {b} of {plan.nbatch} shot batches")
                    yield b
                    ev = torch.cuda.Event()
                    ev.record(st)
                    if prev is not None:
                        prev.synchronize()
                    prev = ev

            if req.kind == "gauss-newton":
                return self._gauss_newton(req, plan, m, w, sp, mws, st)
            if req.kind == "forward":
                bws = torch.empty(plan.batch_bytes(_lib.MODE_FORWARD), dtype=torch.uint8, device=dev)
                data = torch.empty((plan.n_tx, plan.nt, plan.n_rx), dtype=torch.float32, device=dev)
                _lib.check(lib.usct_model_prepare(plan.handle, _ptr(mws), _ptr(m), _ptr(sp), None,
                                                  _ptr(w), s))
                for b in batches():
                    _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), b,
                                                      _lib.MODE_FORWARD, _ptr(data), s))
                plan.check(st)
                return {"traces": data.cpu().numpy()}
            if req.dobs is None or np.shape(req.dobs) != (plan.n_tx, plan.nt, plan.n_rx):
                raise ValueError(f"dobs must have shape {(plan.n_tx, plan.nt, plan.n_rx)}")
            mt = _check_misfit(req.misfit_type)
            tw = _time_weights(req.time_weights, plan, dev)
            dobs = _to_dev(req.dobs, torch.float32, dev)
            bws = torch.empty(plan.batch_bytes(_lib.MODE_GRADIENT), dtype=torch.uint8, device=dev)
            J = torch.zeros(plan.n_tx, dtype=torch.float64, device=dev)
            g = torch.empty(plan.shape, dtype=torch.float64, device=dev)
            _lib.check(lib.usct_model_prepare(plan.handle, _ptr(mws), _ptr(m), _ptr(sp), None,
                                              _ptr(w), s))
            for b in batches():
                _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), b,
                                                  _lib.MODE_GRADIENT, None, s))
                _lib.check(lib.usct_batch_misfit_tw(plan.handle, _ptr(bws), b, _ptr(dobs), _ptr(tw),
                                                    mt, _ptr(J), s))
                _lib.check(lib.usct_batch_backward(plan.handle, _ptr(mws), _ptr(bws), b, s))
            _lib.check(lib.usct_model_gradient(plan.handle, _ptr(mws), _ptr(m), _ptr(g), s))
            plan.check(st)
            return {"J": float(J.sum().item()), "g": g.cpu().numpy()}

    # -- forward requests sharing launches --------------------------------------
    def merge_key(self, req):
        """Requests with equal keys can share a plan with per-channel models:
        forward requests of the same grid, spacing, time axis and wavelet,
        without sponge or footprints; None for any other request."""
        if not self.merge or req.kind != "forward" or req.sponge is not None \
                or req.footprints is not None or req.batch is not None:
            return None
        w = np.ascontiguousarray(req.wavelet, np.float64)[: req.nt]
        return (tuple(np.shape(req.m)), float(req.h), float(req.dt), int(req.nt), w.tobytes())

    def plan_for_group(self, reqs):
        """One plan for the transmits of all ``reqs`` (in order) and the union of
        their receivers (each distinct receiver once); transmit t uses the model
        of the request it came from."""
        from .backend import Plan
        from .geometry import element_csr
        shape = tuple(np.shape(reqs[0].m))
        parts = [element_csr(q.geom, shape, q.src_list, None) for q in reqs]
        padded = [_pad_rows(t, self.merge_quantum) for t, _ in parts]
        tx = _concat_csr(padded)
        rx, rx_of = _union_rows([r for _, r in parts])
        C = self.merge_width
        q0 = reqs[0]
        plan = Plan(shape, q0.h, q0.dt, q0.nt, tx, rx, batch=C)
        owner = np.concatenate([np.full(t.rows, i, np.int32) for i, t in enumerate(padded)])
        _lib.check(plan._lib.usct_plan_set_channel_models(
            plan.handle, len(reqs), owner.ctypes.data_as(_lib._ip)))
        if not self.graphs:
            plan.set("graphs", 0)
        # (first transmit, transmits, receiver columns) of each request
        starts = np.cumsum([0] + [t.rows for t in padded[:-1]])
        plan.group_parts = [(int(s), t.rows, ix) for s, (t, _), ix in zip(starts, parts, rx_of)]
        return plan

    def footprint_group(self, reqs, plan):
        data = 4 * plan.n_tx * plan.nt * plan.n_rx
        cells = int(np.prod(plan.shape))
        return (plan.model_bytes() + plan.batch_bytes(_lib.MODE_FORWARD) + data +
                8 * len(reqs) * cells + (1 << 20))

    def run_group(self, reqs, plan):
        """The forward sweeps of every request of the group in shared launches;
        returns each request's traces (its transmits x its receivers)."""
        torch = self.torch
        from .backend import _ptr, _stream, _wavelet
        lib = plan._lib
        dev = self.device
        st = torch.cuda.Stream(device=dev)
        with torch.cuda.stream(st):
            models = torch.stack([torch.from_numpy(np.ascontiguousarray(q.m, np.float64))
                                  for q in reqs]).to(dev)
            w = _wavelet(reqs[0].wavelet, reqs[0].nt, dev)
            mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
            bws = torch.empty(plan.batch_bytes(_lib.MODE_FORWARD), dtype=torch.uint8, device=dev)
            data = torch.empty((plan.n_tx, plan.nt, plan.n_rx), dtype=torch.float32, device=dev)
            s = _stream(st)
            _lib.check(lib.usct_model_prepare_channels(plan.handle, _ptr(mws), _ptr(models),
                                                       _ptr(w), s))
            for b in range(plan.nbatch):
                if any(q.cancelled.is_set() for q in reqs):
                    raise Cancelled(f"cancelled after {b} of {plan.nbatch} shot batches")
                _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), b,
                                                  _lib.MODE_FORWARD, _ptr(data), s))
            plan.check(st)
            host = data.cpu().numpy()
        return [{"traces": np.ascontiguousarray(host[t0:t0 + n][:, :, ix])}
                for t0, n, ix in plan.group_parts]

    def _gauss_newton(self, req, plan, m, w, sp, mws, st):
        """``n_iter`` Gauss-Newton iterations of the device-resident invert on
        this request's plan; cancellation is checked between iterations."""
        torch = self.torch
        from .backend import _to_dev
        from .invert import invert
        if req.dobs is None or np.shape(req.dobs) != (plan.n_tx, plan.nt, plan.n_rx):
            raise ValueError(f"dobs must have shape {(plan.n_tx, plan.nt, plan.n_rx)}")
        dobs = _to_dev(req.dobs, torch.float32, self.device)
        bws = torch.empty(plan.batch_bytes(_lib.MODE_BORN), dtype=torch.uint8, device=self.device)
        be = _PlanBackend(plan, mws, bws, w, sp, dobs, st)

        def progress(done, total):
            if req.cancelled.is_set():
                raise Cancelled(f"cancelled after {done} of {total} Gauss-Newton iterations")

        m_out, hist = invert(m, req.geom, req.wavelet, req.dt, req.h, req.nt, dobs,
                             src_list=req.src_list, n_iter=req.n_iter, optimizer="gauss-newton",
                             n_cg=req.n_cg, update_mask=req.update_mask, m_bounds=req.m_bounds,
                             backend=be, progress=progress, footprints=req.footprints)
        plan.check(st)
        return {"m": m_out.cpu().numpy(), "history": [float(v) for v in hist],
                "J": float(hist[-1])}

    def release(self, plan):
        plan.close()


class Engine:
    """Admission, slots and completion bookkeeping around an executor."""

    def __init__(self, executor, budget_bytes, max_active=4):
        self.ex = executor
        self.budget = int(budget_bytes)
        self.max_active = int(max_active)
        self.lock = threading.Condition()
        self._merge_keys = {}   # request index -> merge key (one run_stream)
        self.reserved = 0
        self.active = 0
        self.peak_reserved = 0
        self.max_concurrent = 0

    # -- one request ------------------------------------------------------------
    def _worker(self, req, plan, fp, res, t0, on_done):
        try:
            if req.cancelled.is_set():
                raise Cancelled("cancelled before it started")
            out = self.ex.run(req, plan)
            res.ok = True
            res.traces = out.get("traces")
            res.J = out.get("J")
            res.g = out.get("g")
            res.m = out.get("m")
            res.history = out.get("history")
        except Exception as exc:   # the request fails, the service goes on
            res.ok = False
            res.error = f"{type(exc).__name__}: {exc}"[:300]
        finally:
            try:
                self.ex.release(plan)
            except Exception:
                pass
            res.t_done = time.perf_counter() - t0
            with self.lock:
                self.reserved -= fp
                self.active -= 1
                self.lock.notify_all()
            on_done(res)

    def _worker_group(self, members, plan, fp, t0, on_done):
        """Requests sharing one plan with per-channel models."""
        reqs = [m[1] for m in members]
        results = [m[2] for m in members]
        try:
            outs = self.ex.run_group(reqs, plan)
            for res, out in zip(results, outs):
                res.ok = True
                res.traces = out.get("traces")
        except Exception as exc:
            for res in results:
                res.ok = False
                res.error = f"{type(exc).__name__}: {exc}"[:300]
        finally:
            try:
                self.ex.release(plan)
            except Exception:
                pass
            t = time.perf_counter() - t0
            for res in results:
                res.t_done = t
                res.group = len(members)
            with self.lock:
                self.reserved -= fp
                self.active -= 1
                self.lock.notify_all()
            for res in results:
                on_done(res)

    def _group_for(self, head, others, results):
        """Waiting requests that share ``head``'s launches, as (index, request)
        pairs starting with head; None for none.  Separate plans on their own
        streams overlap on the device while slots are free, and a shared
        launch reads the model once per shot, so requests are grouped only
        when more compatible ones wait than there are free slots:
        ceil(waiting / free) requests per group, in arrival order, their shots
        up to one batch."""
        key_of = getattr(self.ex, "merge_key", None)
        if key_of is None:
            return None
        keys = self._merge_keys          # each request's key, computed once

        def key_for(j, q):
            if j not in keys:
                keys[j] = key_of(q)
            return keys[j]

        i, rq = head
        width = getattr(self.ex, "merge_width", 32)
        quantum = getattr(self.ex, "merge_quantum", 1)

        def shots_of(q):   # channels a request takes in a group
            return -(-q.n_shots // quantum) * quantum

        key = key_for(i, rq)
        if key is None or shots_of(rq) >= width:
            return None
        cands = [it for it in sorted(others, key=lambda it: (it[0], it[1]))
                 if not it[2].cancelled.is_set() and key_for(it[1], it[2]) == key]
        free = max(1, self.max_active - self.active)
        size = -(-(len(cands) + 1) // free)
        if size < 2:
            return None
        group, shots = [head], shots_of(rq)
        for item in cands:
            if len(group) == size:
                break
            j, oq = item[1], item[2]
            if shots + shots_of(oq) > width:
                continue
            group.append((j, oq))
            shots += shots_of(oq)
        return group if len(group) > 1 else None

    # -- a whole stream ----------------------------------------------------------
    def run_stream(self, requests, realtime=True):
        """Replay ``requests`` (sorted by arrival) and return their Results in
        request order.  With ``realtime`` the arrival times are honoured."""
        reqs = sorted(enumerate(requests), key=lambda kv: kv[1].arrival)
        results = [None] * len(requests)
        self._merge_keys = {}
        pending = []          # (arrival, order, req, plan, fp)
        threads = []
        t0 = time.perf_counter()
        done_count = [0]

        def on_done(r):
            with self.lock:
                done_count[0] += 1
                self.lock.notify_all()

        nxt = 0
        while True:
            now = time.perf_counter() - t0
            # arrivals
            while nxt < len(reqs) and (not realtime or reqs[nxt][1].arrival <= now):
                i, rq = reqs[nxt]
                rq.rid = i
                res = Result(rid=i, kind=rq.kind, ok=False, shots=rq.n_shots,
                             t_arrival=rq.arrival if realtime else now)
                results[i] = res
                try:
                    plan = self.ex.plan_for(rq)
                    fp = int(self.ex.footprint(rq, plan))
                except Exception as exc:
                    res.error = f"{type(exc).__name__}: {exc}"[:300]
                    res.t_done = res.t_admit = now
                    with self.lock:
                        done_count[0] += 1
                    nxt += 1
                    continue
                res.footprint = fp
                if fp > self.budget:
                    res.error = (f"rejected: needs {fp} bytes of device memory, the budget is "
                                 f"{self.budget}")
                    res.t_done = res.t_admit = now
                    self.ex.release(plan)
                    with self.lock:
                        done_count[0] += 1
                else:
                    heapq.heappush(pending, (res.t_arrival, i, rq, plan, fp))
                nxt += 1
            # admissions: first come first served, later ones may pass a head that
            # does not fit yet
            drop = []            # plans to free once the lock is released
            with self.lock:
                keep = []
                while pending:
                    item = heapq.heappop(pending)
                    _, i, rq, plan, fp = item
                    if rq.cancelled.is_set():          # withdrawn while queued
                        res = results[i]
                        res.error = "Cancelled: withdrawn before admission"
                        res.t_done = res.t_admit = time.perf_counter() - t0
                        drop.append(plan)
                        done_count[0] += 1
                        continue
                    group = None
                    if self.active < self.max_active:
                        group = self._group_for((i, rq), pending + keep, results)
                    if group:
                        gplan, gfp = None, 0
                        try:
                            gplan = self.ex.plan_for_group([q for _, q in group])
                            gfp = int(self.ex.footprint_group([q for _, q in group], gplan))
                        except Exception:
                            if gplan is not None:
                                drop.append(gplan)
                            gplan = None
                        if gplan is not None and self.reserved + gfp <= self.budget:
                            taken = {j for j, _ in group}
                            for it in pending + keep:
                                if it[1] in taken:
                                    drop.append(it[3])
                            drop.append(plan)
                            pending[:] = [it for it in pending if it[1] not in taken]
                            heapq.heapify(pending)
                            keep = [it for it in keep if it[1] not in taken]
                            self.reserved += gfp
                            self.active += 1
                            self.peak_reserved = max(self.peak_reserved, self.reserved)
                            self.max_concurrent = max(self.max_concurrent, self.active)
                            now_a = time.perf_counter() - t0
                            members = []
                            for j, q in group:
                                results[j].t_admit = now_a
                                members.append((j, q, results[j]))
                            th = threading.Thread(target=self._worker_group,
                                                  args=(members, gplan, gfp, t0, on_done),
                                                  daemon=True)
                            threads.append(th)
                            th.start()
                            continue
                        if gplan is not None:
                            drop.append(gplan)
                    if self.active < self.max_active and self.reserved + fp <= self.budget:
                        self.reserved += fp
                        self.active += 1
                        self.peak_reserved = max(self.peak_reserved, self.reserved)
                        self.max_concurrent = max(self.max_concurrent, self.active)
                        res = results[i]
                        res.t_admit = time.perf_counter() - t0
                        th = threading.Thread(target=self._worker,
                                              args=(rq, plan, fp, res, t0, on_done), daemon=True)
                        threads.append(th)
                        th.start()
                    else:
                        if self.active < self.max_active:   # held back by the budget
                            results[i].waited_for_budget = True
                        keep.append(item)
                for item in keep:
                    heapq.heappush(pending, item)
                finished = done_count[0] == len(reqs)
                if not finished and not drop:
                    wait = None
                    if nxt < len(reqs) and realtime:
                        wait = max(0.0, reqs[nxt][1].arrival - (time.perf_counter() - t0))
                    self.lock.wait(timeout=wait if wait is not None else 0.05)
            # freeing device memory waits for the device: never under the lock,
            # so admission does not stall behind running sweeps
            for pl in drop:
                try:
                    self.ex.release(pl)
                except Exception:      # a plan that fails to close must not stop admission
                    pass
            if finished:
                break
        for th in threads:
            th.join()
        return results


def write_records(results, path):
    """One JSON line per request (Result.record) -- the service's log."""
    import json
    with open(path, "w") as f:
        for r in results:
            f.write(json.dumps(r.record()) + "\n")


def summarize(results, engine=None):
    ok = [r for r in results if r.ok]
    lat = [r.latency for r in ok]
    t_first = min((r.t_arrival for r in results), default=0.0)
    t_last = max((r.t_done for r in ok), default=0.0)
    span = max(t_last - t_first, 1e-9)
    shots = sum(r.shots for r in ok)
    return Stats(n=len(results), ok=len(ok),
                 rejected=sum(1 for r in results if not r.ok and r.error and
                              r.error.startswith("rejected")),
                 p50_s=percentile(lat, 50), p99_s=percentile(lat, 99),
                 mean_s=float(np.mean(lat)) if lat else float("nan"), makespan_s=span,
                 shots=shots, shots_per_s=shots / span,
                 max_concurrent=engine.max_concurrent if engine else 0,
                 peak_reserved_bytes=engine.peak_reserved if engine else 0,
                 waited_for_budget=sum(1 for r in results if r.waited_for_budget),
                 merged=sum(1 for r in results if r.ok and r.group > 1))


# ---------------------------------------------------------------------------
# seeded request streams with the serving configuration's mix
# ---------------------------------------------------------------------------
def make_stream(n_requests, rate_hz, seed=0, sizes_2d=(128, 1024), sizes_3d=(96, 256),
                elements_2d=(32, 256), elements_3d=(64, 512), frac_3d=0.5, frac_gradient=0.3,
                nt_cap=None, dobs_fn=None):
    """Poisson arrivals at ``rate_hz``; each request a 2D ring or 3D cylinder
    problem (disc or random-field model), forward-only or gradient (then
    ``dobs_fn(true_problem)`` supplies the observed data).  nt follows the
    builder's rule t_end = 2.2 * 2R / 1450 with R = 0.8 x half the domain."""
    from . import problems
    from .geometry import CylinderGeometry, RingGeometry, ricker
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        is3d = rng.uniform() < frac_3d
        kind = "gradient" if rng.uniform() < frac_gradient else "forward"
        if is3d:
            n = int(rng.integers(sizes_3d[0] // 8, sizes_3d[1] // 8 + 1)) * 8
            h = 0.2e-3
            ne = int(rng.integers(elements_3d[0] // 8, elements_3d[1] // 8 + 1)) * 8
            rings = 2 if ne < 128 else 4
            R = 0.8 * (n - 1) * h / 2
            geom = CylinderGeometry(rings, ne // rings, R, 0.5 * (n - 1) * h, (n - 1) * h, h)
            shape = (n, n, n)
        else:
            n = int(rng.integers(sizes_2d[0] // 16, sizes_2d[1] // 16 + 1)) * 16
            h = 0.15e-3
            ne = int(rng.integers(elements_2d[0] // 8, elements_2d[1] // 8 + 1)) * 8
            R = 0.8 * (n - 1) * h / 2
            geom = RingGeometry(ne, R, (n - 1) * h, h)
            shape = (n, n)
        if rng.uniform() < 0.5:
            f = problems.random_field(shape, 0.002 / h, 0.03, rng)
            c = 1500.0 * (1.0 + f)
        else:
            c = np.full(shape, 1500.0)
            centre = (n - 1) * h / 2
            grids = np.meshgrid(*[np.arange(s) * h for s in shape], indexing="ij")
            for rad, cv in ((0.25 * R, 1450.0), (0.35 * R, 1580.0)):
                off = rng.uniform(-0.3 * R, 0.3 * R, size=len(shape))
                r2 = sum((gx - centre - o) ** 2 for gx, o in zip(grids, off))
                c[r2 <= rad * rad] = cv
        dt = 0.3 * h / float(c.max())
        nt = int(np.ceil(2.2 * 2 * R / 1450.0 / dt))
        if nt_cap:
            nt = min(nt, nt_cap)
        wav = ricker(nt, dt, 1e6)
        m_true = 1.0 / c ** 2
        req = Request(kind=kind, m=m_true, geom=geom, wavelet=wav, dt=dt, h=h, nt=nt,
                      arrival=t)
        if kind == "gradient":
            req.m = np.full(shape, 1.0 / 1500.0 ** 2)
            req.dobs = dobs_fn(m_true, geom, wav, dt, h, nt) if dobs_fn else None
        out.append(req)
    return out
