"""The wave solver as a differentiable PyTorch operator.

``fmc(model, problem)`` maps a model on the grid to full-matrix-capture traces
``(n_tx, nt, n_rx)`` with the batched forward kernels; its backward is the
exact discrete adjoint of the same leapfrog scheme (simulation/ringfwi/fwi.py:
306-331 with the adjoint source replaced by ``grad_output``), run from
checkpoints every k steps with bit-identical segment recompute.  For the L2
loss ``0.5 * ((traces - dobs)**2).sum()`` the model gradient equals
``misfit_and_gradient``'s bit for bit.

Parametrisations: ``"m"`` (squared slowness, the reference's variable) or
``"slowness"`` (s, m = s^2, so dL/ds = 2 s dL/dm).

Checkpoints: the forward keeps every batch's checkpoints on the device when
they fit ``keep_bytes`` (no recompute in backward); otherwise it keeps none
and the backward re-runs each batch's forward sweep before reversing it.
"""

from __future__ import annotations

import torch

from . import _lib
from .backend import (Plan, _on_exec_stream, _ptr, _stream, batch_bytes_estimate, choose_batch,
                      default_ckpt_k)
from .geometry import element_csr


class FMCProblem:
    """Geometry, time axis and engine plan shared by forward and backward."""

    def __init__(self, shape, geom, wavelet, dt, h, nt, src_list=None, footprints=None,
                 sponge=None, batch=None, ckpt_k=None, keep_bytes=None, device=None):
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.shape = tuple(int(s) for s in shape)
        tx, rx = element_csr(geom, self.shape, src_list, footprints)
        free, total = torch.cuda.mem_get_info(self.device)
        if not batch:
            batch = choose_batch(self.shape, nt, tx.rows, rx.rows, len(rx.cell), ckpt_k or 0,
                                 _lib.MODE_GRADIENT, int(0.4 * free))
        keep = int(0.5 * free) if keep_bytes is None else int(keep_bytes)
        if not ckpt_k:
            # the backend's default interval; when every batch's checkpoints can
            # be kept from forward to backward, sized so that they all fit
            nb = -(-tx.rows // batch)
            least = batch_bytes_estimate(self.shape, nt, rx.rows, len(rx.cell), batch, 0,
                                         _lib.MODE_GRADIENT)
            share = keep // nb if keep // nb >= least else None
            ckpt_k = default_ckpt_k(self.shape, nt, rx.rows, len(rx.cell), batch,
                                    _lib.MODE_GRADIENT, budget_bytes=share)
        self.plan = Plan(self.shape, h, dt, nt, tx, rx, batch=batch, ckpt_k=ckpt_k or 0)
        from .backend import _grid_array, _wavelet
        self.wavelet = _wavelet(wavelet, nt, self.device)
        self.sponge = _grid_array(sponge, shape, "sponge", self.device)
        self.keep_bytes = keep
        self.n_tx, self.nt, self.n_rx = self.plan.n_tx, self.plan.nt, self.plan.n_rx


def _bytes(plan):
    return plan.batch_bytes(_lib.MODE_GRADIENT)


class _FMC(torch.autograd.Function):
    @staticmethod
    def forward(ctx, model, problem, param):
        plan = problem.plan
        lib = plan._lib
        dev = problem.device
        x = model.detach().to(device=dev, dtype=torch.float64).contiguous()
        m = x if param == "m" else x * x
        mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
        keep = plan.nbatch * _bytes(plan) <= problem.keep_bytes
        traces = torch.empty((plan.n_tx, plan.nt, plan.n_rx), dtype=torch.float32, device=dev)
        ws = []
        with _on_exec_stream() as st:
            s = _stream(st)
            _lib.check(lib.usct_model_prepare(plan.handle, _ptr(mws), _ptr(m), _ptr(problem.sponge),
                                              None, _ptr(problem.wavelet), s))
            scratch = None
            for b in range(plan.nbatch):
                if keep:
                    w = torch.empty(_bytes(plan), dtype=torch.uint8, device=dev)
                    ws.append(w)
                    mode = _lib.MODE_GRADIENT
                else:
                    if scratch is None:
                        scratch = torch.empty(plan.batch_bytes(_lib.MODE_FORWARD),
                                              dtype=torch.uint8, device=dev)
                    w, mode = scratch, _lib.MODE_FORWARD
                _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(w), b, mode,
                                                  _ptr(traces), s))
            plan.check(st)
        ctx.problem = problem
        ctx.param = param
        ctx.keep = keep
        ctx.ws = ws
        ctx.mws = mws
        ctx.save_for_backward(x)
        return traces

    @staticmethod
    def backward(ctx, grad_traces):
        (x,) = ctx.saved_tensors
        problem = ctx.problem
        plan = problem.plan
        lib = plan._lib
        dev = problem.device
        m = x if ctx.param == "m" else x * x
        adj = grad_traces.detach().to(device=dev, dtype=torch.float32).contiguous()
        g = torch.empty(plan.shape, dtype=torch.float64, device=dev)
        mws = ctx.mws
        with _on_exec_stream() as st:
            s = _stream(st)
            # the accumulator starts at zero (the model is already prepared)
            _lib.check(lib.usct_model_prepare(plan.handle, _ptr(mws), _ptr(m), _ptr(problem.sponge),
                                              None, _ptr(problem.wavelet), s))
            w = None
            for b in range(plan.nbatch):
                if ctx.keep:
                    w = ctx.ws[b]
                else:
                    if w is None:
                        w = torch.empty(_bytes(plan), dtype=torch.uint8, device=dev)
                    _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(w), b,
                                                      _lib.MODE_GRADIENT, None, s))
                _lib.check(lib.usct_batch_adjoint_source(plan.handle, _ptr(w), b, _ptr(adj), s))
                _lib.check(lib.usct_batch_backward(plan.handle, _ptr(mws), _ptr(w), b, s))
            _lib.check(lib.usct_model_gradient(plan.handle, _ptr(mws), _ptr(m), _ptr(g), s))
            plan.check(st)
        ctx.ws = None
        ctx.mws = None
        if ctx.param == "slowness":
            g = 2.0 * x * g
        return g.to(grad_traces.device), None, None


def fmc(model, problem, param="m"):
    """Differentiable FMC forward: ``model`` (CUDA tensor, grid-shaped) -> traces."""
    if param not in ("m", "slowness"):
        raise ValueError("param must be 'm' or 'slowness'")
    if tuple(model.shape) != problem.shape:
        raise ValueError(f"model shape {tuple(model.shape)} != problem shape {problem.shape}")
    return _FMC.apply(model, problem, param)
