"""Shot sharding across GPUs, one process per GPU.

Shots are independent and the misfit and its gradient are sums over shots
(simulation/ringfwi/fwi.py:294-331), so a multi-GPU ``misfit_and_gradient``
gives each rank a contiguous block of the transmits, runs the batched engine
on it, and sums (J, g) across ranks once -- the only exchange on the path.
(The benchmark runs independent replicas and needs no exchange at all.)
"""

from __future__ import annotations

import numpy as np


def shard(n_items, rank, world):
    """Contiguous block of item indices owned by ``rank`` (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(n_items), int(world))
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def misfit_and_gradient(m, geom, wavelet, dt, h, nt, dobs, sponge=None, src_list=None,
                        misfit_type="l2", footprints=None, time_weights=None, *, group=None,
                        compute=None, **kw):
    """Sharded L2/GCN misfit and gradient; every rank returns the full (J, g).

    ``compute`` defaults to :func:`openusct_gb300.backend.misfit_and_gradient`.
    ``time_weights`` (one window per transmit) is split with the transmits.
    """
    import torch
    import torch.distributed as dist
    if compute is None:
        from .backend import misfit_and_gradient as compute
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    shots = list(range(len(geom.idx))) if src_list is None else [int(s) for s in src_list]
    mine = shard(len(shots), rank, world)
    shape = tuple(np.shape(m))
    if mine:
        if time_weights is not None:
            kw["time_weights"] = [time_weights[i] for i in mine]
        J, g = compute(m, geom, wavelet, dt, h, nt, np.asarray(dobs)[mine], sponge,
                       [shots[i] for i in mine], misfit_type=misfit_type, footprints=footprints,
                       **kw)
    else:
        J, g = 0.0, np.zeros(shape)
    if world == 1:
        return float(J), np.asarray(g)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else "cpu"
    buf = torch.empty(int(np.prod(shape)) + 1, dtype=torch.float64, device=dev)
    buf[:-1] = torch.as_tensor(np.asarray(g, np.float64).reshape(-1), device=dev)
    buf[-1] = float(J)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    out = buf.cpu().numpy()
    return float(out[-1]), out[:-1].reshape(shape)
