"""The sharded gradient sum, world size 2 over gloo on the CPU."""

import os

import numpy as np
import pytest

from openusct_gb300.shard import shard


def test_shard_partitions_every_item_once():
    for n in (0, 1, 7, 64, 257):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard(n, r, world)]
            assert got == list(range(n))
            sizes = [len(shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1


def _fake_compute(m, geom, wavelet, dt, h, nt, dobs, sponge, src_list, misfit_type="l2",
                  footprints=None, time_weights=None):
    # per-shot contributions that are easy to sum serially
    g = np.zeros(np.shape(m))
    J = 0.0
    tws = [None] * len(dobs) if time_weights is None else list(time_weights)
    assert len(tws) == len(dobs)
    for s, d, w in zip(src_list, dobs, tws):
        g += (s + 1) * np.arange(g.size, dtype=float).reshape(g.shape) + float(d.sum())
        J += 0.5 * (s + 1) ** 2
        if w is not None:   # the window must travel with its own transmit
            J += float(np.sum(w * d))
    return J, g


class _Geom:
    idx = [(i, i) for i in range(5)]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from openusct_gb300 import shard as sh
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = np.ones((3, 4))
    dobs = np.arange(5 * 2 * 5, dtype=float).reshape(5, 2, 5)
    J, g = sh.misfit_and_gradient(m, _Geom(), None, 1.0, 1.0, 2, dobs, compute=_fake_compute)
    tw = [np.full((2, 5), 0.1 * (i + 1)) for i in range(5)]
    Jw, _ = sh.misfit_and_gradient(m, _Geom(), None, 1.0, 1.0, 2, dobs, time_weights=tw,
                                   compute=_fake_compute)
    out.put((rank, J, g, Jw))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_sum_equals_serial_on_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    dobs = np.arange(5 * 2 * 5, dtype=float).reshape(5, 2, 5)
    J0, g0 = _fake_compute(np.ones((3, 4)), _Geom(), None, 1.0, 1.0, 2, dobs, None, range(5))
    tw = [np.full((2, 5), 0.1 * (i + 1)) for i in range(5)]
    Jw0, _ = _fake_compute(np.ones((3, 4)), _Geom(), None, 1.0, 1.0, 2, dobs, None, range(5),
                           time_weights=tw)
    for _, J, g, Jw in res:
        assert J == pytest.approx(J0)
        assert np.allclose(g, g0)
        assert Jw == pytest.approx(Jw0)
