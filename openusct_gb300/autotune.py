"""Launch-shape autotuner and per-kernel timer.

The engine's tile shape (threads along the row x rows per CTA), z-chunk and
kernel variant are picked per (dimension, grid, batch width) by timing one
short forward sweep and one short backward sweep of each candidate with CUDA
events and keeping the fastest.  Results are cached in a JSON file
(``$OPENUSCT_GB300_CACHE`` or ``~/.cache/openusct_gb300/autotune.json``).

It is also the entry point for per-kernel profiling::

    python -m openusct_gb300.autotune --n 128 --batch 16 --nt 24 --what fwd --tiles 64x4x0x1

Tiles are written tile_x x tile_y [x zchunk [x variant [x stages]]].
"""

from __future__ import annotations

import argparse
import json
import os
import threading

import numpy as np

from . import _lib
from .geometry import CylinderGeometry, RingGeometry, element_csr, ricker

_CACHE_LOCK = threading.Lock()

# (tile_x, tile_y, zchunk, variant): variant 1 = TMA ring, 0 = register queue
CANDIDATES_3D = [(64, 4, 0, 1), (32, 8, 0, 1), (64, 2, 0, 1), (32, 4, 0, 1), (64, 4, 0, 0),
                 (64, 2, 0, 0)]
CANDIDATES_2D = [(128, 1, 0, 1), (64, 1, 0, 1), (128, 1, 0, 0), (64, 1, 0, 0)]


def cache_path():
    return os.environ.get("OPENUSCT_GB300_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "openusct_gb300",
                                       "autotune.json"))


def _load_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _save_cache(d):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1)
        os.replace(tmp, p)
    except OSError:
        pass


def key(shape, C):
    return f"{len(shape)}d:{'x'.join(str(int(s)) for s in shape)}:C{int(C)}"


def lookup(shape, C):
    with _CACHE_LOCK:
        v = _load_cache().get(key(shape, C))
    return tuple(v["tile"]) if v else None


def _synthetic(shape, nt):
    """A homogeneous medium with elements on a ring/cylinder that fits the grid."""
    n = min(shape)
    h = 2e-4
    if len(shape) == 2:
        geom = RingGeometry(8, 0.4 * (n - 1) * h, (n - 1) * h, h)
    else:
        geom = CylinderGeometry(2, 8, 0.4 * (n - 1) * h, 0.3 * (n - 1) * h, (n - 1) * h, h)
    idx = [tuple(min(int(a), s - 2) for a, s in zip(t, shape)) for t in geom.idx]
    from .geometry import IndexGeometry
    m = np.full(shape, 1.0 / 1500.0 ** 2)
    dt = 0.3 * h / 1500.0
    return IndexGeometry(idx), m, h, dt, ricker(nt, dt, 1e6)


def time_kernels(shape, C, nt, tile, what=("fwd", "adj"), reps=2, tblock=0, tblock_stages=0,
                 tblock_zchunk=0):
    """Per-launch milliseconds of the forward, Born-forward and adjoint stencils
    for a tile (``what`` names those timed: "fwd", "born", "adj").  With
    ``tblock`` (a two-step tile W*100+H, or 1 for the default) the forward sweep
    takes two levels per launch and ``fwd_ms`` is per level."""
    import torch
    from .backend import Plan, _ptr, _stream
    geom, m, h, dt, wav = _synthetic(shape, nt)
    nsh = len(geom.idx)
    shots = [i % nsh for i in range(C)]
    tx, rx = element_csr(geom, shape, shots, None)
    plan = Plan(shape, h, dt, nt, tx, rx, batch=C, ckpt_k=max(2, nt - 1), tile_x=tile[0],
                tile_y=tile[1], zchunk=tile[2], variant=tile[3] if len(tile) > 3 else None,
                stages=tile[4] if len(tile) > 4 else None)
    if len(tile) > 5:
        plan.set("stages_adj", int(tile[5]))
    if tblock_stages:
        plan.set("tblock_stages", int(tblock_stages))
    if tblock_zchunk:
        plan.set("tblock_zchunk", int(tblock_zchunk))
    if tblock:
        plan.set("tblock", int(tblock))
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    md = torch.from_numpy(m).to(dev)
    wd = torch.from_numpy(wav).to(dev)
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    mode = (_lib.MODE_BORN if "born" in what else
            _lib.MODE_GRADIENT if "adj" in what else _lib.MODE_FORWARD)
    bws = torch.empty(plan.batch_bytes(mode), dtype=torch.uint8, device=dev)
    s = _stream()
    # a Born perturbation (1 % of m, smooth) when the Born sweep is timed
    vd = (0.01 * md).contiguous() if "born" in what else None
    _lib.check(lib.usct_model_prepare(plan.handle, _ptr(mws), _ptr(md), None, _ptr(vd), _ptr(wd),
                                      s))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    ts = torch.cuda.current_stream()
    # forward sweep (FORWARD mode: nt-1 stencil launches + 1 gather)
    _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), 0, _lib.MODE_FORWARD,
                                      None, s))
    if "fwd" in what:
        e0.record(ts)
        for _ in range(reps):
            _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), 0,
                                              _lib.MODE_FORWARD, None, s))
        e1.record(ts)
        torch.cuda.synchronize()
        out["fwd_ms"] = e0.elapsed_time(e1) / (reps * (nt - 1))
    if "born" in what:
        # background and Born fields in lockstep: nt-1 launches of the Born stencil
        e0.record(ts)
        for _ in range(reps):
            _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), 0,
                                              _lib.MODE_BORN, None, s))
        e1.record(ts)
        torch.cuda.synchronize()
        out["born_ms"] = e0.elapsed_time(e1) / (reps * (nt - 1))
    if "adj" in what:
        _lib.check(lib.usct_batch_forward(plan.handle, _ptr(mws), _ptr(bws), 0,
                                          _lib.MODE_GRADIENT, None, s))
        adj = torch.zeros((C, nt, plan.n_rx), dtype=torch.float32, device=dev)
        adj[:, nt // 2, :] = 1.0
        _lib.check(lib.usct_batch_adjoint_source(plan.handle, _ptr(bws), 0, _ptr(adj), s))
        e0.record(ts)
        for _ in range(reps):
            _lib.check(lib.usct_batch_backward(plan.handle, _ptr(mws), _ptr(bws), 0, s))
        e1.record(ts)
        torch.cuda.synchronize()
        # one segment (k = nt-1): the backward is nt-1 adjoint launches, no recompute
        out["adj_ms"] = e0.elapsed_time(e1) / (reps * (nt - 1))
    cells = int(np.prod(shape))
    if "fwd_ms" in out:
        out["fwd_GBs"] = (12 * C + 4) * cells / (out["fwd_ms"] * 1e-3) / 1e9
    if "adj_ms" in out:
        out["adj_GBs"] = (16 * C + 20) * cells / (out["adj_ms"] * 1e-3) / 1e9
    if "born_ms" in out:
        # the plan is one checkpoint segment, so every Born launch also writes
        # the background's d2p stash (the last segment's): 24 C + 8 + 4 C
        out["born_GBs"] = (28 * C + 8) * cells / (out["born_ms"] * 1e-3) / 1e9
    plan.check()
    out["tile"] = [plan.info("tile_x"), plan.info("tile_y"), plan.info("zchunk"),
                   plan.info("variant")] + [int(v) for v in tile[4:6]]
    if tblock:
        out["tblock"] = plan.info("tblock")
    plan.close()
    return out


def tune(shape, C, nt=24, candidates=None, store=True):
    """Time every candidate launch shape; return (best_tile, results)."""
    cands = candidates or (CANDIDATES_3D if len(shape) == 3 else CANDIDATES_2D)
    res = []
    for t in cands:
        if 4 * t[0] < C:
            continue
        try:
            r = time_kernels(shape, C, nt, t)
        except Exception as exc:  # an unsupported shape is skipped, not fatal
            r = {"tile": list(t), "error": str(exc)[:200]}
        res.append(r)
    ok = [r for r in res if "fwd_ms" in r]
    best = min(ok, key=lambda r: 2 * r["fwd_ms"] + r.get("adj_ms", 0.0)) if ok else None
    if best and store:
        with _CACHE_LOCK:
            d = _load_cache()
            d[key(shape, C)] = {"tile": best["tile"], "results": res}
            _save_cache(d)
    return (tuple(best["tile"]) if best else None), res


def _parse_tiles(s):
    out = []
    for part in s.split(","):
        f = [int(v) for v in part.lower().split("x")]
        out.append(tuple([f[0], f[1], f[2] if len(f) > 2 else 0] + f[3:]))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--nt", type=int, default=24)
    ap.add_argument("--what", default="fwd,adj")
    ap.add_argument("--tiles", default="")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--store", action="store_true")
    ap.add_argument("--tblock", default="",
                    help="two-step forward tiles W*100+H (1 = default), comma-separated")
    ap.add_argument("--tblock-stages", type=int, default=0)
    ap.add_argument("--tblock-zchunk", default="0")
    a = ap.parse_args()
    shape = (a.n,) * a.dim
    what = tuple(a.what.split(","))
    if a.tblock:
        t = _parse_tiles(a.tiles)[0] if a.tiles else (0, 0, 0)
        for tb in [int(v) for v in a.tblock.split(",")]:
            for zc in [int(v) for v in a.tblock_zchunk.split(",")]:
                print(json.dumps({"shape": shape, "C": a.batch, "tblock_zchunk": zc,
                                  **time_kernels(shape, a.batch, a.nt, t, what, a.reps, tb,
                                                 a.tblock_stages, zc)}))
    elif a.tiles:
        for t in _parse_tiles(a.tiles):
            print(json.dumps({"shape": shape, "C": a.batch, **time_kernels(shape, a.batch, a.nt,
                                                                           t, what, a.reps)}))
    else:
        best, res = tune(shape, a.batch, a.nt, store=a.store)
        for r in res:
            print(json.dumps({"shape": shape, "C": a.batch, **r}))
        print(json.dumps({"best": best}))


if __name__ == "__main__":
    main()
