"""Benchmark: batched, checkpointed 3D FMC L2 gradient on one GB300.

Workload (N=1): the 192^3 cylinder acquisition (dx = 0.2 mm, 8 rings x 32
elements = 256 shots, nt = 2000, 1 MHz Ricker, seeded Gaussian random-field
model) -- the gradient configuration the headline metric is quoted on.  One
step = the exact discrete-adjoint L2 gradient of one batch of 32 shots (one
ring): forward sweep with checkpoints every k steps, residual, backward sweep
with bit-identical segment recompute and the fused imaging condition, all 32
shots advancing in one launch per time step.  Inputs are larger than L2 (every
launch streams ~0.9 GB per wavefield level).

Reported alongside: the kernel roofline of the dominant kernel (the forward
stencil, timed live with CUDA events on its stream), the end-to-end rate
through the public backend API with host buffers, the plain one-shot-per-launch
GPU form on the same workload, the reference scheme on the host cores (the
oracle's FP64 restatement, bit-identical to the reference C++ core), SM clocks
sampled during the timed region and the number of kernels launched.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Other workloads (not the default line): --workload fmc3d (the forward FMC of
the 192^3 cylinder acquisition: all 256 shots, nt=2000), ring2d (the 2D 256^2
ring, all 64 shots per launch), gn3d (the 224^3 Gauss-Newton Hessian-vector product),
grad3d_large (320^3, 512 shots, 8 per launch), tfm2d (the TFM image of a
64 x 1500 x 64 FMC), invert2d (iterations of the device-resident inversion
loop on the 2D ring), io (the Dataset HDF5 file of the 192^3 acquisition:
save and load on the host cores, no GPU).  --misfit gcn and --windows run the gradient workloads
with the GCN misfit and with P-arrival data windows.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))

METRIC = "Grad shots/s + p50/p99, batched serve vs per-shot plain, same GB300, relerr≤1e-4"
WORKLOAD = ("3D acoustic cylinder FMC L2 gradient, 192^3, dx=0.2mm, 8x32 elements (256 shots), "
            "nt=2000, FP32, 32 shots per launch, the backend's default checkpoint interval (the "
            "last segment, never recomputed, as long as 70% of the device allows)")

# name -> (description, problem builder, shots per launch, checkpoint k (0: the
# backend's default interval), mode)
#   mode "grad": one step = the L2 gradient of one batch (model: 44 B/shot + 20 B/batch
#   per cell-step); "gn": one step = the Gauss-Newton product of one batch
#   (44 + 12 B/shot + 24 B/batch)
WORKLOADS = {
    "grad3d": (WORKLOAD, lambda: __import__("openusct_gb300.problems").problems.cylinder3d(seed=0),
               32, 0, "grad"),
    "ring2d": ("2D ring FWI L2 gradient, 256^2, dx=0.15mm, 64-element ring r=16mm, two seeded "
               "discs, 1 MHz Ricker, nt=1500, FP32, all 64 shots in one launch",
               lambda: __import__("openusct_gb300.problems").problems.ring2d(seed=0), 64, 0, "grad"),
    "gn3d": ("3D Gauss-Newton Hessian-vector product (Born + adjoint), 224^3, dx=0.18mm, 8x32 "
             "elements (256 shots), nt=2500, FP32, 16 shots per launch",
             lambda: __import__("openusct_gb300.problems").problems.gn3d(seed=0), 16, 0, "gn"),
    "grad3d_large": ("3D cylinder FMC L2 gradient, 320^3, dx=0.12mm, 16x32 elements (512 shots), "
                     "nt=3000, FP32, 8 shots per launch",
                     lambda: __import__("openusct_gb300.problems").problems.cylinder3d_large(seed=0),
                     8, 0, "grad"),
}


def schedule_bytes(cells, C, nt, k, mode):
    """Algorithmic bytes of one batch through the engine's schedule: the
    forward sweep (12 C + 4, Born 24 C + 8 per cell-step) on every level, the
    d2p stash it writes on the last segment's levels (4 C), the segment
    recompute (16 C + 4) on every other level, the adjoint (16 C + 20: S and
    the FP64 gradient read-modify-write per batch) on every level."""
    k = min(max(2, k), max(2, nt - 1))
    nseg = (nt - 1 + k - 1) // k
    rec = (nseg - 1) * k
    tail = nt - 1 - rec
    fwd = 24 * C + 8 if mode == "gn" else 12 * C + 4
    return cells * ((nt - 1) * (fwd + 16 * C + 20) + tail * 4 * C + rec * (16 * C + 4)), rec, tail


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clock / throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
                for nm, v in zip(names, f[3:7]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


def host_available_bytes():
    """MemAvailable of this host (bytes), 0 when it cannot be read."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def cpu_shot_interval(prob, mode, frac=0.65):
    """The FP64 oracle's memory plan for one whole shot on this host: k = 0 --
    the full history of every level, no recompute, the reference core's own
    plan (libuap.hpp:179-186) -- when that history fits ``frac`` of the
    available host memory, else the longest checkpoint interval whose
    checkpoints and segment fit (the Gauss-Newton restatement always
    checkpoints).  Returns (k, bytes)."""
    import numpy as np
    N = int(np.prod(prob.shape))
    nt = prob.nt
    if mode == "fwd":   # three levels in flight, no history
        return 0, 3 * N * 8
    avail = host_available_bytes() or (64 << 30)
    budget = frac * avail
    hist = nt * N * 8
    if mode != "gn" and hist <= budget:
        return 0, hist
    for k in range(nt - 1, 1, -1):
        nseg = (nt - 1 + k - 1) // k
        need = (2 * nseg + k + 2 + (4 if mode == "gn" else 0)) * N * 8
        if need <= budget:
            return k, need
    return 2, (2 * (nt - 1) + 8) * N * 8


def cpu_whole_shot(prob, shot, k, dobs1=None, mode="grad", misfit="l2"):
    """Time the FP64 oracle's gradient (or Gauss-Newton product) of one whole
    shot over the full time axis with memory plan k: (seconds, text)."""
    import numpy as np
    import oracle
    geom = prob.geom
    grid = "x".join(str(v) for v in prob.shape)
    if mode == "fwd":
        t0 = time.perf_counter()
        oracle.forward_fmc(prob.m_true, geom, prob.wavelet, prob.dt, prob.h, prob.nt, None,
                           [shot])
        return time.perf_counter() - t0, (f"1 whole shot ({prob.nt} levels) of the {grid} "
                                          "forward FMC, every receiver recorded")
    if mode == "gn":
        t0 = time.perf_counter()
        oracle.gn_hessian_vector(prob.m0, geom, prob.wavelet, prob.dt, prob.h, prob.nt, prob.v,
                                 src_list=[shot], k=k)
        return time.perf_counter() - t0, (f"1 whole shot ({prob.nt} levels) of the Gauss-Newton "
                                          f"product, background checkpointed every {k} steps")
    t0 = time.perf_counter()
    oracle.misfit_and_gradient(prob.m0, geom, prob.wavelet, prob.dt, prob.h, prob.nt,
                               np.asarray(dobs1, np.float64), None, [shot], k=k,
                               misfit_type=misfit)
    plan = ("full history, no recompute (the reference core's memory plan)" if k == 0 else
            f"checkpoints every {k} steps (the full history does not fit this host)")
    return time.perf_counter() - t0, f"1 whole shot ({prob.nt} levels) of the {grid} gradient, {plan}"


SERVE_STREAM = ("seeded Poisson stream at 20 req/s, 30% gradient / 70% forward, half 2D rings "
                "(128^2-1024^2, 32-256 elements) half 3D cylinders (96^3-256^3, 64-512 elements), "
                "disc or random-field models, nt = 2.2*2R/1450/dt (the serving configuration's "
                "distribution; the first {n} of its 2000 requests); HBM budget 150 GB, 12 slots, "
                "each request's batch workspace sized within 50 GB")


def serve_phase(args):
    """Continuous-batching service on a scaled request stream: p50/p99 latency
    and shots/s, against the same requests solved one shot at a time by the
    plain one-shot-per-launch GPU form (timed on one shot of each request)."""
    import numpy as np
    import torch
    import openusct_gb300.backend as gb
    from openusct_gb300.serve import Engine, GpuExecutor, make_stream, summarize

    def dobs_fn(m, geom, wav, dt, h, nt):
        return gb.forward_fmc(m, geom, wav, dt, h, nt)

    reqs = make_stream(args.serve_requests, rate_hz=20.0, seed=11, sizes_2d=(128, 1024),
                       sizes_3d=(96, 256), elements_2d=(32, 256), elements_3d=(64, 512),
                       frac_gradient=0.3, dobs_fn=dobs_fn)
    gb.release()
    budget = 150 << 30
    eng = Engine(GpuExecutor(workspace_bytes=budget // 3), budget_bytes=budget, max_active=12)
    res = eng.run_stream(reqs)
    st = summarize(res, eng)
    # plain form: one shot of every request, the median of three timed calls
    # (CUDA events), scaled by the request's shot count
    plain_s = 0.0
    for q in reqs:
        one = [0]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if q.kind == "forward":
            call = lambda: gb.plain_forward_fmc(q.m, q.geom, q.wavelet, q.dt, q.h, q.nt,  # noqa
                                                src_list=one)
        else:
            d1 = q.dobs[:1]
            call = lambda: gb.plain_misfit_and_gradient(q.m, q.geom, q.wavelet, q.dt, q.h,  # noqa
                                                        q.nt, d1, src_list=one)
        call()
        runs = []
        for _ in range(3):
            e0.record()
            call()
            e1.record()
            torch.cuda.synchronize()
            runs.append(e0.elapsed_time(e1) / 1000.0)
        plain_s += statistics.median(runs) * q.n_shots
    gb.release()
    plain_rate = st.shots / plain_s if plain_s > 0 else None
    co = co_admission()
    lat = latency_stream(dobs_fn)
    return {"stream": SERVE_STREAM.format(n=st.n), "requests": st.n, "ok": st.ok,
            "rejected": st.rejected, "waited_for_budget": st.waited_for_budget,
            "merged_into_shared_launches": st.merged,
            "budget_gb": budget / 2 ** 30,
            "p50_s": st.p50_s, "p99_s": st.p99_s, "mean_s": st.mean_s,
            "makespan_s": st.makespan_s, "shots": st.shots, "shots_per_s": st.shots_per_s,
            "max_concurrent": st.max_concurrent,
            "peak_reserved_gb": st.peak_reserved_bytes / 2 ** 30,
            "plain_sequential_shots_per_s": plain_rate,
            "co_admission": co,
            "latency_stream": lat,
            "speedup_vs_plain_sequential": (st.shots_per_s / plain_rate) if plain_rate else None}


GN_WORKLOAD = ("3D Gauss-Newton Hessian-vector product (Born + adjoint), 224^3, dx=0.18mm, 8x32 "
               "elements (256 shots), nt=2500, FP32, seeded smooth perturbation, 16 shots per "
               "launch, the backend's default checkpoint interval; one step = one 16-shot batch")


def gauss_newton_phase(args):
    """The Gauss-Newton configuration: the 224^3 Hessian-vector product timed
    on one 16-shot batch (device-resident inputs, CUDA events), and four
    Gauss-Newton iterations of the 2D ring problem served as one long-lived
    device-resident request (arrival -> final model on the host)."""
    import ctypes
    import numpy as np
    import torch
    import openusct_gb300.backend as gb
    from openusct_gb300 import _lib, problems
    from openusct_gb300.geometry import element_csr
    from openusct_gb300.serve import Engine, GpuExecutor, Request

    dev = torch.device("cuda", torch.cuda.current_device())
    prob = problems.gn3d(seed=0)
    C = 16
    shots = list(range(C))
    tx, rx = element_csr(prob.geom, prob.shape, shots, None)
    k = gb.default_ckpt_k(prob.shape, prob.nt, rx.rows, len(rx.cell), C, _lib.MODE_BORN)
    plan = gb.Plan(prob.shape, prob.h, prob.dt, prob.nt, tx, rx, batch=C, ckpt_k=k)
    lib = _lib.load()
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    m0 = torch.from_numpy(prob.m0).to(dev)
    v = torch.from_numpy(prob.v).to(dev)
    wav = torch.from_numpy(prob.wavelet).to(dev)
    hv = torch.empty(prob.shape, dtype=torch.float64, device=dev)
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    bws = torch.empty(plan.batch_bytes(_lib.MODE_BORN), dtype=torch.uint8, device=dev)
    call = lambda: _lib.check(lib.usct_gn_hessian_vector_dev(  # noqa: E731
        plan.handle, P(m0), None, P(wav), P(v), P(hv), None, P(mws), P(bws), sp))
    call()
    reps = 2
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(reps):
        call()
    e1.record(s)
    torch.cuda.synchronize()
    plan.check()
    t = e0.elapsed_time(e1) / 1000.0 / reps
    cells = int(np.prod(prob.shape))
    hbm, peak_kind = _peaks()
    k_used = plan.info("ckpt_k")
    sched, _, _ = schedule_bytes(cells, C, prob.nt, k_used, "gn")
    del bws, mws
    plan.close()
    torch.cuda.empty_cache()
    # four Gauss-Newton iterations of the 2D ring problem as one served request
    ring = problems.ring2d(seed=0)
    geo = (ring.geom, ring.wavelet, ring.dt, ring.h, ring.nt)
    dobs = gb.forward_fmc(ring.m_true, *geo)
    n = ring.shape[0]
    yy, xx = np.mgrid[0:n, 0:n].astype(float) * ring.h
    cc = (n - 1) * ring.h / 2
    mask = (np.hypot(xx - cc, yy - cc) <= 0.8 * 0.016).astype(float)
    req = Request(kind="gauss-newton", m=ring.m0.copy(), geom=ring.geom, wavelet=ring.wavelet,
                  dt=ring.dt, h=ring.h, nt=ring.nt, dobs=dobs, update_mask=mask, n_iter=4,
                  n_cg=8)
    gb.release()
    res = Engine(GpuExecutor(), budget_bytes=150 << 30, max_active=2).run_stream([req])[0]
    served = {"problem": "2D ring configuration (256^2, 64 shots, nt=1500), 4 iterations, "
                         "8 CG steps each, radial update mask",
              "ok": res.ok, "error": res.error, "latency_s": res.latency if res.ok else None,
              "misfit_history": res.history}
    return {"workload": GN_WORKLOAD, "value": C / t, "unit": "shots/s", "ms_per_batch": t * 1e3,
            "ckpt_k": k_used,
            "pipeline_frac": sched / t / 1e9 / hbm, "peak_kind": peak_kind,
            "served_gauss_newton_request": served}


def latency_stream(dobs_fn, n=200):
    """Latency percentiles over a longer stream: 200 seeded requests at 20
    req/s (the serving configuration's mix and rate) with sizes scaled to
    128^2-512^2 / 64^3-128^3 and 32-128 elements, so that p99 is a percentile
    rather than the slowest request (the 24-request stream's p99 is)."""
    from openusct_gb300.serve import Engine, GpuExecutor, make_stream, summarize
    reqs = make_stream(n, rate_hz=20.0, seed=12, sizes_2d=(128, 512), sizes_3d=(64, 128),
                       elements_2d=(32, 128), elements_3d=(64, 128), frac_gradient=0.3,
                       dobs_fn=dobs_fn)
    budget = 150 << 30
    eng = Engine(GpuExecutor(workspace_bytes=budget // 3), budget_bytes=budget, max_active=12)
    res = eng.run_stream(reqs)
    st = summarize(res, eng)
    return {"stream": f"{n} seeded requests at 20 req/s, 30% gradient, 2D 128^2-512^2 / 3D "
                      "64^3-128^3, 32-128 elements; 150 GB budget, 12 slots",
            "requests": st.n, "ok": st.ok, "p50_s": st.p50_s, "p99_s": st.p99_s,
            "mean_s": st.mean_s, "makespan_s": st.makespan_s, "shots_per_s": st.shots_per_s,
            "max_concurrent": st.max_concurrent}


def co_admission():
    """Compatible small forward requests (48 requests of 8 shots on one 2D
    256^2 grid, each on its own model, arriving together: more than the 12
    slots) served with shared launches (per-channel models, up to 32 shots a
    launch) and with one plan per request; shots/s both ways, and that the
    traces agree."""
    import numpy as np
    from openusct_gb300 import problems
    from openusct_gb300.serve import Engine, GpuExecutor, Request, summarize
    base = problems.ring2d(seed=0)
    rng = np.random.default_rng(5)
    reqs = []
    for k in range(48):
        m = base.m_true * (1.0 + 0.005 * rng.standard_normal(base.m_true.shape))
        src = [int(s) for s in rng.choice(len(base.geom.idx), size=8, replace=False)]
        reqs.append(Request(kind="forward", m=m, geom=base.geom, wavelet=base.wavelet,
                            dt=base.dt, h=base.h, nt=base.nt, src_list=src))
    out = {}
    traces = {}
    for slots in (12, 2):
        for name, merge in (("shared", True), ("separate", False)):
            Engine(GpuExecutor(merge=merge), budget_bytes=150 << 30,
                   max_active=slots).run_stream(reqs[:2], realtime=False)   # warm-up
            eng = Engine(GpuExecutor(merge=merge), budget_bytes=150 << 30, max_active=slots)
            res = eng.run_stream(reqs, realtime=False)
            st = summarize(res, eng)
            key = f"{name}_{slots}_slots"
            out[key + "_shots_per_s"] = st.shots_per_s
            out[key + "_groups"] = len({(r.t_admit, r.group) for r in res if r.ok})
            traces[key] = [r.traces for r in res]
    ref = traces["separate_12_slots"]
    out["traces_equal"] = all(all(np.array_equal(a, b) for a, b in zip(t, ref))
                              for t in traces.values())
    out["stream"] = ("48 forward requests of 8 shots, 2D 256^2 ring (64 elements), nt=1500, each "
                     "on its own perturbed model, arriving together; 12 and 2 slots")
    return out


def run_reference(args, prob, desc_w, mode):
    """--impl reference: the reference scheme's CPU path on the host cores.
    One step = the gradient (or Gauss-Newton product) of one whole shot over
    the full time axis, by the oracle's FP64 restatement of the reference core
    (bit-identical to it), with the reference's full-history memory plan when
    it fits this host.  The observed data of the shot come from one untimed
    FP64 forward run."""
    import oracle
    oracle.build()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    kind = "port"
    k, mem = cpu_shot_interval(prob, mode)
    shot = 0
    dobs1 = None
    if mode == "grad":
        dobs1 = oracle.forward_fmc(prob.m_true, prob.geom, prob.wavelet, prob.dt, prob.h,
                                   prob.nt, None, [shot])
    secs = []
    desc = ""
    for i in range(args.warmup + args.steps):
        s_i, desc = cpu_whole_shot(prob, shot, k, dobs1, mode)
        if i >= args.warmup:
            secs.append(s_i)
    ms = 1000.0 * sum(secs) / len(secs)
    value = 1000.0 / ms
    line = {"metric": FMC_METRIC if mode == "fwd" else METRIC, "value": value,
            "unit": "shots/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": desc_w, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": value, "unit": "shots/s", "cores": cores, "kind": kind,
                             "sample": desc, "host_bytes": mem,
                             "seconds_per_step": [round(v, 3) for v in secs]},
            "e2e": {"value": value, "unit": "shots/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


FMC_METRIC = "Forward FMC shots/s (all transmits x all receivers x nt), same GB300, relerr<=1e-5"
FMC_WORKLOAD = ("3D acoustic cylinder forward FMC, 192^3, dx=0.2mm, 8x32 elements (all 256 "
                "shots), nt=2000, FP32 (the seeded random-field model); one step = the whole "
                "acquisition, 256 x 2000 x 256 traces")


def bench_fmc(args, prob):
    """--workload fmc3d: the forward FMC of a whole acquisition (fwi.forward_fmc,
    fwi.py:109-118) -- every transmit's forward sweep with every receiver
    recorded, C shots per launch.  One step = all transmits."""
    import ctypes
    import numpy as np
    import torch
    from openusct_gb300 import _lib, backend
    from openusct_gb300.geometry import element_csr

    dev = torch.device("cuda", 0)
    torch.cuda.set_stream(torch.cuda.Stream(device=dev))
    C = args.batch or 32
    tx, rx = element_csr(prob.geom, prob.shape, None, None)
    plan = backend.Plan(prob.shape, prob.h, prob.dt, prob.nt, tx, rx, batch=C)
    lib = _lib.load()
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    m = torch.from_numpy(prob.m_true).to(dev)
    wav = torch.from_numpy(prob.wavelet).to(dev)
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    bws = torch.empty(plan.batch_bytes(_lib.MODE_FORWARD), dtype=torch.uint8, device=dev)
    data = torch.empty((plan.n_tx, prob.nt, plan.n_rx), dtype=torch.float32, device=dev)

    def step():
        _lib.check(lib.usct_forward_fmc_dev(plan.handle, P(m), None, P(wav), P(data), P(mws),
                                            P(bws), sp))

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    launches0 = plan.info("launches")
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        torch.cuda.synchronize()
        ev0.record(s)
        for _ in range(args.steps):
            step()
        ev1.record(s)
        torch.cuda.synchronize()
    launches = plan.info("launches") - launches0
    t_ms = ev0.elapsed_time(ev1) / args.steps
    value = plan.n_tx / (t_ms / 1000.0)
    cells = int(np.prod(prob.shape))
    hbm, peak_kind = _peaks()
    # the forward stencil launch alone: two sweeps of one batch, traces not kept
    nrep = 2
    ev0.record(s)
    for _ in range(nrep):
        _lib.check(lib.usct_batch_forward(plan.handle, P(mws), P(bws), 0, _lib.MODE_FORWARD,
                                          None, sp))
    ev1.record(s)
    torch.cuda.synchronize()
    t_launch = ev0.elapsed_time(ev1) / 1000.0 / (nrep * (prob.nt - 1))
    fwd_bytes = (12 * C + 4) * cells
    achieved = fwd_bytes / t_launch / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "k_forward_tma_128cube_C32.md")
    if C == 32 and os.path.exists(prof):
        kv = {}
        for line in open(prof):
            if ":" in line and line.split(":")[0] in ("dram_bytes_per_launch", "cell_channels"):
                kv[line.split(":")[0]] = float(line.split(":")[1])
        if len(kv) == 2:
            traffic = kv["dram_bytes_per_launch"] * (cells * C) / kv["cell_channels"]
    nbatch = plan.nbatch
    step_bytes = nbatch * (prob.nt - 1) * fwd_bytes + data.numel() * 4

    # end to end through the public API: FP64 model and wavelet up, the FP64
    # traces back to the host (the call's own return type)
    del bws, data
    torch.cuda.empty_cache()
    call = lambda: backend.forward_fmc(prob.m_true, prob.geom, prob.wavelet, prob.dt,  # noqa
                                       prob.h, prob.nt, batch=C)
    out = call()
    t0 = time.perf_counter()
    ne = 2
    for _ in range(ne):
        out = call()
    te = (time.perf_counter() - t0) / ne
    e2e = {"value": plan.n_tx / te, "unit": "shots/s",
           "h2d_bytes_per_step": int(prob.m_true.nbytes + prob.wavelet.nbytes),
           "d2h_bytes_per_step": int(out.nbytes), "api": "openusct_gb300.backend.forward_fmc"}
    del out
    backend.release()

    plain = None
    if not args.no_plain:
        torch.cuda.empty_cache()
        tx1, rx1 = element_csr(prob.geom, prob.shape, [0], None)
        pplan = backend.Plan(prob.shape, prob.h, prob.dt, prob.nt, tx1, rx1, batch=1)
        pws = torch.empty(pplan.plain_bytes(False), dtype=torch.uint8, device=dev)
        d1 = torch.empty((1, prob.nt, pplan.n_rx), dtype=torch.float32, device=dev)
        args_p = (pplan.handle, P(m), P(wav), P(d1), P(pws), sp)
        _lib.check(lib.usct_plain_forward_fmc_dev(*args_p))
        torch.cuda.synchronize()
        times = []
        for _ in range(3):   # the median of three timed calls
            ev0.record(s)
            _lib.check(lib.usct_plain_forward_fmc_dev(*args_p))
            ev1.record(s)
            torch.cuda.synchronize()
            times.append(ev0.elapsed_time(ev1) / 1000.0)
        tp = statistics.median(times)
        plain = {"value": 1.0 / tp, "unit": "shots/s", "ms_per_shot": tp * 1000.0,
                 "ms_per_shot_runs": [t * 1000.0 for t in times],
                 "speedup_batched_vs_plain": value * tp}
        del pws, d1
        pplan.close()

    cpu = None
    if not args.no_cpu:
        try:
            import oracle
            oracle.build()
            secs, desc = cpu_whole_shot(prob, 0, 0, None, "fwd")
            cpu = {"value": 1.0 / secs, "unit": "shots/s",
                   "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                   "kind": "port", "sample": desc, "seconds": secs}
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "error": str(exc)[:200]}

    line = {"metric": FMC_METRIC, "value": value, "unit": "shots/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": t_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian random-field model)",
            "config": {"workload": FMC_WORKLOAD, "grid": list(prob.shape), "nt": prob.nt,
                       "shots": plan.n_tx, "receivers": plan.n_rx, "batch_shots": C,
                       "tile": [plan.info("tile_x"), plan.info("tile_y"), plan.info("zchunk")],
                       "parallelism": "single", "l2": "inputs larger than L2 (no flush needed)"},
            "grid_updates_per_s": value * cells * (prob.nt - 1),
            "roofline": {"bound": "hbm",
                         "kernel": f"k_forward_tma (3D, {C} shots per launch)",
                         "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": traffic,
                         "traffic_source": ("profiles/k_forward_tma_128cube_C32.md, scaled by "
                                            "cell-channels" if traffic is not None else None),
                         "algorithmic_bytes_per_launch": fwd_bytes,
                         "launch_ms": t_launch * 1000.0},
            "pipeline_roofline": {"bytes_per_step": step_bytes,
                                  "achieved": step_bytes / (t_ms / 1000.0) / 1e9,
                                  "frac": step_bytes / (t_ms / 1000.0) / 1e9 / hbm,
                                  "model": f"12C+4 B per cell on {prob.nt - 1} levels of each of "
                                           f"{nbatch} batches, plus the FP32 traces written"},
            "e2e": e2e, "plain": plain, "cpu_baseline": cpu, "gpu_launches": launches,
            "clocks": clk.summary()}
    print(json.dumps(line))


IO_WORKLOAD = ("Dataset HDF5 file (dataset.py:112-174 layout) of the 192^3 cylinder acquisition: "
               "256 x 2000 x 256 FP32 traces (524 MB), gzip level 4 as the reference writes "
               "them; one step = save + load")


def bench_io(args):
    """--workload io: the portable Dataset file written and read by
    openusct_gb300.dataset_io (no h5py) on the host cores."""
    import tempfile
    import numpy as np
    from openusct_gb300 import dataset_io
    from openusct_gb300.acquire import ArrayGeometry, Dataset
    rng = np.random.default_rng(0)
    n_tx, nt, n_rx = 256, 2000, 256
    t = np.arange(nt)
    # band-limited seeded traces (compressibility like recorded wavelets, not noise)
    data = (np.sin(0.05 * t[None, :, None] + rng.uniform(0, 2 * np.pi, (n_tx, 1, n_rx))) *
            np.exp(-((t[None, :, None] - 1000) / 400.0) ** 2) * 1e-3).astype(np.float32)
    ds = Dataset(ArrayGeometry(rng.standard_normal((n_rx, 3)) * 0.01, 0.015, 1e6, "cylinder"),
                 data, 1 / 4.0e-8, np.zeros(nt), 1e6, 1500.0, np.arange(n_tx), None, {})
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "acq.h5")
        saves, loads = [], []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            dataset_io.save(ds, path)
            t1 = time.perf_counter()
            got = dataset_io.load(path)
            t2 = time.perf_counter()
            if i >= args.warmup:
                saves.append(t1 - t0)
                loads.append(t2 - t1)
        assert np.array_equal(got.data, data)
        size = os.path.getsize(path)
    ts, tl = statistics.median(saves), statistics.median(loads)
    mb = data.nbytes / 1e6
    cores = os.cpu_count() or 1
    line = {"metric": "Dataset file MB/s (save + load of the FP32 traces)",
            "value": 2 * mb / (ts + tl), "unit": "MB/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * (ts + tl), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": IO_WORKLOAD, "file_mb": size / 1e6, "cores": cores},
            "save_mb_per_s": mb / ts, "load_mb_per_s": mb / tl,
            "e2e": {"value": 2 * mb / (ts + tl), "unit": "MB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0, "api": "openusct_gb300.dataset_io.save/load"},
            "cpu_baseline": None, "gpu_launches": 0}
    print(json.dumps(line))


INVERT_WORKLOAD = ("FWI inversion loop (fwi.invert: steepest descent on the Gaussian-smoothed "
                   "gradient, backtracking line search), 2D 256^2 ring, dx=0.15mm, 64 elements, "
                   "two seeded discs, nt=1500, L2, model and gradient kept on the GPU")


def bench_invert(args):
    """--workload invert2d: iterations/s of the device-resident fwi.invert
    (openusct_gb300.invert.invert, fwi.py:535-660) on the 2D ring problem; one
    step = one iteration: the gradient over all 64 shots, its smoothing and
    scaling, and the line search's trial misfits."""
    import numpy as np
    import torch
    from openusct_gb300 import backend, problems
    from openusct_gb300.invert import invert

    prob = problems.ring2d(seed=0)
    dev = torch.device("cuda", 0)
    geo = (prob.geom, prob.wavelet, prob.dt, prob.h, prob.nt)
    dobs_h = backend.forward_fmc(prob.m_true, *geo)
    dobs_d = torch.from_numpy(np.asarray(dobs_h, np.float32)).to(dev)
    m0_d = torch.from_numpy(prob.m0).to(dev)
    invert(m0_d, *geo, dobs_d, n_iter=max(3, args.warmup))
    s = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        torch.cuda.synchronize()
        ev0.record(s)
        _m, hist = invert(m0_d, *geo, dobs_d, n_iter=args.steps)
        ev1.record(s)
        torch.cuda.synchronize()
    t_ms = ev0.elapsed_time(ev1) / args.steps
    # end to end: the same call with host arrays (the model, data and wavelet
    # go up once per call, the model comes back)
    t0 = time.perf_counter()
    m_h, _ = invert(prob.m0, *geo, dobs_h, n_iter=args.steps)
    e2e_s = (time.perf_counter() - t0) / args.steps
    h2d = prob.m0.nbytes + np.asarray(dobs_h).nbytes + prob.wavelet.nbytes
    cpu = None
    if not args.no_cpu:
        try:
            import oracle
            from oracle import invert as oinv
            oracle.build()
            sub = [0, 16, 32, 48]
            t0 = time.perf_counter()
            oinv.invert(prob.m0, *geo, np.asarray(dobs_h)[sub], src_list=sub, n_iter=1,
                        backend=oinv.FP64Backend())
            secs = time.perf_counter() - t0
            cpu = {"value": len(sub) / 64.0 / secs, "unit": "iterations/s",
                   "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                   "kind": "port",
                   "sample": "1 iteration of the host restatement of fwi.invert (oracle/invert.py, "
                             "FP64 C core) with 4 of the 64 shots, scaled by 16",
                   "seconds": secs}
        except Exception as exc:  # reported, never required
            cpu = {"value": None, "error": str(exc)[:200]}
    line = {"metric": "FWI iterations/s (device-resident invert)", "value": 1000.0 / t_ms,
            "unit": "iterations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (two seeded discs; the data from the true model on the GPU)",
            "config": {"workload": INVERT_WORKLOAD, "grid": list(prob.shape), "nt": prob.nt,
                       "shots": 64, "l2": "three wavefield levels of all 64 shots (50 MB) fit "
                                         "in L2"},
            "misfit_history": [float(v) for v in hist],
            "e2e": {"value": 1.0 / e2e_s, "unit": "iterations/s",
                    "h2d_bytes_per_step": int(h2d / args.steps),
                    "d2h_bytes_per_step": int(m_h.nbytes / args.steps),
                    "api": "openusct_gb300.invert.invert"},
            "cpu_baseline": cpu, "clocks": clk.summary()}
    print(json.dumps(line))


TFM_WORKLOAD = ("TFM delay-and-sum envelope image (imaging.tfm), 64-element ring r=16mm, "
                "64x1500x64 FMC (dt=0.3*0.15mm/1580 m/s), 120x120 pixels over 0.95 r")


def bench_tfm(args):
    """--workload tfm2d: the reference's TFM (imaging.py:27-74) at the C1
    acquisition size; one step = one envelope image (analytic signal of every
    trace + the delay-and-sum over all pairs and pixels)."""
    import numpy as np
    import torch
    from openusct_gb300 import _lib, imaging
    from openusct_gb300.geometry import RingGeometry

    h, n_el, nt, npix = 0.15e-3, 64, 1500, 120
    ring = RingGeometry(n_el, 0.016, 255 * h, h)
    dt = 0.3 * h / 1580.0
    rng = np.random.default_rng(0)
    data = rng.standard_normal((n_el, nt, n_el))

    class Geom:
        element_pos = np.asarray(ring.element_positions, np.float64)
        radius_m = 0.016
        dim = 2

    class DS:
        geometry = Geom()
        tx_elements = np.arange(n_el)
        nominal_speed_m_s = 1500.0
        sample_rate_hz = 1.0 / dt

    DS.data = data
    dev = torch.device("cuda", 0)
    lib = _lib.load()
    s = torch.cuda.current_stream()
    sp = ctypes_void(s.cuda_stream)
    P = lambda t: ctypes_void(t.data_ptr())  # noqa: E731
    axes = imaging.image_axes(DS, npix)
    dd = torch.from_numpy(data).to(dev)
    taps = torch.from_numpy(imaging.hilbert_taps(nt).astype(np.float32)).to(dev)
    A = torch.empty((n_el, n_el, nt, 2), dtype=torch.float32, device=dev)
    txp = torch.from_numpy(Geom.element_pos.copy()).to(dev)
    ax = torch.from_numpy(np.stack(axes)).to(dev)
    ore = torch.empty(npix * npix, dtype=torch.float64, device=dev)
    oim = torch.empty_like(ore)
    import ctypes

    def step():
        _lib.check(lib.usct_analytic_dev(P(dd), P(A), n_el, nt, n_el, P(taps), sp))
        _lib.check(lib.usct_tfm_dev(P(A), n_el, n_el, nt, P(txp), P(txp), 2, P(ax), npix,
                                    ctypes.c_double(DS.nominal_speed_m_s),
                                    ctypes.c_double(DS.sample_rate_hz), P(ore), P(oim), sp))

    for _ in range(max(3, args.warmup)):
        step()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    with Clocks(0) as clk:
        ev[0].record(s)
        for _ in range(args.steps):
            step()
        ev[1].record(s)
        torch.cuda.synchronize()
    t_ms = ev[0].elapsed_time(ev[1]) / args.steps
    # the two calls separately (k_real + k_analytic, then k_tfm), each the
    # mean of args.steps launches between its own events
    reps = max(1, args.steps)
    ev[0].record(s)
    for _ in range(reps):
        _lib.check(lib.usct_analytic_dev(P(dd), P(A), n_el, nt, n_el, P(taps), sp))
    ev[1].record(s)
    for _ in range(reps):
        _lib.check(lib.usct_tfm_dev(P(A), n_el, n_el, nt, P(txp), P(txp), 2, P(ax), npix,
                                    ctypes.c_double(DS.nominal_speed_m_s),
                                    ctypes.c_double(DS.sample_rate_hz), P(ore), P(oim), sp))
    ev[2].record(s)
    torch.cuda.synchronize()
    t_an = ev[0].elapsed_time(ev[1]) / reps
    t_das = ev[1].elapsed_time(ev[2]) / reps
    # end to end through imaging.tfm with the host dataset
    imaging.tfm(DS, npix=npix)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        imaging.tfm(DS, npix=npix)
    e2e_s = (time.perf_counter() - t0) / args.steps
    cpu = None
    if not args.no_cpu:
        import oracle.tfm as otfm
        t0 = time.perf_counter()
        otfm.tfm(data, Geom.element_pos, DS.tx_elements, DS.nominal_speed_m_s, DS.sample_rate_hz,
                 0.016, npix)
        cs = time.perf_counter() - t0
        cpu = {"value": 1.0 / cs, "unit": "images/s", "cores": 1, "kind": "port",
               "sample": "one full image with the reference algorithm (NumPy/scipy FP64)",
               "seconds": cs}
    pairs = npix * npix * n_el * n_el
    line = {"metric": "TFM images/s", "value": 1000.0 / t_ms, "unit": "images/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian traces; TFM cost does not depend on values)",
            "config": {"workload": TFM_WORKLOAD, "n_tx": n_el, "n_rx": n_el, "nt": nt,
                       "npix": npix, "l2": "the 49 MB analytic signal is L2-resident"},
            "pairs_per_s": pairs / (t_ms / 1000.0),
            "kernels_ms": {"k_real+k_analytic": t_an, "k_tfm": t_das},
            # non-zero taps only (for even nt every other tap is zero and skipped)
            "analytic_gflops": 2.0 * n_el * n_el * nt * (nt // 2 if nt % 2 == 0 else nt)
                               / (t_an / 1000.0) / 1e9,
            "e2e": {"value": 1.0 / e2e_s, "unit": "images/s", "h2d_bytes_per_step": data.nbytes,
                    "d2h_bytes_per_step": 2 * 8 * npix * npix, "api": "openusct_gb300.imaging.tfm"},
            "cpu_baseline": cpu, "gpu_launches": 3 * args.steps, "clocks": clk.summary()}
    print(json.dumps(line))


def ctypes_void(v):
    import ctypes
    return ctypes.c_void_p(v)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="grad3d",
                    choices=sorted(WORKLOADS) + ["fmc3d", "tfm2d", "invert2d", "io"])
    ap.add_argument("--n", type=int, default=0, help="override the grid size (smaller variants)")
    ap.add_argument("--nt", type=int, default=0, help="override the time levels")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--ckpt", type=int, default=-1)
    ap.add_argument("--misfit", default="l2", choices=["l2", "gcn"],
                    help="gradient workloads: the misfit (L2 or GCN, libuap.hpp:125-162)")
    ap.add_argument("--windows", action="store_true",
                    help="gradient workloads: P-arrival data windows as time_weights")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=24)
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    import numpy as np
    from openusct_gb300 import problems

    if args.workload in ("tfm2d", "invert2d"):
        if args.impl == "reference" or rank != 0:
            return
        import torch
        torch.cuda.set_device(0)
        (bench_tfm if args.workload == "tfm2d" else bench_invert)(args)
        return

    if args.workload == "io":
        if rank != 0:
            return
        if args.impl == "reference":   # Dataset.save/load need h5py, absent here
            print(json.dumps({"impl": "reference", "unavailable": "the reference's Dataset.save/"
                              "load need h5py, which is not installed on this machine"}))
            return
        bench_io(args)
        return
    if args.workload == "fmc3d":
        if rank != 0:
            return
        prob = problems.cylinder3d(seed=0, nt=args.nt or 2000)
        desc = FMC_WORKLOAD if not args.nt else f"nt={prob.nt} variant of: " + FMC_WORKLOAD
        if args.impl == "reference":
            run_reference(args, prob, desc, "fwd")
            return
        import torch
        torch.cuda.set_device(0)
        bench_fmc(args, prob)
        return

    desc_w, build_prob, C0, k0, mode = WORKLOADS[args.workload]
    if args.workload == "gn3d" and args.nt and not args.n:
        # a shortened time axis (launch lists under ncu)
        prob = problems.gn3d(seed=0, nt=args.nt)
        desc_w = f"nt={prob.nt} variant of: " + desc_w
    elif args.n or args.nt:
        if args.workload != "grad3d":
            raise SystemExit("--n/--nt overrides apply to grad3d (and --nt to gn3d) only")
        n = args.n or 192
        prob = problems.cylinder3d(seed=0, n=n, h=0.2e-3 * 191 / (n - 1), nt=args.nt or 2000)
        desc_w = f"{n}^3 nt={prob.nt} variant of: " + desc_w
    else:
        prob = build_prob()
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, prob, desc_w, mode)
        return

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl")
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # a non-default stream: batch sweeps of launch-bound sizes run as CUDA graphs
    torch.cuda.set_stream(torch.cuda.Stream(device=dev))

    from openusct_gb300 import _lib, backend
    from openusct_gb300.geometry import element_csr
    import ctypes

    C = args.batch or C0
    ckpt = args.ckpt if args.ckpt >= 0 else k0
    # replicas: rank r owns the batch of shots r*C .. r*C+C-1
    shots = [(C * rank + i) % prob.n_shots for i in range(C)]
    tx, rx = element_csr(prob.geom, prob.shape, shots, None)
    bmode_ = _lib.MODE_BORN if mode == "gn" else _lib.MODE_GRADIENT
    if not ckpt:   # the public API's default interval (the same the e2e call below gets)
        ckpt = backend.default_ckpt_k(prob.shape, prob.nt, rx.rows, len(rx.cell), C, bmode_)
    plan = backend.Plan(prob.shape, prob.h, prob.dt, prob.nt, tx, rx, batch=C, ckpt_k=ckpt)
    bmode = _lib.MODE_BORN if mode == "gn" else _lib.MODE_GRADIENT
    lib = _lib.load()
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    m_true = torch.from_numpy(prob.m_true).to(dev)
    m0 = torch.from_numpy(prob.m0).to(dev)
    wav = torch.from_numpy(prob.wavelet).to(dev)
    need = plan.batch_bytes(bmode)
    free = torch.cuda.mem_get_info(dev)[0]
    if need > 0.95 * free:
        raise SystemExit(f"the {C}-shot batch workspace needs {need / 2**30:.0f} GiB even with the "
                         f"smallest checkpoint plan (k = {plan.info('ckpt_k')}); "
                         f"{free / 2**30:.0f} GiB are free: use a smaller --batch")
    mws = torch.empty(plan.model_bytes(), dtype=torch.uint8, device=dev)
    bws = torch.empty(need, dtype=torch.uint8, device=dev)
    dobs = torch.empty((C, prob.nt, plan.n_rx), dtype=torch.float32, device=dev)
    # observed data from the true model (same engine, forward only)
    _lib.check(lib.usct_forward_fmc_dev(plan.handle, P(m_true), None, P(wav), P(dobs), P(mws),
                                        P(bws), sp))
    J = torch.zeros(C, dtype=torch.float64, device=dev)
    g = torch.empty(prob.shape, dtype=torch.float64, device=dev)
    vt = torch.from_numpy(prob.v).to(dev) if mode == "gn" else None
    # the f1 options: GCN misfit and P-arrival windows (fwi.p_window_weights) as
    # time_weights, both through the windowed entry point
    mt = 1 if args.misfit == "gcn" else 0
    tw = None
    if args.windows and mode == "grad":
        from openusct_gb300 import imaging
        tw = imaging.p_window_weights(dobs, prob.dt, prob.f0, as_tensor=True).float().contiguous()
    variant = mode == "grad" and (mt != 0 or tw is not None)
    tw_p = P(tw) if tw is not None else ctypes.c_void_p(0)

    def step():
        if mode == "gn":
            _lib.check(lib.usct_gn_hessian_vector_dev(plan.handle, P(m0), None, P(wav), P(vt),
                                                      P(g), None, P(mws), P(bws), sp))
        elif variant:
            _lib.check(lib.usct_misfit_and_gradient_tw_dev(plan.handle, P(m0), None, P(wav),
                                                           P(dobs), tw_p, mt, P(J), P(g), P(mws),
                                                           P(bws), sp))
        else:
            _lib.check(lib.usct_misfit_and_gradient_dev(plan.handle, P(m0), None, P(wav),
                                                        P(dobs), P(J), P(g), P(mws), P(bws), sp))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    launches0 = plan.info("launches")
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        ev0.record(s)
        for _ in range(args.steps):
            step()
        ev1.record(s)
        torch.cuda.synchronize()
    launches = plan.info("launches") - launches0
    t_ms = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        tt = torch.tensor([t_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
    value = C * world / (t_ms / 1000.0)
    cells = int(np.prod(prob.shape))
    hbm, peak_kind = _peaks()
    pipeline_bytes, rec_lv, tail_lv = schedule_bytes(cells, C, prob.nt, plan.info("ckpt_k"), mode)
    pipeline_model = (("Born forward 24C+8" if mode == "gn" else "forward 12C+4")
                      + f" and adjoint 16C+20 B per cell on all {prob.nt - 1} levels, stash 4C on "
                      f"the {tail_lv} levels of the last segment, recompute 16C+4 on the other "
                      f"{rec_lv} (k = {plan.info('ckpt_k')})")

    # dominant kernel: the forward stencil launch, timed live (forward-only sweep)
    fws = bws
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _lib.check(lib.usct_model_prepare(plan.handle, P(mws), P(m0), None, None, P(wav), sp))
    nrep = 2
    e0.record(s)
    for _ in range(nrep):
        _lib.check(lib.usct_batch_forward(plan.handle, P(mws), P(fws), 0, _lib.MODE_FORWARD,
                                          None, sp))
    e1.record(s)
    torch.cuda.synchronize()
    t_launch = e0.elapsed_time(e1) / 1000.0 / (nrep * (prob.nt - 1))
    fwd_bytes = (12 * C + 4) * cells
    achieved = fwd_bytes / t_launch / 1e9
    # DRAM traffic of the same kernel from the committed ncu capture of a smaller
    # case (128^3, 32 shots: the same template instance), scaled by
    # cell-channels to this launch
    traffic = None
    prof = os.path.join(ROOT, "profiles", "k_forward_tma_128cube_C32.md")
    if os.path.exists(prof):
        try:
            kv = {}
            for line in open(prof):
                if ":" in line and line.split(":")[0] in ("dram_bytes_per_launch", "cell_channels"):
                    kv[line.split(":")[0]] = float(line.split(":")[1])
            traffic = kv["dram_bytes_per_launch"] * (cells * C) / kv["cell_channels"]
        except Exception:
            traffic = None

    # end to end through the public API with host buffers (it allocates its own
    # workspace, so release the timed one first)
    del bws, fws
    torch.cuda.empty_cache()
    e2e = None
    # every rank runs its own batch through the public API (replicas), timed
    # between barriers; the job's rate uses the slowest rank
    m0_h = prob.m0
    dobs_h = dobs.double().cpu().numpy()
    # the public API's own checkpoint interval unless --ckpt names one
    kw = dict(src_list=shots, batch=C, ckpt_k=args.ckpt if args.ckpt > 0 else None)
    tw_h = tw.cpu().numpy() if tw is not None else None
    call = (lambda: backend.gn_hessian_vector(m0_h, prob.geom, prob.wavelet, prob.dt, prob.h,
                                              prob.nt, prob.v, **kw)) if mode == "gn" else \
        (lambda: backend.misfit_and_gradient(m0_h, prob.geom, prob.wavelet, prob.dt, prob.h,
                                             prob.nt, dobs_h, misfit_type=args.misfit,
                                             time_weights=tw_h, **kw)[1])
    call()   # first call builds the plan (and, for small grids, captures graphs)
    ne = 3 if cells * C > (1 << 24) else 5
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ne):
        gh = call()
    te = (time.perf_counter() - t0) / ne
    if world > 1:
        tt = torch.tensor([te], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        te = float(tt.item())
    # the host arrays go up as they are (FP64 data narrowed on the device)
    h2d = m0_h.nbytes + prob.wavelet.nbytes + (prob.v.nbytes if mode == "gn" else
                                                dobs_h.nbytes)
    if tw_h is not None:
        h2d += tw_h.nbytes
    e2e = {"value": C * world / te, "unit": "shots/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(gh.nbytes + (0 if mode == "gn" else 8 * C)),
           "api": "openusct_gb300.backend." + ("gn_hessian_vector" if mode == "gn"
                                               else "misfit_and_gradient")}
    backend.release()

    # plain one-shot-per-launch GPU form, same workload, one shot
    plain = None
    no_plain = args.no_plain or variant   # the plain form is the reference's L2 GPU path
    if rank == 0 and not no_plain and mode == "grad":
        backend._PLANS.clear()
        torch.cuda.empty_cache()
        tx1, rx1 = element_csr(prob.geom, prob.shape, [0], None)
        pplan = backend.Plan(prob.shape, prob.h, prob.dt, prob.nt, tx1, rx1, batch=1)
        need = pplan.plain_bytes(True)
        free = torch.cuda.mem_get_info(dev)[0]
    if rank == 0 and not no_plain and mode == "grad" and need > 0.95 * free:
        plain = {"value": None, "unit": "shots/s",
                 "infeasible": f"the plain form keeps the full FP32 history: {need / 2**30:.0f} GiB "
                               f"> {free / 2**30:.0f} GiB free HBM"}
    elif rank == 0 and not no_plain and mode == "grad":
        pws = torch.empty(pplan.plain_bytes(True), dtype=torch.uint8, device=dev)
        J1 = torch.zeros(1, dtype=torch.float64, device=dev)
        d1 = dobs[0:1].contiguous()
        args_p = (pplan.handle, P(m0), P(wav), P(d1), P(J1), P(g), P(pws), sp)
        _lib.check(lib.usct_plain_misfit_and_gradient_dev(*args_p))
        torch.cuda.synchronize()
        times = []
        for _ in range(3):   # the median of three timed calls
            e0.record(s)
            _lib.check(lib.usct_plain_misfit_and_gradient_dev(*args_p))
            e1.record(s)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
        tp = statistics.median(times)
        plain = {"value": 1.0 / tp, "unit": "shots/s", "ms_per_shot": tp * 1000.0,
                 "ms_per_shot_runs": [t * 1000.0 for t in times],
                 "speedup_batched_vs_plain": value / world / (1.0 / tp)}
        del pws

    gn = None
    if rank == 0 and not args.no_serve and args.workload == "grad3d" and not variant:
        try:
            gn = gauss_newton_phase(args)
        except Exception as exc:   # reported, never fatal for the main line
            gn = {"error": f"{type(exc).__name__}: {exc}"[:300]}

    serve = None
    if rank == 0 and not args.no_serve and args.workload == "grad3d" and not variant:
        try:
            serve = serve_phase(args)
        except Exception as exc:   # reported, never fatal for the main line
            serve = {"error": f"{type(exc).__name__}: {exc}"[:300]}

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            import oracle
            oracle.build()
            # the same procedure as the reference arm: one whole shot, timed
            kc, mem = cpu_shot_interval(prob, mode)
            d1 = dobs[0:1].double().cpu().numpy() if mode != "gn" else None
            secs, desc = cpu_whole_shot(prob, shots[0], kc, d1, mode, args.misfit)
            v = 1.0 / secs
            if tw is not None:
                desc += "; without the data windows (an elementwise product of the residual)"
            cpu = {"value": v, "unit": "shots/s",
                   "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                   "kind": "port", "sample": desc, "seconds": secs, "host_bytes": mem}
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "error": str(exc)[:200]}

    if rank == 0:
        level_bytes = 4 * cells * C
        l2_note = ("inputs larger than L2 (no flush needed)" if 3 * level_bytes > 129e6 else
                   f"one sweep's three wavefield levels ({3 * level_bytes / 1e6:.0f} MB) fit in "
                   "L2: the stencils run from L2 and the DRAM roofline fraction understates them")
        line = {
            "metric": METRIC if mode == "grad" else "Gauss-Newton Hv shots/s (Born + adjoint)",
            "value": value, "unit": "shots/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian random-field model)",
            "config": {"workload": desc_w,
                       "grid": list(prob.shape), "nt": prob.nt, "batch_shots": C,
                       "ckpt_k": plan.info("ckpt_k"), "tile": [plan.info("tile_x"),
                                                              plan.info("tile_y"),
                                                              plan.info("zchunk")],
                       "parallelism": f"replicas{world}" if world > 1 else "single",
                       "misfit": args.misfit if mode == "grad" else None,
                       "time_weights": ("P-arrival windows (imaging.p_window_weights)"
                                        if tw is not None else None),
                       "l2": l2_note},
            "grid_updates_per_s": value * cells * (prob.nt - 1),
            "roofline": {"bound": "hbm",
                         "kernel": f"k_forward_tma ({len(prob.shape)}D, {C} shots per launch)",
                         "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind,
                         "traffic": traffic,
                         "traffic_source": "profiles/k_forward_tma_128cube_C32.md, scaled by "
                                           "cell-channels (128^3x32 -> this launch)",
                         "algorithmic_bytes_per_launch": fwd_bytes,
                         "launch_ms": t_launch * 1000.0},
            "pipeline_roofline": {"bytes_per_step": pipeline_bytes,
                                  "achieved": pipeline_bytes / (t_ms / 1000.0) / 1e9,
                                  "frac": pipeline_bytes / (t_ms / 1000.0) / 1e9 / hbm,
                                  "model": pipeline_model},
            "e2e": e2e, "plain": plain, "serve": serve, "gauss_newton": gn, "cpu_baseline": cpu,
            "gpu_launches": launches, "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
