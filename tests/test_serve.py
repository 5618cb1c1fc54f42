"""Serving scheduler logic on the CPU (a fake executor stands in for the GPU)."""

import threading
import time

import numpy as np
import pytest

from openusct_gb300.serve import Engine, Request, percentile, summarize


class FakePlan:
    def __init__(self, fp, dur, fail=False):
        self.fp, self.dur, self.fail = fp, dur, fail


class FakeExecutor:
    """Footprint and run time come from the request's ``m`` (a 3-vector)."""

    def __init__(self):
        self.lock = threading.Lock()
        self.running = 0
        self.peak = 0
        self.released = 0

    def plan_for(self, req):
        fp, dur, fail = req.m
        if fp < 0:
            raise ValueError("bad request")
        return FakePlan(int(fp), float(dur), bool(fail))

    def footprint(self, req, plan):
        return plan.fp

    def run(self, req, plan):
        with self.lock:
            self.running += 1
            self.peak = max(self.peak, self.running)
        time.sleep(plan.dur)
        with self.lock:
            self.running -= 1
        if plan.fail:
            raise RuntimeError("injected device failure")
        return {"J": float(plan.fp)}

    def release(self, plan):
        with self.lock:
            self.released += 1


def req(fp, dur, arrival=0.0, fail=False):
    return Request(kind="gradient", m=(fp, dur, fail), geom=type("G", (), {"idx": [0, 1]})(),
                   wavelet=None, dt=1.0, h=1.0, nt=2, arrival=arrival)


def test_admission_never_exceeds_the_budget_and_requests_overlap():
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=8)
    rs = eng.run_stream([req(40, 0.15, 0.0), req(40, 0.15, 0.01), req(40, 0.15, 0.02),
                         req(30, 0.05, 0.03)])
    assert all(r.ok for r in rs)
    assert eng.peak_reserved <= 100
    assert eng.max_concurrent >= 2 and ex.peak >= 2
    assert ex.released == 4


def test_request_larger_than_budget_is_rejected_immediately():
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=2)
    rs = eng.run_stream([req(500, 0.01, 0.0), req(50, 0.01, 0.0)])
    assert not rs[0].ok and rs[0].error.startswith("rejected")
    assert rs[0].latency < 0.05
    assert rs[1].ok


def test_smaller_request_passes_a_blocked_head():
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=4)
    # a long 60-byte job runs; a 60-byte head must wait; a 30-byte one can go ahead
    rs = eng.run_stream([req(60, 0.3, 0.0), req(60, 0.05, 0.02), req(30, 0.05, 0.04)])
    assert all(r.ok for r in rs)
    assert rs[2].t_admit < rs[1].t_admit


def test_requests_held_back_by_the_budget_are_counted():
    """A request that finds a free slot but not enough budget waits and is
    counted as held back by the budget; one that waits for a slot is not."""
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=2)
    rs = eng.run_stream([req(60, 0.2, 0.0), req(60, 0.02, 0.01)])
    assert all(r.ok for r in rs)
    assert not rs[0].waited_for_budget and rs[1].waited_for_budget
    assert summarize(rs, eng).waited_for_budget == 1
    ex2 = FakeExecutor()
    eng2 = Engine(ex2, budget_bytes=10 ** 9, max_active=1)
    rs2 = eng2.run_stream([req(1, 0.1, 0.0), req(1, 0.01, 0.01)])
    assert not any(r.waited_for_budget for r in rs2)
    assert rs2[1].record()["waited_for_budget"] is False


def test_a_failing_request_does_not_stop_the_service():
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=2)
    rs = eng.run_stream([req(10, 0.02, 0.0, fail=True), req(10, 0.02, 0.0), req(-1, 0.0, 0.0)])
    assert not rs[0].ok and "injected" in rs[0].error
    assert rs[1].ok
    assert not rs[2].ok and "bad request" in rs[2].error
    assert eng.reserved == 0 and eng.active == 0


def test_slots_cap_concurrency():
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=10 ** 9, max_active=2)
    eng.run_stream([req(1, 0.05, 0.0) for _ in range(6)])
    assert ex.peak <= 2


def test_percentiles_and_summary():
    assert percentile([1, 2, 3, 4], 50) == pytest.approx(2.5)
    assert percentile(list(range(101)), 99) == pytest.approx(99.0)
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=4)
    rs = eng.run_stream([req(10, 0.02, 0.01 * i) for i in range(8)])
    st = summarize(rs, eng)
    assert st.ok == 8 and st.shots == 16
    assert st.p50_s <= st.p99_s
    assert st.shots_per_s > 0


class SteppingExecutor(FakeExecutor):
    """Runs in ten steps and honours cancellation between them, like the GPU
    executor between shot batches."""

    def __init__(self):
        super().__init__()
        self.steps_run = {}

    def run(self, req, plan):
        from openusct_gb300.serve import Cancelled
        for k in range(10):
            if req.cancelled.is_set():
                raise Cancelled(f"cancelled after {k} of 10 steps")
            time.sleep(plan.dur / 10)
            self.steps_run[req.rid] = k + 1
        return {"J": float(plan.fp)}


def test_cancelled_while_queued_is_never_run():
    ex = SteppingExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=4)
    a, b, c = req(80, 0.3, 0.0), req(80, 0.05, 0.01), req(10, 0.05, 0.02)
    threading.Timer(0.1, b.cancel).start()          # b waits behind a for the budget
    rs = eng.run_stream([a, b, c])
    assert rs[0].ok and rs[2].ok
    assert not rs[1].ok and rs[1].error.startswith("Cancelled")
    assert 1 not in ex.steps_run
    assert ex.released == 3 and eng.reserved == 0


def test_cancelled_while_running_stops_and_frees_its_budget():
    ex = SteppingExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=4)
    a, b = req(90, 2.0, 0.0), req(90, 0.05, 0.01)
    threading.Timer(0.3, a.cancel).start()
    t0 = time.perf_counter()
    rs = eng.run_stream([a, b])
    assert time.perf_counter() - t0 < 1.5           # a did not run its 2 s
    assert not rs[0].ok and rs[0].error.startswith("Cancelled")
    assert 0 < ex.steps_run.get(0, 0) < 10
    assert rs[1].ok and rs[1].t_admit >= rs[0].t_done - 1e-3   # b got a's budget afterwards
    assert eng.reserved == 0 and eng.active == 0


def test_per_request_records(tmp_path):
    import json
    from openusct_gb300.serve import write_records
    ex = FakeExecutor()
    eng = Engine(ex, budget_bytes=100, max_active=2)
    rs = eng.run_stream([req(40, 0.05, 0.0), req(500, 0.05, 0.0), req(40, 0.05, 0.01)])
    path = tmp_path / "requests.jsonl"
    write_records(rs, path)
    recs = [json.loads(line) for line in path.read_text().splitlines()]
    assert [r["rid"] for r in recs] == [0, 1, 2]
    assert recs[0]["ok"] and recs[0]["latency_s"] > 0 and recs[0]["device_bytes"] == 40
    assert not recs[1]["ok"] and recs[1]["error"].startswith("rejected")
    assert recs[1]["latency_s"] is None
    assert all(r["queue_s"] >= 0 for r in recs)


class MergingExecutor(FakeExecutor):
    """Forward requests tagged alike (``m[3]``) may share launches."""

    merge_width = 32

    def __init__(self):
        super().__init__()
        self.groups = []

    def merge_key(self, req):
        return req.m[3] if req.kind == "forward" and len(req.m) > 3 else None

    def plan_for(self, req):
        fp, dur, fail = req.m[:3]
        return FakePlan(int(fp), float(dur), bool(fail))

    def plan_for_group(self, reqs):
        return FakePlan(sum(int(q.m[0]) for q in reqs), max(float(q.m[1]) for q in reqs))

    def footprint_group(self, reqs, plan):
        return plan.fp

    def run_group(self, reqs, plan):
        self.groups.append([q.rid for q in reqs])
        time.sleep(plan.dur)
        return [{"traces": np.full(2, q.rid)} for q in reqs]


def fwd(fp, dur, arrival, tag, shots=2):
    r = Request(kind="forward", m=(fp, dur, False, tag),
                geom=type("G", (), {"idx": list(range(shots))})(), wavelet=None, dt=1.0, h=1.0,
                nt=2, arrival=arrival)
    return r


def test_waiting_compatible_forward_requests_share_one_launch_group():
    """While a long request holds the only slot, three compatible forward
    requests and one of another grid queue; when the slot frees, the first
    admitted takes the other compatible one that fits one batch of shots into
    its group, each gets its own result, and the other grid runs alone."""
    ex = MergingExecutor()
    eng = Engine(ex, budget_bytes=1000, max_active=1)
    rs = eng.run_stream([req(10, 0.2, 0.0), fwd(10, 0.02, 0.01, "a"), fwd(10, 0.02, 0.02, "a"),
                         fwd(10, 0.02, 0.03, "b"), fwd(10, 0.02, 0.04, "a", shots=40)])
    assert all(r.ok for r in rs)
    assert ex.groups == [[1, 2]]
    assert rs[1].group == 2 and rs[2].group == 2 and rs[3].group == 1 and rs[4].group == 1
    assert list(rs[1].traces) == [1, 1] and list(rs[2].traces) == [2, 2]
    assert summarize(rs, eng).merged == 2
    assert eng.reserved == 0 and eng.active == 0


def test_concatenated_element_lists():
    from openusct_gb300.geometry import element_csr
    from openusct_gb300.serve import _concat_csr
    a = element_csr([(1, 2), (3, 4), (5, 6)], (8, 8), [0, 2])
    b = element_csr([(7, 7), (0, 1)], (8, 8), [1])
    tx = _concat_csr([a[0], b[0]])
    rx = _concat_csr([a[1], b[1]])
    assert list(tx.ptr) == [0, 1, 2, 3] and list(tx.cell) == [1 * 8 + 2, 5 * 8 + 6, 0 * 8 + 1]
    assert list(rx.ptr) == [0, 1, 2, 3, 4, 5] and rx.rows == 5 and len(rx.w) == 5


def test_padded_transmit_rows_and_group_quantum():
    from openusct_gb300.geometry import element_csr
    from openusct_gb300.serve import _pad_rows
    tx = element_csr([(1, 2), (3, 4), (5, 6)], (8, 8), [0, 2, 1, 0, 2])[0]
    p = _pad_rows(tx, 4)
    assert p.rows == 8 and list(p.ptr) == [0, 1, 2, 3, 4, 5, 5, 5, 5]
    assert np.array_equal(p.cell, tx.cell) and _pad_rows(p, 4) is p
    # with a quantum of 4, requests of 5 shots take 8 channels: 4 of them fill 32
    ex = MergingExecutor()
    ex.merge_quantum = 4
    eng = Engine(ex, budget_bytes=10 ** 6, max_active=1)
    reqs = [fwd(10, 0.05, 0.0, "a", shots=5) for _ in range(6)]
    rs = eng.run_stream(reqs, realtime=False)
    assert all(r.ok for r in rs)
    assert max(len(g) for g in ex.groups) == 4


def test_receiver_union_keeps_each_distinct_row_once():
    from openusct_gb300.geometry import element_csr
    from openusct_gb300.serve import _union_rows
    g1 = [(1, 2), (3, 4), (5, 6)]
    g2 = [(5, 6), (7, 7)]
    r1 = element_csr(g1, (8, 8), [0])[1]
    r2 = element_csr(g1, (8, 8), [2])[1]      # the same elements: the same receivers
    r3 = element_csr(g2, (8, 8), [0])[1]      # shares one element with g1
    u, idx = _union_rows([r1, r2, r3])
    assert u.rows == 4
    assert [list(i) for i in idx] == [[0, 1, 2], [0, 1, 2], [2, 3]]
    for r, ix in zip((r1, r2, r3), idx):
        for j, k in enumerate(ix):
            assert list(u.cell[u.ptr[k]:u.ptr[k + 1]]) == list(r.cell[r.ptr[j]:r.ptr[j + 1]])
            assert list(u.w[u.ptr[k]:u.ptr[k + 1]]) == list(r.w[r.ptr[j]:r.ptr[j + 1]])


def test_requests_are_grouped_only_when_they_outnumber_the_free_slots():
    ex = MergingExecutor()
    eng = Engine(ex, budget_bytes=10 ** 6, max_active=4)
    rs = eng.run_stream([fwd(10, 0.05, 0.0, "a") for _ in range(3)], realtime=False)
    assert all(r.ok and r.group == 1 for r in rs) and ex.groups == []
    ex = MergingExecutor()
    eng = Engine(ex, budget_bytes=10 ** 6, max_active=4)
    rs = eng.run_stream([fwd(10, 0.05, 0.0, "a") for _ in range(10)], realtime=False)
    assert all(r.ok for r in rs)
    # 10 waiting for 4 slots: groups of ceil(10/4) = 3, then ceil(7/3) = 3,
    # ceil(4/2) = 2 and ceil(2/1) = 2 -- every request admitted at once
    assert sorted(len(g) for g in ex.groups) == [2, 2, 3, 3]
    assert eng.max_concurrent == 4


def test_launch_group_layout_pads_requests_to_whole_quads(monkeypatch):
    """plan_for_group on the host: each request's transmits start on a group
    of four channels (padded with transmits that inject nothing), the owner
    map names one model per group, and each request's traces are cut from
    its own first transmit and its receivers' columns of the union."""
    import openusct_gb300.backend as gb
    from openusct_gb300.geometry import IndexGeometry
    from openusct_gb300.serve import GpuExecutor, Request
    seen = {}

    class FakeLib:
        @staticmethod
        def usct_plan_set_channel_models(handle, n, owner_ptr):
            seen["models"] = (n, np.ctypeslib.as_array(owner_ptr, shape=(seen["tx"].rows,)).copy())
            return 0

    class FakePlan:
        _lib = FakeLib()
        handle = None

        def __init__(self, shape, h, dt, nt, tx, rx, batch=None):
            seen["tx"], seen["rx"], seen["batch"] = tx, rx, batch

        def set(self, *a):
            pass

    monkeypatch.setattr(gb, "Plan", FakePlan)
    ex = GpuExecutor.__new__(GpuExecutor)
    ex.graphs = False
    geom = IndexGeometry([(1, 1), (1, 6), (6, 1), (6, 6), (3, 4), (4, 3)])
    other = IndexGeometry([(1, 1), (2, 5)])           # shares one element with geom
    m = np.ones((8, 8))
    reqs = [Request(kind="forward", m=m, geom=g, wavelet=np.zeros(4), dt=1.0, h=1.0, nt=4,
                    src_list=sl) for g, sl in ((geom, [0, 1, 2, 3, 4]), (other, [0, 1]),
                                               (geom, [5, 4, 3]))]
    plan = ex.plan_for_group(reqs)
    tx = seen["tx"]
    assert tx.rows == 8 + 4 + 4 and seen["batch"] == 32
    n, owner = seen["models"]
    assert n == 3 and list(owner) == [0] * 8 + [1] * 4 + [2] * 4
    assert all(owner[t] == owner[t & ~3] for t in range(tx.rows))
    assert [p[:2] for p in plan.group_parts] == [(0, 5), (8, 2), (12, 3)]
    rows = np.diff(tx.ptr)
    assert list(rows) == [1] * 5 + [0] * 3 + [1] * 2 + [0] * 2 + [1] * 3 + [0]
    assert seen["rx"].rows == 7                        # 6 + 1 new receiver
    assert list(plan.group_parts[0][2]) == [0, 1, 2, 3, 4, 5]
    assert list(plan.group_parts[1][2]) == [0, 6]
    assert list(plan.group_parts[2][2]) == [0, 1, 2, 3, 4, 5]
