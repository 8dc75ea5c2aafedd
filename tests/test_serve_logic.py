"""The serving loop's host logic on the CPU, with the device replaced by a
stand-in context that takes a little wall time per step: admission by
device-memory footprint (one at a time when the budget holds one request,
overlapping when it holds several), FIFO order, small compatible requests
grouped into one batch slot, and a failing slot reported on its requests
while the loop goes on."""
import threading
import time

import pytest

from rheotool_gb300 import serve
from rheotool_gb300.case import Fields, cavity_case
from rheotool_gb300.mesh import cavity_mesh


class _Stand:
    lock = threading.Lock()
    active = 0
    peak = 0
    order = []
    batches = []
    carried = []
    steps = {}
    fail_cells = None


class FakeContext:
    def __init__(self, device=0):
        self.case = None
        self.batch_cases = None
        with _Stand.lock:
            _Stand.active += 1
            _Stand.peak = max(_Stand.peak, _Stand.active)

    def setup_case(self, case, fields=None):
        if _Stand.fail_cells is not None and case.mesh.nCells == _Stand.fail_cells:
            raise RuntimeError("stand-in failure")
        self.case = case
        with _Stand.lock:
            _Stand.order.append(case.name)

    def step(self, n):
        time.sleep(0.002 * n)
        with _Stand.lock:
            for c in (self.batch_cases or [self.case]):
                _Stand.steps[id(c)] = _Stand.steps.get(id(c), 0) + n

    def sync(self):
        pass

    def fields(self):
        return Fields.zeros(self.case.mesh)

    def close(self):
        with _Stand.lock:
            _Stand.active -= 1


class FakeBatch:
    def __init__(self, cases, ctx=None):
        self.cases = cases
        ctx.batch_cases = list(cases)
        with _Stand.lock:
            _Stand.batches.append(len(cases))
            _Stand.order.extend(c.name for c in cases)

    def set_case_fields(self, states):
        with _Stand.lock:
            _Stand.carried.extend(states)

    def fields(self):
        return [Fields.zeros(c.mesh) for c in self.cases]


@pytest.fixture
def stand(monkeypatch):
    monkeypatch.setattr(serve, "Context", FakeContext)
    monkeypatch.setattr(serve, "BatchContext", FakeBatch)
    monkeypatch.setattr(serve, "device_bytes", lambda: 0)
    _Stand.active = _Stand.peak = 0
    _Stand.order, _Stand.batches, _Stand.carried, _Stand.fail_cells = [], [], [], None
    _Stand.steps = {}
    return _Stand


def _cases(k, n=8):
    m = cavity_mesh(n)
    out = []
    for i in range(k):
        c = cavity_case(n, mesh=m)
        c.name = f"r{i}"
        out.append(c)
    return out


def _serve(cases, steps, **kw):
    srv = serve.Server(**kw)
    reqs = [srv.submit(c, steps) for c in cases]
    for r in reqs:
        assert r.done.wait(30)
    srv.close()
    return reqs


def test_budget_for_one_request_serialises(stand):
    cases = _cases(5)
    fp = int(1000.0 * cases[0].mesh.nCells) + 1000
    reqs = _serve(cases, 5, slots=3, hbm_budget=fp, batch_cells=0, bytes_per_cell=1000.0, slot_bytes=1000,
                  quantum=2)
    assert stand.peak == 1
    assert stand.order == [c.name for c in cases]          # FIFO
    assert all(r.error is None and r.fields is not None for r in reqs)
    assert all(r.admitted >= r.arrival and r.finished >= r.admitted for r in reqs)


def test_budget_for_several_requests_overlaps(stand):
    cases = _cases(6)
    reqs = _serve(cases, 20, slots=3, hbm_budget=1 << 40, batch_cells=0, quantum=2)
    assert stand.peak >= 2
    assert all(r.error is None for r in reqs)


def test_small_compatible_requests_are_batched(stand):
    cases = _cases(6)
    # the loop admits the whole waiting group at once: submit before it looks
    srv = serve.Server(slots=1, hbm_budget=1 << 40, batch_cells=10 ** 6, batch_max=4, quantum=5)
    reqs = [srv.submit(c, 10) for c in cases]
    for r in reqs:
        assert r.done.wait(30)
    srv.close()
    assert max(stand.batches, default=1) <= 4
    assert any(b > 1 for b in stand.batches)
    assert all(r.error is None and r.fields is not None for r in reqs)


def test_failing_slot_reports_and_loop_continues(stand):
    cases = _cases(2) + [cavity_case(6)]
    stand.fail_cells = cases[-1].mesh.nCells
    reqs = _serve(cases, 3, slots=2, hbm_budget=1 << 40, batch_cells=0)
    assert reqs[-1].error is not None and "stand-in failure" in reqs[-1].error
    assert all(r.error is None for r in reqs[:2])


def test_requests_join_and_leave_a_running_batch(stand):
    """Continuous batching: requests that arrive while a batch runs join it at
    a quantum boundary (a new layout carrying the running cases' fields), and
    a request leaves as soon as its own steps are done, whatever the others'."""
    cases = _cases(6)
    srv = serve.Server(slots=1, hbm_budget=1 << 40, batch_cells=10 ** 6, batch_max=8, quantum=2)
    first = [srv.submit(cases[0], 40), srv.submit(cases[1], 4)]
    time.sleep(0.05)                        # the first two are running
    later = [srv.submit(c, 6) for c in cases[2:]]
    reqs = first + later
    for r in reqs:
        assert r.done.wait(30)
    srv.close()
    assert all(r.error is None and r.fields is not None for r in reqs)
    assert any(r.joined for r in later)                 # joined a running batch
    for r in reqs:                                      # every request took exactly its steps
        assert stand.steps[id(r.case)] == r.steps, (r.rid, stand.steps[id(r.case)], r.steps)
    assert srv.relayouts >= 1 and stand.carried          # running cases carried into the new layout
    assert first[1].finished < first[0].finished        # the short request left first
    assert len(stand.batches) >= 2


def test_measured_footprint_sizes_admission(stand, monkeypatch):
    """After the first admission the prediction is the measured bytes per
    cell, not the default."""
    calls = iter(range(0, 10 ** 9, 64 * 1000))
    monkeypatch.setattr(serve, "device_bytes", lambda: next(calls))
    cases = _cases(2)
    srv = serve.Server(slots=1, hbm_budget=1 << 40, batch_cells=0, bytes_per_cell=1e6, quantum=2)
    for r in [srv.submit(c, 2) for c in cases]:
        assert r.done.wait(30)
    srv.close()
    assert srv.measured and srv.bytes_per_cell != 1e6
