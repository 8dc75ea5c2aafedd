"""Serving form: a request loop with continuous batching of independent cases.

Requests (a case and a number of time steps) arrive at any time.  The loop
keeps a set of slots, each driven by its own worker thread on its own CUDA
stream.  A large request runs in a slot of its own; small compatible requests
share a batch slot (one device mesh, every stage of the step one launch for
all of them).  A batch slot steps its cases in quanta of a few steps and, at
every quantum boundary, retires the requests that have taken all their steps
(their fields go back to the client) and admits waiting compatible requests
into the running batch: the batch is laid out again with the new membership
and the running cases carry their fields into it, so a request joins while
others are mid-flight and leaves as soon as it is done, whatever their step
counts.  A request is admitted when a slot (or a running batch) has room and
its predicted device-memory footprint fits what the budget leaves after the
requests already on the device; the prediction is bytes per cell times cells
plus a per-slot part, the bytes per cell being the mean of what the library's
allocation counter measured at the earlier admissions (a default before the
first).  Fields stay on the device between steps, and a case gives the same
result alone as in the mix: a slot is an independent context, a batch solves
every case with its own Krylov scalars and stopping points, and a relayout
carries each running case's fields unchanged.

No reference counterpart: rheoFoam runs one case per process.
"""
from __future__ import annotations

import ctypes as C
import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import abi
from .batch import BatchContext
from .case import Case, Fields
from .runtime import Context


def device_bytes() -> int:
    lib = abi.load_library()
    v = C.c_int64()
    st = lib.rt_device_bytes(C.byref(v))
    if st != abi.RT_OK:
        raise RuntimeError("rt_device_bytes failed")
    return int(v.value)


@dataclass
class Request:
    case: Case
    steps: int
    rid: int = 0
    arrival: float = 0.0
    admitted: float = 0.0
    finished: float = 0.0
    fields: Optional[Fields] = None
    error: Optional[str] = None
    joined: bool = False          # admitted into a batch that was already running
    done: threading.Event = field(default_factory=threading.Event)

    @property
    def time_to_solution(self) -> float:
        return self.finished - self.arrival


class Server:
    """Continuous-batching request loop.

    slots: concurrent slots (worker threads, CUDA streams);
    hbm_budget: device bytes the admitted cases may hold (default: 90 % of
    the free device memory at start);
    batch_cells: requests of at most this many cells share batch slots, up to
    batch_max requests in one;
    quantum: steps a slot takes between two looks at its requests;
    bytes_per_cell: the footprint prediction before any admission has been
    measured."""

    def __init__(self, slots: int = 4, hbm_budget: Optional[int] = None, batch_cells: int = 40000,
                 batch_max: int = 16, quantum: int = 10, device: int = 0, bytes_per_cell: float = 4000.0,
                 slot_bytes: int = 16 << 20):
        self.slots = slots
        self.batch_cells = batch_cells
        self.batch_max = batch_max
        self.quantum = quantum
        self.device = device
        if hbm_budget is None:
            import torch  # noqa: F401  (only to query free memory when available)
            free, _ = torch.cuda.mem_get_info(device)
            hbm_budget = int(0.9 * free)
        self.budget = hbm_budget - device_bytes()   # what the admitted cases may add
        self.default_bytes_per_cell = bytes_per_cell
        self.slot_bytes = slot_bytes
        self.measured: List[float] = []              # bytes per cell of each layout
        self.pending: "queue.Queue[Request]" = queue.Queue()
        self._waiting: List[Request] = []
        self._lock = threading.Lock()
        self._reserved = 0
        self._stop = False
        self._workers = [threading.Thread(target=self._worker, daemon=True) for _ in range(slots)]
        self._next = 0
        self.finished: List[Request] = []
        self.relayouts = 0                           # batch layouts rebuilt for joins and departures
        for w in self._workers:
            w.start()

    # ---- client side ---------------------------------------------------------
    def submit(self, case: Case, steps: int) -> Request:
        r = Request(case=case, steps=steps, rid=self._next, arrival=time.perf_counter())
        self._next += 1
        self.pending.put(r)
        return r

    def close(self, wait: bool = True):
        if wait:
            while True:
                with self._lock:
                    busy = self._reserved > 0 or self._waiting or not self.pending.empty()
                if not busy:
                    break
                time.sleep(0.01)
        self._stop = True
        for w in self._workers:
            w.join()

    # ---- admission ---------------------------------------------------------
    @property
    def bytes_per_cell(self) -> float:
        """The footprint per cell: the mean measured so far, else the default."""
        with self._lock:
            return float(np.mean(self.measured)) if self.measured else self.default_bytes_per_cell

    def _cells_bytes(self, cells: int) -> int:
        return int((float(np.mean(self.measured)) if self.measured else self.default_bytes_per_cell) * cells)

    def _drain(self):
        while not self.pending.empty():
            self._waiting.append(self.pending.get_nowait())

    def _take(self) -> Optional[List]:
        """The next group to admit into a new slot (FIFO; small compatible
        requests grouped) with its reservation as the last item, or None."""
        with self._lock:
            self._drain()
            if not self._waiting:
                return None
            head = self._waiting[0]
            group = [head]
            if head.case.mesh.nCells <= self.batch_cells:
                for r in self._waiting[1:]:
                    if len(group) >= self.batch_max:
                        break
                    if r.case.mesh.nCells <= self.batch_cells and self._batchable(head.case, r.case):
                        group.append(r)
            shares = {r.rid: self._cells_bytes(r.case.mesh.nCells) for r in group}
            need = sum(shares.values()) + self.slot_bytes
            if self._reserved + need > self.budget:
                if len(group) > 1:
                    group = [head]
                    shares = {head.rid: shares[head.rid]}
                    need = shares[head.rid] + self.slot_bytes
                if self._reserved + need > self.budget:
                    return None
            for r in group:
                self._waiting.remove(r)
            self._reserved += need
            now = time.perf_counter()
            for r in group:
                r.admitted = now
            return [group, shares, need]

    def _join(self, like: Case, room: int) -> List:
        """Waiting requests compatible with a running batch (up to `room`),
        each with its reservation: [(request, bytes), ...]."""
        out = []
        if room <= 0:
            return out
        with self._lock:
            self._drain()
            for r in list(self._waiting):
                if len(out) >= room:
                    break
                if r.case.mesh.nCells > self.batch_cells or not self._batchable(like, r.case):
                    continue
                need = self._cells_bytes(r.case.mesh.nCells)
                if self._reserved + need > self.budget:
                    break                     # first come first served: no overtaking past the budget
                self._waiting.remove(r)
                self._reserved += need
                r.admitted = time.perf_counter()
                r.joined = True
                out.append((r, need))
        return out

    def _release(self, nbytes: int):
        with self._lock:
            self._reserved -= nbytes

    @staticmethod
    def _batchable(a: Case, b: Case) -> bool:
        return all(getattr(a, k) == getattr(b, k) for k in ("deltaT", "divU", "divTheta", "solverU", "solverP",
                                                            "solverTheta", "precision", "ddt")) and \
            np.array_equal(a.mesh.solveDir, b.mesh.solveDir) and len(a.models) == 1 and len(b.models) == 1

    # ---- slots ---------------------------------------------------------------
    def _worker(self):
        while not self._stop:
            got = self._take()
            if got is None:
                time.sleep(0.002)
                continue
            group, shares, need = got
            held = {"bytes": need}
            try:
                if len(group) == 1 and group[0].case.mesh.nCells > self.batch_cells:
                    self._run_solo(group[0])
                else:
                    self._run_batch(group, held, shares)
            except Exception as e:   # the slot's requests fail, the loop goes on
                for r in group:
                    if not r.done.is_set():
                        r.error = f"{type(e).__name__}: {e}"
                        r.finished = time.perf_counter()
                        r.done.set()
            finally:
                self._release(held["bytes"])

    def _finish(self, reqs: List[Request], fields: List[Fields]):
        now = time.perf_counter()
        for r, f in zip(reqs, fields):
            r.fields = f
            r.finished = now
            r.done.set()
        with self._lock:
            self.finished.extend(reqs)

    def _run_solo(self, r: Request):
        """A large request in a slot of its own (its own context)."""
        ctx = None
        try:
            before = device_bytes()
            ctx = Context(self.device)
            ctx.setup_case(r.case)
            used = device_bytes() - before    # (other slots may allocate meanwhile: an upper bound)
            if used > 0:
                with self._lock:
                    self.measured.append(used / r.case.mesh.nCells)
            done = 0
            while done < r.steps:
                n = min(self.quantum, r.steps - done)
                ctx.step(n)
                done += n
            ctx.sync()
            self._finish([r], [ctx.fields()])
        finally:
            if ctx is not None:
                ctx.close()

    def _run_batch(self, group: List[Request], held: Dict[str, int], shares: Dict[int, int]):
        """A batch slot: step the running requests in quanta; at every
        quantum boundary retire the finished ones and admit waiting compatible
        ones into the running batch (a new layout that carries the running
        cases' fields)."""
        running = list(group)
        done = {r.rid: 0 for r in running}
        states: Dict[int, Fields] = {}       # rid -> fields carried into the next layout
        ctx = slot = None
        try:
            while running:
                if slot is None:
                    if ctx is not None:
                        ctx.close()
                    before = device_bytes()
                    ctx = Context(self.device)
                    slot = BatchContext([r.case for r in running], ctx=ctx)
                    slot.set_case_fields({i: states[r.rid] for i, r in enumerate(running) if r.rid in states})
                    states.clear()
                    used = device_bytes() - before
                    if used > 0:
                        with self._lock:
                            self.measured.append(used / sum(r.case.mesh.nCells for r in running))
                q = min([self.quantum] + [r.steps - done[r.rid] for r in running])
                ctx.step(q)
                for r in running:
                    done[r.rid] += q
                leaving = [r for r in running if done[r.rid] >= r.steps]
                staying = [r for r in running if done[r.rid] < r.steps]
                joiners = self._join(running[0].case, self.batch_max - len(staying))
                if not leaving and not joiners:
                    continue
                ctx.sync()
                per_case = slot.fields()
                fin = []
                for r, f in zip(running, per_case):
                    if r in leaving:
                        fin.append((r, f.copy()))
                    else:
                        states[r.rid] = f.copy()
                self._finish([r for r, _ in fin], [f for _, f in fin])
                for r, _ in fin:                      # a finished request's share of the reservation
                    nb = shares.pop(r.rid)
                    held["bytes"] -= nb
                    self._release(nb)
                for r, nb in joiners:
                    shares[r.rid] = nb
                    held["bytes"] += nb
                    done[r.rid] = 0
                running = staying + [r for r, _ in joiners]
                slot = None
                if running:
                    with self._lock:
                        self.relayouts += 1
        finally:
            if ctx is not None:
                ctx.close()


def percentile(xs: List[float], q: float) -> float:
    return float(np.percentile(np.asarray(xs), q)) if xs else float("nan")


def poisson_run(cases: List[Case], steps: int, rate: float, seed: int = 20261203, **server_kw) -> Dict:
    """Submit the cases at Poisson arrival times (rate per second), wait for
    all, and report time-to-solution percentiles and aggregate throughput."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(cases))
    srv = Server(**server_kw)
    t0 = time.perf_counter()
    reqs = []
    for c, g in zip(cases, gaps):
        time.sleep(g)
        reqs.append(srv.submit(c, steps))
    for r in reqs:
        r.done.wait()
    t1 = time.perf_counter()
    srv.close(wait=True)
    ok = [r for r in reqs if r.error is None]
    tts = [r.time_to_solution for r in ok]
    cell_steps = sum(r.case.mesh.nCells * r.steps for r in ok)
    return {"requests": len(reqs), "completed": len(ok), "errors": [r.error for r in reqs if r.error][:3],
            "p50_s": percentile(tts, 50), "p99_s": percentile(tts, 99), "mean_s": float(np.mean(tts)) if tts else None,
            "wall_s": t1 - t0, "cell_steps_per_s": cell_steps / (t1 - t0),
            "joined_running_batch": sum(1 for r in reqs if r.joined), "relayouts": srv.relayouts,
            "bytes_per_cell_measured": srv.bytes_per_cell, "requests_list": reqs}
