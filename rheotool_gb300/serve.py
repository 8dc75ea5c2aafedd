"""Serving form: a request loop with continuous batching of independent cases.

Requests (a case and a number of time steps) arrive at any time.  The loop
keeps a set of slots, each driven by its own worker thread on its own CUDA
stream: a slot holds either one case in its own context or several small
cases admitted together as one batch (one device mesh, every stage of the
step one launch for all of them).  A waiting request is admitted as soon as
a slot is free and its predicted device-memory footprint (bytes per cell
times its cells, plus a fixed per-slot part) fits in what the budget leaves
after the footprints of the requests already on the device; the measured
footprint of each admission is recorded from the library's own allocation
counter.  Fields stay on the device between steps;
a slot steps its cases in quanta of a few steps, so the work of all admitted
requests overlaps on the GPU, and each finished request returns its fields
and its time to solution.  A case gives the same result alone as in the mix:
a slot is an independent context, and a batch solves every case with its own
Krylov scalars and stopping points.

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
    done: threading.Event = field(default_factory=threading.Event)

    @property
    def time_to_solution(self) -> float:
        return self.finished - self.arrival


class Server:
    """Continuous-batching request loop.

    slots: concurrent slots (worker threads, CUDA streams);
    hbm_budget: device bytes the admitted cases may hold (default: 90 % of
    the free device memory at start);
    batch_cells: requests at most this many cells are admitted in groups of
    up to batch_max as one batch slot;
    quantum: steps a slot takes between two looks at its requests."""

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
        self.bytes_per_cell = bytes_per_cell
        self.slot_bytes = slot_bytes
        self.measured: List[float] = []              # bytes per cell of each admission
        self.pending: "queue.Queue[Request]" = queue.Queue()
        self._waiting: List[Request] = []
        self._lock = threading.Lock()
        self._reserved = 0
        self._stop = False
        self._workers = [threading.Thread(target=self._worker, daemon=True) for _ in range(slots)]
        self._next = 0
        self.finished: List[Request] = []
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
    def _footprint(self, cells: int) -> int:
        return int(self.bytes_per_cell * cells) + self.slot_bytes

    def _take(self) -> Optional[List[Request]]:
        """The next group to admit (FIFO; small requests grouped), or None."""
        with self._lock:
            while not self.pending.empty():
                self._waiting.append(self.pending.get_nowait())
            if not self._waiting:
                return None
            head = self._waiting[0]
            group = [head]
            if head.case.mesh.nCells <= self.batch_cells:
                for r in self._waiting[1:]:
                    if len(group) >= self.batch_max:
                        break
                    if r.case.mesh.nCells <= self.batch_cells and self._batchable(head.case, r.case) \
                            and r.steps == head.steps:
                        group.append(r)
            cells = sum(r.case.mesh.nCells for r in group)
            need = self._footprint(cells)
            if self._reserved + need > self.budget:
                if len(group) > 1:
                    group = [head]
                    need = self._footprint(head.case.mesh.nCells)
                if self._reserved + need > self.budget:
                    return None
            for r in group:
                self._waiting.remove(r)
            self._reserved += need
            for r in group:
                r.admitted = time.perf_counter()
            return group + [need]

    @staticmethod
    def _batchable(a: Case, b: Case) -> bool:
        return all(getattr(a, k) == getattr(b, k) for k in ("deltaT", "divU", "divTheta", "solverU", "solverP",
                                                            "solverTheta", "precision")) and \
            np.array_equal(a.mesh.solveDir, b.mesh.solveDir)

    # ---- slots ---------------------------------------------------------------
    def _worker(self):
        while not self._stop:
            got = self._take()
            if got is None:
                time.sleep(0.002)
                continue
            need = [got.pop()]

            def release():
                with self._lock:
                    self._reserved -= need[0]
                    need[0] = 0

            # a context per admission: closing it gives the slot's device
            # memory back before the next admission is sized
            ctx = None
            try:
                before = device_bytes()
                ctx = Context(self.device)
                self._run(ctx, got, before, release)
            except Exception as e:   # the request fails, the loop goes on
                for r in got:
                    r.error = f"{type(e).__name__}: {e}"
                    r.finished = time.perf_counter()
                    r.done.set()
            finally:
                if ctx is not None:
                    ctx.close()
                release()

    def _run(self, ctx: Context, group: List[Request], before: int, release):
        """Set up the slot, step it to the end, hand back the fields; the
        footprint reservation is held until the worker closes the context."""
        if len(group) == 1:
            r = group[0]
            ctx.setup_case(r.case)
            slot = None
        else:
            slot = BatchContext([r.case for r in group], ctx=ctx)
        cells = sum(r.case.mesh.nCells for r in group)
        used = device_bytes() - before    # (other slots may allocate meanwhile: an upper bound)
        with self._lock:
            self.measured.append(used / cells)
        steps = group[0].steps
        done = 0
        while done < steps:
            n = min(self.quantum, steps - done)
            ctx.step(n)
            done += n
        ctx.sync()
        if slot is None:
            group[0].fields = ctx.fields()
        else:
            for r, f in zip(group, slot.fields()):
                r.fields = f
        now = time.perf_counter()
        for r in group:
            r.finished = now
            r.done.set()
        with self._lock:
            self.finished.extend(group)


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
            "wall_s": t1 - t0, "cell_steps_per_s": cell_steps / (t1 - t0), "requests_list": reqs}
