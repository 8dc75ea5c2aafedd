"""Serving form: requests admitted while others run, slots overlapping on the
device, small requests batched; every result equals the same case run alone.

The bar: a case served in a slot of its own is bit-identical to the case alone
(same kernels, same order); a case served inside a batch differs from it alone
only by the grouping of its reductions (1e-8 relative L2 in FP64; the mixed
form's bar, max(1e-6, 3 x the FP64 oracle's solver-tolerance error), when
served in mixed precision).
"""
import time

import numpy as np
import pytest

from rheotool_gb300 import abi
from rheotool_gb300.case import cavity_case, contraction_case
from rheotool_gb300.mesh import cavity_mesh, contraction_mesh
from rheotool_gb300.runtime import Context
from rheotool_gb300.serve import Server

from test_gpu_parity import rel

pytestmark = pytest.mark.gpu

NAMES = ("U", "p", "phi", "theta", "tau")


def mix(precision):
    cases = [
        cavity_case(12, model="Oldroyd-BLog", Wi=0.5, dt=5e-3),
        cavity_case(16, model="GiesekusLog", Wi=1.0, dt=5e-3, alpha=0.1),
        contraction_case(contraction_mesh(16, 14, 8, 4, two_d=True), dt=5e-3),
        cavity_case(20, model="FENE-PLog", Wi=0.3, dt=5e-3, L2=100.0),
        cavity_case(10, model="GiesekusLog", Wi=2.0, dt=5e-3, alpha=0.1),
        cavity_case(24, model="Oldroyd-BLog", Wi=1.0, dt=5e-3),
    ]
    for c in cases:
        c.precision = precision
    return cases


def alone(case, steps):
    ctx = Context(0)
    try:
        ctx.setup_case(case)
        ctx.step(steps)
        return ctx.fields()
    finally:
        ctx.close()


@pytest.mark.parametrize("precision", [abi.RT_PREC_FP64, abi.RT_PREC_MIXED])
def test_served_results_equal_alone(precision):
    steps = 6
    cases = mix(precision)
    srv = Server(slots=3, hbm_budget=8 << 30, batch_cells=300, batch_max=3, quantum=2)
    reqs = []
    try:
        for i, c in enumerate(cases):
            reqs.append(srv.submit(c, steps))
            time.sleep(0.02 * (i % 2))        # some arrive while others run
        for r in reqs:
            assert r.done.wait(120), "request not served"
    finally:
        srv.close()
    bar = 1e-8 if precision == abi.RT_PREC_FP64 else 1e-6
    for r in reqs:
        assert r.error is None, r.error
        ref = alone(r.case, steps)
        for n in NAMES:
            e = rel(getattr(r.fields, n), getattr(ref, n))
            assert e < bar, (r.rid, n, e)
    # continuous batching: at least two requests were on the device at once
    spans = sorted((r.admitted, r.finished) for r in reqs)
    assert any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1))


def test_admission_waits_for_memory():
    """A budget that holds one case at a time serialises the requests."""
    cases = mix(abi.RT_PREC_FP64)[:3]
    from rheotool_gb300.serve import device_bytes
    base = device_bytes()
    srv = Server(slots=3, hbm_budget=base + (24 << 20), batch_cells=0, quantum=3, slot_bytes=16 << 20)
    try:
        reqs = [srv.submit(c, 3) for c in cases]
        for r in reqs:
            assert r.done.wait(120)
    finally:
        srv.close()
    assert all(r.error is None for r in reqs)
    spans = sorted((r.admitted, r.finished) for r in reqs)
    assert all(spans[i + 1][0] >= spans[i][1] - 1e-3 for i in range(len(spans) - 1))


@pytest.mark.parametrize("precision", [abi.RT_PREC_FP64, abi.RT_PREC_MIXED])
def test_request_joining_a_running_batch_equals_alone(precision):
    """Continuous batching on the device: requests submitted while a batch is
    running join it at a quantum boundary (the batch is laid out again and the
    running case carries its fields into the new layout) and leave when their
    own steps are done; every result equals the case run alone (1e-8 FP64,
    1e-6 mixed), the long-running case's included."""
    cases = mix(precision)
    long_case, joiners = cases[1], [cases[0], cases[3], cases[4]]
    srv = Server(slots=1, hbm_budget=8 << 30, batch_cells=2000, batch_max=4, quantum=2)
    try:
        first = srv.submit(long_case, 40)
        t0 = time.time()
        while first.admitted == 0.0 and time.time() - t0 < 60:
            time.sleep(0.005)
        time.sleep(0.05)
        later = [srv.submit(c, 4 + 2 * i) for i, c in enumerate(joiners)]
        for r in [first] + later:
            assert r.done.wait(300), "request not served"
    finally:
        srv.close()
    assert first.error is None and all(r.error is None for r in later)
    assert any(r.joined for r in later), "no request joined the running batch"
    assert srv.relayouts >= 1
    bar = 1e-8 if precision == abi.RT_PREC_FP64 else 1e-6
    for r in [first] + later:
        ref = alone(r.case, r.steps)
        for n in NAMES:
            e = rel(getattr(r.fields, n), getattr(ref, n))
            assert e < bar, (r.rid, r.joined, n, e)
