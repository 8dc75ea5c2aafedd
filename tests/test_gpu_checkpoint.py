"""Checkpoint and resume on the GPU: a run stopped after k steps, written,
and resumed in a fresh context continues bit for bit as the run that did not
stop (FP64 and mixed forms, a multiMode model)."""
import numpy as np
import pytest

from rheotool_gb300 import abi, checkpoint
from rheotool_gb300.case import cavity_case
from rheotool_gb300.runtime import Context

from test_gpu_parity import multimode_case

pytestmark = pytest.mark.gpu


def _fields_equal(a, b):
    for name, x in a.__dict__.items():
        if isinstance(x, np.ndarray):
            assert np.array_equal(getattr(b, name), x), name
    assert len(a.modes) == len(b.modes)
    for ma, mb in zip(a.modes, b.modes):
        for name, x in ma.__dict__.items():
            assert np.array_equal(getattr(mb, name), x), name


@pytest.mark.parametrize("kind", ["fp64", "mixed", "multimode"])
def test_resume_continues_bit_for_bit(ctx, tmp_path, kind):
    case = cavity_case(16, model="GiesekusLog", Wi=1.0, dt=5e-3, alpha=0.1)
    if kind == "mixed":
        case.precision = abi.RT_PREC_MIXED
    if kind == "multimode":
        case = multimode_case(case)
    ctx.setup_case(case)
    ctx.step(6)
    whole = ctx.fields()
    ctx.setup_case(case)
    ctx.step(3)
    path = str(tmp_path / "snap.npz")
    checkpoint.save(ctx, path, step=3, time=3 * case.deltaT)
    with Context(0) as fresh:
        meta = checkpoint.resume(fresh, case, path)
        assert meta["step"] == 3
        fresh.step(3)
        resumed = fresh.fields()
    _fields_equal(whole, resumed)
