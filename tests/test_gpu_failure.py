"""Failure detection on the GPU, in the forms that fault, trap or hang no GPU.

* A bounded device-side wait that runs out: RT_OPT_STALL_TEST makes the next
  systolic sweep's first plane of each thread-block cluster wait for a
  hand-off word that no plane writes.  The wait gives up after the spins set
  by RT_OPT_WAIT_LIMIT, raises the sweep's error flag, every other wait of the
  launch gives up on seeing it, and the call returns RT_ETIMEOUT.  The same
  context then solves normally and matches the oracle.
* A NaN in a host array handed to rt_field_set: the time step returns
  RT_ENAN (the reference stops with a FatalError on a failed solve,
  newConstitutiveEq.C:47-58 is its abort-on-error style); a fresh case setup
  on the same context then steps to the oracle's fields.
* rt_constitutive_correct_iter with newTimeStep = 0 after a completed time
  step, a plain correct() or a new theta: RT_ENOTREADY, not a silent solve
  against an earlier step's old-time theta.
"""
import time

import numpy as np
import pytest

from rheotool_gb300 import abi
from rheotool_gb300.case import SolverControl, cavity_case, contraction_case
from rheotool_gb300.mesh import contraction_mesh

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def poisson(mesh, rng):
    F, N = mesh.nFaces, mesh.nCells
    g = mesh.magSf * mesh.deltaCoeffs * (1.0 + rng.random(F))
    diag = np.zeros(N)
    np.subtract.at(diag, mesh.owner, g)
    np.subtract.at(diag, mesh.neighbour, g)
    diag -= 1e-3 * mesh.V
    return diag, g.copy(), g.copy()


def test_sweep_wait_runs_out_then_the_context_recovers(ctx):
    from oracle.pyoracle import Oracle
    from rheotool_gb300.runtime import RheoGpuError
    mesh = contraction_mesh(12, 10, 30, 10, 6, 4.0, 4.0)   # structured, 6 planes
    rng = np.random.default_rng(31)
    diag, upper, lower = poisson(mesh, rng)
    b = rng.normal(size=mesh.nCells) * mesh.V
    ctl = SolverControl("PCG", "DIC", 1e-10, 0.0, 0, 500)
    ctx.upload_mesh(mesh)
    try:
        ctx.set_option(abi.RT_OPT_SWEEP_PLANES, 1)        # every plane its own cluster
        ctx.set_option(abi.RT_OPT_WAIT_LIMIT, 1 << 18)
        ctx.set_option(abi.RT_OPT_STALL_TEST, 1)
        x = np.zeros((1, mesh.nCells))
        t0 = time.perf_counter()
        with pytest.raises(RheoGpuError) as e:
            ctx.ldu_solve(diag, upper, lower, b[None], x, ctl)
        assert e.value.status == abi.RT_ETIMEOUT
        assert time.perf_counter() - t0 < 60.0
    finally:
        ctx.set_option(abi.RT_OPT_STALL_TEST, 0)
        ctx.set_option(abi.RT_OPT_WAIT_LIMIT, 1 << 24)
    # the same context, normal waits: the oracle's solve, on one plane per
    # cluster and on the default clusters
    orc = Oracle(contraction_case(mesh))
    xo = np.zeros(mesh.nCells)
    po = orc.ldu_solve(diag, upper, lower, b.copy(), xo, ctl)
    for planes in (1, 16):
        ctx.set_option(abi.RT_OPT_SWEEP_PLANES, planes)
        x = np.zeros((1, mesh.nCells))
        pg = ctx.ldu_solve(diag, upper, lower, b[None], x, ctl)[0]
        assert pg.converged and pg.nIterations == po.nIterations
        assert rel(x[0], xo) < 1e-9


def test_wait_limit_option_bounds():
    from rheotool_gb300.runtime import Context, RheoGpuError
    with Context(0) as c:
        for bad in (0, 63, (1 << 40) + 1):
            with pytest.raises(RheoGpuError) as e:
                c.set_option(abi.RT_OPT_WAIT_LIMIT, bad)
            assert e.value.status == abi.RT_EINVAL
        with pytest.raises(RheoGpuError):
            c.set_option(abi.RT_OPT_STALL_TEST, -1)


def test_nan_in_a_field_gives_enan_then_the_context_recovers(ctx):
    from oracle.pyoracle import Oracle
    from rheotool_gb300.runtime import RheoGpuError
    case = cavity_case(12, model="GiesekusLog", alpha=0.1)
    ctx.setup_case(case)
    ctx.step(2)
    f = ctx.fields()
    U = f.U.copy()
    U[37, 0] = np.nan
    ctx.set_field(abi.RT_FIELD_U, U, f.Ub)
    with pytest.raises(RheoGpuError) as e:
        ctx.step(1)
    assert e.value.status == abi.RT_ENAN
    # a fresh setup on the same context steps normally
    ref = Oracle(case)
    ref.step(3)
    ctx.setup_case(case)
    ctx.step(3)
    got = ctx.fields()
    for name in ("U", "p", "theta", "tau"):
        assert rel(getattr(got, name), getattr(ref.f, name)) < 1e-9, name


def test_nan_in_a_standalone_solve_gives_enan(ctx):
    from rheotool_gb300.runtime import RheoGpuError
    mesh = contraction_mesh(12, 10, 30, 10, 6, 4.0, 4.0)
    rng = np.random.default_rng(32)
    diag, upper, lower = poisson(mesh, rng)
    b = rng.normal(size=mesh.nCells) * mesh.V
    b[5] = np.inf
    ctx.upload_mesh(mesh)
    x = np.zeros((1, mesh.nCells))
    t0 = time.perf_counter()
    with pytest.raises(RheoGpuError) as e:
        ctx.ldu_solve(diag, upper, lower, b[None], x, SolverControl("PCG", "DIC", 1e-10, 0.0, 0, 500))
    assert e.value.status == abi.RT_ENAN
    assert time.perf_counter() - t0 < 30.0


@pytest.mark.parametrize("after", ["step", "correct", "set_theta"])
def test_inner_iteration_after_a_new_step_is_not_ready(ctx, after):
    from rheotool_gb300.runtime import RheoGpuError
    case = cavity_case(8, model="GiesekusLog", alpha=0.1)
    ctx.setup_case(case)
    ctx.step(1)
    ctx.constitutive_correct(newTimeStep=True)
    ctx.constitutive_correct(newTimeStep=False)          # same time step: fine
    if after == "step":
        ctx.step(1)
    elif after == "correct":
        ctx.constitutive_correct()
    else:
        f = ctx.fields()
        ctx.set_field(abi.RT_FIELD_THETA, f.theta, f.thetab)
    with pytest.raises(RheoGpuError) as e:
        ctx.constitutive_correct(newTimeStep=False)
    assert e.value.status == abi.RT_ENOTREADY
    ctx.constitutive_correct(newTimeStep=True)            # a new time step starts
