"""The periodic channel (cyclic patches in x and z, body-force driven, the
precision-sweep configuration) on the GPU, through the C ABI, against the
FP64 oracle: the LDU solvers on a mesh with coupled faces, full FP64 steps
with both sweep schedules (1e-9 relative L2), and the mixed-precision form
(within max(1e-6, 3 x the oracle's own solver-tolerance error))."""
import copy

import numpy as np
import pytest

from rheotool_gb300 import abi
from rheotool_gb300.case import SolverControl, periodic_channel_case, periodic_channel_state
from rheotool_gb300.mesh import periodic_channel_mesh

from test_gpu_parity import TOL_STEP, laplacian_system, rel

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-6


def _mesh():
    return periodic_channel_mesh(12, 10, 6, L=2.0, H=1.0, depth=1.0, wall_ratio=2.0)


def _case(mesh, Wi=2.0, model="PTTLog", **kw):
    return periodic_channel_case(mesh, model=model, Wi=Wi, dt=5e-3, **kw)


@pytest.mark.parametrize("sweep", [abi.SWEEP_LEVELS, abi.SWEEP_SYSTOLIC])
@pytest.mark.parametrize("solver,pre", [("PCG", "DIC"), ("PBiCGStab", "DILU")])
def test_ldu_solve_with_coupled_faces(ctx, sweep, solver, pre):
    """A x includes the coupled (cyclic) faces, DIC/DILU leave them out: the
    device solvers take the oracle's iterations and reach its solution."""
    from oracle.pyoracle import Oracle
    mesh = _mesh()
    rng = np.random.default_rng(17)
    diag, upper, lower = laplacian_system(mesh, rng, asym=3.0 if solver == "PBiCGStab" else 0.0)
    b = rng.normal(size=mesh.nCells) * mesh.V
    ctl = SolverControl(solver, pre, 1e-10, 0.0, 0, 2000)
    o = Oracle(_case(mesh))
    xo = np.zeros(mesh.nCells)
    po = o.ldu_solve(diag, upper, lower, b, xo, ctl)
    ctx.upload_mesh(mesh)
    ctx.set_sweep(sweep)
    try:
        xg = np.zeros((1, mesh.nCells))
        pg = ctx.ldu_solve(diag, upper, lower, b[None], xg, ctl)[0]
    finally:
        ctx.set_sweep(abi.SWEEP_AUTO)
    assert po.nIterations > 3
    assert abs(pg.nIterations - po.nIterations) <= 1, (pg.nIterations, po.nIterations)
    assert rel(xg[0], xo) < TOL_STEP


@pytest.mark.parametrize("sweep", [abi.SWEEP_LEVELS, abi.SWEEP_SYSTOLIC])
@pytest.mark.parametrize("Wi", [0.5, 8.0])
def test_step_periodic_channel_ptt(ctx, sweep, Wi):
    from oracle.pyoracle import Oracle
    mesh = _mesh()
    case = _case(mesh, Wi=Wi)
    f0 = periodic_channel_state(case, sigma=0.1, seed=20261203)
    o = Oracle(case, fields=f0.copy())
    o.step(4)
    ctx.set_sweep(sweep)
    try:
        ctx.setup_case(case, f0.copy())
        ctx.step(4)
        got = ctx.fields()
    finally:
        ctx.set_sweep(abi.SWEEP_AUTO)
    for n in ("U", "p", "phi", "theta", "tau"):
        e = rel(getattr(got, n), getattr(o.f, n))
        assert e < TOL_STEP, (n, e)


def test_step_periodic_channel_mixed(ctx):
    from oracle.pyoracle import Oracle
    mesh = _mesh()
    case = _case(mesh, Wi=2.0)
    f0 = periodic_channel_state(case, sigma=0.1, seed=20261203)
    ref = Oracle(case, fields=f0.copy())
    ref.step(5)
    tight = copy.copy(case)
    tight.solverU, tight.solverP, tight.solverTheta = [
        SolverControl(s.solver, s.preconditioner, s.tolerance * 1e-2, s.relTol, s.minIter, 4 * s.maxIter)
        for s in (case.solverU, case.solverP, case.solverTheta)]
    ref_t = Oracle(tight, fields=f0.copy())
    ref_t.step(5)
    case.precision = abi.RT_PREC_MIXED
    ctx.setup_case(case, f0.copy())
    ctx.step(5)
    got = ctx.fields()
    for n in ("U", "p", "phi", "theta", "tau"):
        floor = rel(getattr(ref_t.f, n), getattr(ref.f, n))
        err = rel(getattr(got, n), getattr(ref.f, n))
        assert err < max(TOL_MIXED, 3.0 * floor), (n, err, floor)
