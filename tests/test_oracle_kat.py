"""Known-answer tests that pin the FP64 CPU oracle.

The reference (rheoTool on OpenFOAM v9 + Eigen) cannot be built here and ships
no golden fields, so the oracle is pinned by closed-form rheology, by the
conformation-tensor form of each model integrated independently with scipy,
by dense linear algebra, and by exactness properties of the discretisation.
The committed golden vectors in tests/golden/ freeze these results.
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle
from oracle.pyoracle import Oracle
from rheotool_gb300.case import Fields, SolverControl, cavity_case, contraction_case, channel_case
from rheotool_gb300.mesh import cavity_mesh, contraction_mesh

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# ---------------------------------------------------------------------------
# eigen decomposition
# ---------------------------------------------------------------------------
def test_eig3_matches_numpy():
    rng = np.random.default_rng(1)
    for _ in range(200):
        s = rng.normal(size=6) * rng.choice([1e-3, 1.0, 30.0])
        mu, V = pyoracle.eig3(s)
        A = np.array([[s[0], s[1], s[2]], [s[1], s[3], s[4]], [s[2], s[4], s[5]]])
        w = np.linalg.eigvalsh(A)
        scale = max(np.abs(w).max(), 1e-300)
        assert np.max(np.abs(mu - w)) < 1e-14 * scale * 10
        assert np.max(np.abs(V @ np.diag(mu) @ V.T - A)) < 1e-13 * scale * 10
        assert np.max(np.abs(V.T @ V - np.eye(3))) < 1e-14
        assert np.all(np.diff(mu) >= 0)


def test_eig3_exact_cases():
    mu, V = pyoracle.eig3([0, 0, 0, 0, 0, 0])
    assert np.array_equal(mu, [0, 0, 0]) and np.array_equal(V, np.eye(3))
    mu, V = pyoracle.eig3([3.0, 0, 0, 1.0, 0, 2.0])
    assert np.array_equal(mu, [1.0, 2.0, 3.0])
    assert np.array_equal(np.abs(V), np.eye(3)[:, [1, 2, 0]])
    # a 2-D conformation keeps e_z exactly and its eigenvalue exactly
    mu, V = pyoracle.eig3([0.3, 0.7, 0.0, -0.2, 0.0, 0.0])
    k = int(np.argmax(np.abs(V[2])))
    assert V[2, k] in (1.0, -1.0) and mu[k] == 0.0
    assert np.all(V[:2, k] == 0.0) and np.all(V[2, [i for i in range(3) if i != k]] == 0.0)


# ---------------------------------------------------------------------------
# LDU solvers against dense solves
# ---------------------------------------------------------------------------
def dense(mesh, diag, upper, lower):
    A = np.diag(diag)
    A[mesh.neighbour, mesh.owner] = lower
    A[mesh.owner, mesh.neighbour] = upper
    return A


def test_pcg_dic_matches_dense_solve():
    mesh = cavity_mesh(9)
    rng = np.random.default_rng(2)
    g = 1.0 + rng.random(mesh.nFaces)
    diag = np.zeros(mesh.nCells)
    np.subtract.at(diag, mesh.owner, g)
    np.subtract.at(diag, mesh.neighbour, g)
    diag[0] *= 2.0                     # setReference makes it definite
    b = rng.normal(size=mesh.nCells)
    x = np.zeros(mesh.nCells)
    o = Oracle(cavity_case(9))
    p = o.ldu_solve(diag, g, g, b, x, SolverControl("PCG", "DIC", 1e-13, 0, 0, 1000))
    xd = np.linalg.solve(dense(mesh, diag, g, g), b)
    assert p.converged
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-9
    # DIC must beat no preconditioning
    x2 = np.zeros(mesh.nCells)
    p2 = o.ldu_solve(diag, g, g, b, x2, SolverControl("PCG", "none", 1e-13, 0, 0, 1000))
    assert p.nIterations < p2.nIterations


@pytest.mark.parametrize("pre", ["DILU", "diagonal", "none"])
def test_pbicgstab_matches_dense_solve(pre):
    mesh = contraction_mesh(6, 5, 4, 2, 3, 2.0, 2.0)
    rng = np.random.default_rng(3)
    phi = rng.normal(size=mesh.nFaces)
    u = (phi >= 0).astype(float)
    lower = -u * phi - 1.0
    upper = (1 - u) * phi - 1.0
    diag = np.zeros(mesh.nCells)
    np.subtract.at(diag, mesh.owner, lower)
    np.subtract.at(diag, mesh.neighbour, upper)
    diag += 0.5
    b = rng.normal(size=mesh.nCells)
    x = np.zeros(mesh.nCells)
    p = Oracle(contraction_case(mesh)).ldu_solve(diag, upper, lower, b, x,
                                                  SolverControl("PBiCGStab", pre, 1e-13, 0, 0, 2000))
    xd = np.linalg.solve(dense(mesh, diag, upper, lower), b)
    assert p.converged
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-9


@pytest.mark.parametrize("pre", ["DILU", "diagonal", "none"])
def test_pbicg_matches_dense_solve(pre):
    """PBiCG (OpenFOAM's bi-conjugate gradients, the Contraction41 tutorials'
    U and theta solver) on an upwinded convection-diffusion matrix."""
    mesh = contraction_mesh(6, 5, 4, 2, 3, 2.0, 2.0)
    rng = np.random.default_rng(6)
    phi = rng.normal(size=mesh.nFaces)
    u = (phi >= 0).astype(float)
    lower = -u * phi - 1.0
    upper = (1 - u) * phi - 1.0
    diag = np.zeros(mesh.nCells)
    np.subtract.at(diag, mesh.owner, lower)
    np.subtract.at(diag, mesh.neighbour, upper)
    diag += 0.5
    b = rng.normal(size=mesh.nCells)
    x = np.zeros(mesh.nCells)
    o = Oracle(contraction_case(mesh))
    p = o.ldu_solve(diag, upper, lower, b, x, SolverControl("PBiCG", pre, 1e-13, 0, 0, 2000))
    xd = np.linalg.solve(dense(mesh, diag, upper, lower), b)
    assert p.converged and not p.singular
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-9
    assert o.residual(diag, upper, lower, b, x) < 1e-13


def test_pbicg_on_a_symmetric_matrix_is_pcg():
    """With a symmetric matrix, a symmetric preconditioner and rT = r, the
    shadow recurrences of BiCG repeat the primal ones: PBiCG takes PCG's
    iterations (same counts, the same solution to round-off)."""
    mesh = cavity_mesh(9)
    rng = np.random.default_rng(7)
    g = 1.0 + rng.random(mesh.nFaces)
    diag = np.zeros(mesh.nCells)
    np.subtract.at(diag, mesh.owner, g)
    np.subtract.at(diag, mesh.neighbour, g)
    diag -= 0.1
    b = rng.normal(size=mesh.nCells)
    o = Oracle(cavity_case(9))
    x1, x2 = np.zeros(mesh.nCells), np.zeros(mesh.nCells)
    p1 = o.ldu_solve(diag, g, g, b, x1, SolverControl("PCG", "DIC", 1e-12, 0, 0, 1000))
    p2 = o.ldu_solve(diag, g, g, b, x2, SolverControl("PBiCG", "DIC", 1e-12, 0, 0, 1000))
    assert p1.nIterations == p2.nIterations
    assert np.linalg.norm(x1 - x2) <= 1e-12 * np.linalg.norm(x1)


def test_dilu_preconditioner_is_exact_for_tridiagonal():
    # D-ILU of a tridiagonal matrix has no fill-in: one application solves it
    mesh = cavity_mesh(1, ny=12)       # a 1 x 12 column: tridiagonal LDU
    rng = np.random.default_rng(4)
    lower = -1.0 - rng.random(mesh.nFaces)
    upper = -1.0 - rng.random(mesh.nFaces)
    diag = 4.0 + rng.random(mesh.nCells)
    b = rng.normal(size=mesh.nCells)
    x = np.zeros(mesh.nCells)
    p = Oracle(cavity_case(mesh=mesh)).ldu_solve(diag, upper, lower, b, x,
                                         SolverControl("PBiCGStab", "DILU", 1e-14, 0, 0, 10))
    assert p.nIterations == 1
    assert np.allclose(x, np.linalg.solve(dense(mesh, diag, upper, lower), b), rtol=1e-12)


def test_residual_normalisation_definition():
    mesh = cavity_mesh(5)
    rng = np.random.default_rng(5)
    diag = 4.0 + rng.random(mesh.nCells)
    upper = -rng.random(mesh.nFaces)
    lower = -rng.random(mesh.nFaces)
    b = rng.normal(size=mesh.nCells)
    x = rng.normal(size=mesh.nCells)
    A = dense(mesh, diag, upper, lower)
    Ax = A @ x
    pA = A.sum(1) * x.mean()
    nf = np.sum(np.abs(Ax - pA) + np.abs(b - pA)) + 1e-20
    ref = np.sum(np.abs(b - Ax)) / nf
    got = Oracle(cavity_case(5)).residual(diag, upper, lower, b, x)
    assert abs(got - ref) < 1e-13 * ref


# ---------------------------------------------------------------------------
# discretisation exactness
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mesh_fn", [lambda: cavity_mesh(7), lambda: contraction_mesh(6, 5, 4, 2, 3, 2.0, 2.0)])
def test_gauss_gradient_exact_for_linear_fields(mesh_fn):
    mesh = mesh_fn()
    a = np.array([0.3, -1.7, 2.2])
    if mesh.solveDir[2] == 0:
        a[2] = 0.0
    psi = mesh.C @ a + 0.5
    psib = mesh.bCf @ a + 0.5
    case = cavity_case(7) if mesh.solveDir[2] == 0 else contraction_case(mesh)
    g = Oracle(case).grad(psi, psib)
    assert np.max(np.abs(g - a)) < 1e-11


# ---------------------------------------------------------------------------
# homogeneous flows (0-D driver, rheoTestFoam style): imposed grad U
# ---------------------------------------------------------------------------
def zero_d(model, lam, etaP, dt, **kw):
    """Four uniform cells with phi = 0 and an imposed grad U.  theta starts at
    diag(1e-8, -1e-8, 0): from exactly theta = 0 with R = I, decomposeGradU
    gives B = 0 and Omega.theta - theta.Omega = 0 under pure shear, so the
    log-conformation update (rheoTool's as well) would stay at rest."""
    # model keys that the case builder's own arguments shadow (Rolie-Poly's
    # beta, XPomPom's and WhiteMetznerCY's n)
    late = {k: kw.pop(k) for k in ("beta", "n") if k in kw}
    case = cavity_case(2, model=model, Wi=lam, beta=1.0 - etaP, Re=1.0, dt=dt, **kw)
    for k, v in late.items():
        setattr(case.model, k, v)
    f = Fields.zeros(case.mesh)
    f.theta[:, 0], f.theta[:, 3] = 1e-8, -1e-8
    f.eigVals[:, 0], f.eigVals[:, 1] = np.exp(1e-8), np.exp(-1e-8)
    o = Oracle(case, f)
    return case, o


def shear_L(rate, n):
    L = np.zeros((n, 9))
    L[:, 3] = rate            # d u_x / d y
    return L


def test_oldroydb_startup_shear_closed_form():
    lam, etaP, rate = 0.5, 0.7, 2.0
    dt = lam / 2000
    case, o = zero_d("Oldroyd-BLog", lam, etaP, dt)
    L = shear_L(rate, case.mesh.nCells)
    t = 0.0
    for _ in range(2000):
        o.constitutive_correct(L)
        t += dt
    txy = o.f.tau[:, 1].mean()
    exact = etaP * rate * (1.0 - np.exp(-t / lam))
    assert abs(txy - exact) < 2e-3 * exact


def rp_chi(trA, chiMax):
    c2 = chiMax * chiMax
    return ((3.0 - (trA / 3.0) / c2) * (1.0 - 1.0 / c2)) / ((1.0 - (trA / 3.0) / c2) * (3.0 - 1.0 / c2))


def conformation_steady(model, lam, rate, alpha=0.0, eps=0.0, L2=100.0, lambdaR=1.0, beta=0.0, delta=-0.5,
                        chiMax=0.0, lambdaS=1.0, q=1.0, n=0.0, K=0.0, a=1.0, mlab=None):
    """Steady simple shear of the conformation-tensor form, integrated with
    scipy (an independent formulation of the same model)."""
    from scipy.integrate import solve_ivp
    kap = np.zeros((3, 3))
    kap[0, 1] = rate
    I = np.eye(3)

    def rhs(t, y):
        A = y.reshape(3, 3)
        if model == "Oldroyd-BLog":
            g = A - I
        elif model == "GiesekusLog":
            g = (A - I) + alpha * (A - I) @ (A - I)
        elif model == "PTTLog" and mlab is not None:
            # Gamma(beta) E_{alpha,beta}(z) by its series, with scipy's Gamma
            from scipy.special import gamma
            z = eps * (np.trace(A) - 3.0)
            k = np.arange(60)
            g = gamma(mlab[1]) * np.sum(z ** k / gamma(mlab[0] * k + mlab[1])) * (A - I)
        elif model == "PTTLog":
            g = (1.0 + eps * (np.trace(A) - 3.0)) * (A - I)
        elif model == "FENE-CRLog":
            g = (L2 / (L2 - np.trace(A))) * (A - I)
        elif model == "Rolie-PolyLog":
            trA = np.trace(A)
            M1 = 2.0 * (1.0 - np.sqrt(3.0 / trA)) / lambdaR
            if chiMax > 1.0:
                M1 *= rp_chi(trA, chiMax)
            g = (A - I) + lam * M1 * (A + beta * (trA / 3.0) ** delta * (A - I))
        elif model == "XPomPomLog":
            trA = np.trace(A)
            Lb = np.sqrt(trA / 3.0)
            f = (2.0 * (lam / lambdaS) * np.exp((2.0 / q) * (Lb - 1.0)) * (1.0 - Lb ** -(n + 1.0))
                 + (1.0 - alpha - (alpha / 3.0) * (np.trace(A @ A) - 2.0 * trA)) / Lb ** 2)
            g = A * (f - 2.0 * alpha) + alpha * A @ A + (alpha - 1.0) * I
        elif model == "WhiteMetznerCYLog":
            # Oldroyd-B with the Carreau-Yasuda relaxation time at the shear rate
            g = (A - I) / (1.0 + (K * rate) ** a) ** ((n - 1.0) / a)
        else:
            f = L2 / (L2 - np.trace(A))
            a2 = L2 / (L2 - 3.0)
            g = f * A - a2 * I
        return (kap @ A + A @ kap.T - g / lam).reshape(-1)

    sol = solve_ivp(rhs, (0, 60 * lam), I.reshape(-1), rtol=1e-12, atol=1e-14, method="LSODA")
    A = sol.y[:, -1].reshape(3, 3)
    if model == "FENE-PLog":
        return (L2 / (L2 - np.trace(A))) * A - (L2 / (L2 - 3.0)) * I
    if model == "FENE-CRLog":
        return (L2 / (L2 - np.trace(A))) * (A - I)
    if model == "Rolie-PolyLog" and chiMax > 1.0:
        return rp_chi(np.trace(A), chiMax) * (A - I)
    return A - I


@pytest.mark.parametrize("model,kw,ckw", [
    ("Oldroyd-BLog", {}, {}),
    ("GiesekusLog", {"alpha": 0.3}, {"alpha": 0.3}),
    ("PTTLog", {"epsilon": 0.25}, {"eps": 0.25}),
    ("PTTLog", {"epsilon": 0.25, "destructionFunctionType": "generalized", "alpha": 0.8, "beta": 1.2},
     {"eps": 0.25, "mlab": (0.8, 1.2)}),
    ("FENE-PLog", {"L2": 100.0}, {"L2": 100.0}),
    ("FENE-CRLog", {"L2": 20.0}, {"L2": 20.0}),
    ("Rolie-PolyLog", {"lambdaR": 0.2, "beta": 0.5, "delta": -0.5},
     {"lambdaR": 0.2, "beta": 0.5, "delta": -0.5}),
    ("Rolie-PolyLog", {"lambdaR": 0.3, "beta": 0.3, "delta": -0.5, "chiMax": 5.0},
     {"lambdaR": 0.3, "beta": 0.3, "delta": -0.5, "chiMax": 5.0}),
    ("XPomPomLog", {"lambdaS": 0.4, "q": 2.0, "alpha": 0.15, "n": 0.0},
     {"lambdaS": 0.4, "q": 2.0, "alpha": 0.15, "n": 0.0}),
    ("XPomPomLog", {"lambdaS": 0.25, "q": 5.0, "alpha": 0.1, "n": 1.5},
     {"lambdaS": 0.25, "q": 5.0, "alpha": 0.1, "n": 1.5}),
    ("WhiteMetznerCYLog", {"K": 0.5, "a": 2.0, "n": 0.6}, {"K": 0.5, "a": 2.0, "n": 0.6}),
])
def test_steady_shear_matches_conformation_form(model, kw, ckw):
    lam, etaP, rate = 1.0, 0.8, 1.5
    dt = lam / 40
    case, o = zero_d(model, lam, etaP, dt, **kw)
    L = shear_L(rate, case.mesh.nCells)
    for _ in range(int(60 * lam / dt)):
        o.constitutive_correct(L)
    tau = o.f.tau.mean(0)
    ref = (etaP / lam) * conformation_steady(model, lam, rate, **ckw)
    got = np.array([tau[0], tau[1], tau[2], tau[3], tau[4], tau[5]])
    want = np.array([ref[0, 0], ref[0, 1], ref[0, 2], ref[1, 1], ref[1, 2], ref[2, 2]])
    assert np.max(np.abs(got - want)) < 1e-7 * np.abs(want).max()
    if model == "Oldroyd-BLog":
        assert abs(tau[1] - etaP * rate) < 1e-8
        assert abs((tau[0] - tau[3]) - 2 * etaP * lam * rate ** 2) < 1e-7
    if model == "WhiteMetznerCYLog":
        # closed form: tau_xy = etaP(gd) gd, N1 = 2 etaP(gd) lambda(gd) gd^2
        F = (1.0 + (kw["K"] * rate) ** kw["a"]) ** ((kw["n"] - 1.0) / kw["a"])
        assert abs(tau[1] - etaP * F * rate) < 1e-8
        assert abs((tau[0] - tau[3]) - 2 * etaP * F * lam * F * rate ** 2) < 1e-7


# ---------------------------------------------------------------------------
# time-step invariants
# ---------------------------------------------------------------------------
def test_step_conserves_mass_contraction():
    case = contraction_case(contraction_mesh(8, 6, 4, 3, 3, 3.0, 3.0), dt=0.02)
    o = Oracle(case)
    perf = o.step(3)
    assert perf.p.converged
    m = case.mesh
    div = np.zeros(m.nCells)
    np.add.at(div, m.owner, o.f.phi)
    np.subtract.at(div, m.neighbour, o.f.phi)
    np.add.at(div, m.bCell, o.f.phib)
    inflow = -o.f.phib[o.f.phib < 0].sum()
    assert np.abs(div).sum() < 1e-6 * inflow
    # global balance: what enters leaves
    assert abs(o.f.phib.sum()) < 1e-6 * inflow


def test_step_2d_keeps_out_of_plane_components_zero():
    case = cavity_case(10, model="GiesekusLog", alpha=0.2)
    o = Oracle(case)
    perf = o.step(4)
    assert np.all(o.f.U[:, 2] == 0.0)
    assert np.all(o.f.theta[:, [2, 4]] == 0.0)
    assert np.all(o.f.theta[:, 5] == 0.0)
    assert perf.U[2].nIterations == -1 and perf.theta[2].nIterations == -1


def test_poiseuille_channel_oldroydb():
    """Fully developed Oldroyd-B channel flow: U is the Newtonian parabola of
    eta0 and tau_xy = etaP dU/dy (2-D channel, inlet plug flow)."""
    from rheotool_gb300.mesh import channel_mesh
    mesh = channel_mesh(nx=30, ny=16, L=6.0, H=1.0, two_d=True)
    case = channel_case(mesh, model="Oldroyd-BLog", U_in=1.0, dt=0.02, lambda_=0.1, beta=0.5)
    o = Oracle(case)
    o.step(150)
    ij = mesh.cellIJK
    col = ij[:, 0] == 24
    y = mesh.C[col, 1]
    order = np.argsort(y)
    u = o.f.U[col, 0][order]
    y = y[order]
    exact = 6.0 * y * (1.0 - y)
    assert np.max(np.abs(u - exact)) < 2e-2
    dudy = 6.0 * (1.0 - 2.0 * y)
    txy = o.f.tau[col, 1][order]
    assert np.max(np.abs(txy - 0.5 * dudy)) < 6e-2


# ---------------------------------------------------------------------------
# golden vectors (frozen oracle output, regenerated by tests/golden/make_golden.py)
# ---------------------------------------------------------------------------
def _golden_cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.golden_cases()


@pytest.mark.parametrize("index", range(6))
def test_golden_vectors(index):
    """Every frozen oracle output (the cavity for Oldroyd-B, FENE-CR,
    Rolie-Poly, XPomPom and WhiteMetznerCY, the periodic PTT channel with two
    inner iterations) is
    reproduced to round-off by the current oracle."""
    from oracle.pyoracle import Oracle
    name, case, f0, steps = _golden_cases()[index]
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip("golden file missing")
    g = np.load(path)
    o = Oracle(case, None if f0 is None else f0.copy())
    o.step(steps)
    for field in ("U", "p", "theta", "tau", "phi"):
        ref = g[field]
        assert np.linalg.norm(getattr(o.f, field) - ref) <= 1e-12 * np.linalg.norm(ref), (name, field)


def test_golden_cavity_oracle():
    path = os.path.join(GOLDEN, "cavity16_oldroydb_10steps.npz")
    if not os.path.exists(path):
        pytest.skip("golden file missing")
    g = np.load(path)
    case = cavity_case(16)
    o = Oracle(case)
    o.step(10)
    for name in ("U", "p", "theta", "tau", "phi"):
        ref = g[name]
        assert np.linalg.norm(getattr(o.f, name) - ref) <= 1e-12 * np.linalg.norm(ref), name


# ---------------------------------------------------------------------------
# multiMode (multiMode.C): modes summed
# ---------------------------------------------------------------------------
def test_multimode_of_two_half_modes_is_the_single_mode():
    """Oldroyd-B's conformation does not depend on etaP, so two identical
    modes with etaP/2 each carry half the stress each: their multiMode model
    steps exactly as the single mode (summed tau, summed viscosities)."""
    import copy
    one = cavity_case(10, model="Oldroyd-BLog", Wi=0.5)
    two = copy.copy(one)
    half = copy.copy(one.model)
    half.etaP = one.model.etaP / 2
    half.etaS = one.model.etaS / 2
    two.model = half
    two.moreModes = [copy.copy(half)]
    a, b = Oracle(one), Oracle(two)
    a.step(4)
    b.step(4)
    for name in ("U", "p", "phi", "tau", "theta"):
        x, y = getattr(b.f, name), getattr(a.f, name)
        assert np.linalg.norm(x - y) <= 1e-12 * np.linalg.norm(y), name
    for m in b.f.modes:
        assert np.linalg.norm(2 * m.tau - a.f.tau) <= 1e-12 * np.linalg.norm(a.f.tau)
        assert np.linalg.norm(m.theta - a.f.theta) <= 1e-12 * np.linalg.norm(a.f.theta)


def test_multimode_modes_differ_and_sum():
    """Two different modes (Oldroyd-B lambda 0.5, Giesekus lambda 0.1): each
    mode keeps its own conformation, and tau is their sum."""
    import copy
    case = cavity_case(10, model="Oldroyd-BLog", Wi=0.5)
    m2 = copy.copy(case.model)
    m2.type, m2.lambda_, m2.alpha, m2.etaP, m2.etaS = "GiesekusLog", 0.1, 0.2, 0.3, 0.0
    case.moreModes = [m2]
    o = Oracle(case)
    o.step(3)
    t0, t1 = o.f.modes[0].tau, o.f.modes[1].tau
    assert np.linalg.norm(t0 - t1) > 1e-3 * np.linalg.norm(t0)
    assert np.array_equal(o.f.tau, t0 + t1)
    assert np.array_equal(o.f.theta, o.f.modes[0].theta)


# ---------------------------------------------------------------------------
# Crank-Nicolson ddt (the Cavity tutorial's "CrankNicolson 1")
# ---------------------------------------------------------------------------
def test_crank_nicolson_psi0_is_euler():
    """Off-centering coefficient 0: c = 1 and no old-time derivative term, the
    implicit Euler scheme (the ddtCorr's old-time parts are regrouped, so the
    agreement is to round-off)."""
    import copy
    a_case = cavity_case(10, model="GiesekusLog", alpha=0.1)
    b_case = copy.copy(a_case)
    b_case.ddt, b_case.ddtPsi = "CrankNicolson", 0.0
    a, b = Oracle(a_case), Oracle(b_case)
    a.step(4)
    b.step(4)
    for name in ("U", "p", "phi", "theta", "tau"):
        x, y = getattr(b.f, name), getattr(a.f, name)
        assert np.linalg.norm(x - y) <= 1e-12 * np.linalg.norm(y), name


def test_crank_nicolson_old_time_derivative_recursion():
    """D_1 = (U_1 - U_0)/dt after the implicit Euler first step, then D_2 =
    2 (U_2 - U_1)/dt - D_1 (psi = 1); D is formed at the start of the next
    step, so after three steps the state holds D_2."""
    case = cavity_case(8, model="Oldroyd-BLog")
    case.ddt, case.ddtPsi = "CrankNicolson", 1.0
    o = Oracle(case)
    U = [o.f.U.copy()]
    for _ in range(3):
        o.step(1)
        U.append(o.f.U.copy())
    dt = case.deltaT
    D1 = (U[1] - U[0]) / dt
    D2 = 2.0 * (U[2] - U[1]) / dt - D1
    DU = o._ddt_arrays["DU"].reshape(-1, 3)
    assert np.linalg.norm(DU - D2) <= 1e-9 * np.linalg.norm(D2)
    assert np.array_equal(o._ddt_arrays["Us"].reshape(-1, 3), U[2])
    # and CN differs from Euler by more than round-off
    e = Oracle(cavity_case(8, model="Oldroyd-BLog"))
    e.step(3)
    assert np.linalg.norm(e.f.U - o.f.U) > 1e-6 * np.linalg.norm(o.f.U)
