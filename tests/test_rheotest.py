"""The rheoTestFoam driver (rheotool_gb300/rheotest.py) on the CPU: its time
loop, ramp bookkeeping, extraStress and Report, stepped by the oracle in
place of the GPU (an inner-iteration correct() against the step's old
theta, as rt_constitutive_correct_iter does), against closed-form
Oldroyd-B extension and steady shear, and a case directory."""
import os

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from rheotool_gb300.case import Model
from rheotool_gb300.rheotest import (RheoTestParameters, extra_stress, load_rheotest_case, report_text,
                                     run_rheotest, run_rheotest_case)

UNIAXIAL = np.diag([1.0, -0.5, -0.5])


class OracleBackend:
    """The oracle behind the driver's backend calls (test infrastructure)."""

    calls = 0

    def setup(self, case, fields):
        self.o = Oracle(case, fields.copy())

    def fields(self):
        return self.o.f.copy()

    def correct(self, L, newTimeStep):
        if newTimeStep:
            self.theta0 = self.o.f.theta.copy()
        self.o.constitutive_correct(L, thetaOld=self.theta0)
        self.calls += 1

    def tau(self):
        return self.o.f.tau[0].copy()


def oldroydb_extension(lam, etaP, etaS, rate, t=None):
    """Oldroyd-B in uniaxial extension: A_xx, A_yy relax to 1/(1 - 2 Wi) and
    1/(1 + Wi) (Wi = lambda rate) at rates (1 - 2 Wi)/lambda and (1 + Wi)/lambda."""
    wi = lam * rate
    ax, ay = 1.0 / (1.0 - 2.0 * wi), 1.0 / (1.0 + wi)
    if t is not None:
        ax = ax + (1.0 - ax) * np.exp(-(1.0 - 2.0 * wi) * t / lam)
        ay = ay + (1.0 - ay) * np.exp(-(1.0 + wi) * t / lam)
    tau = (etaP / lam) * np.array([ax - 1.0, 0, 0, ay - 1.0, 0, ay - 1.0])
    return extra_stress(tau, UNIAXIAL * rate, etaS)


def test_extra_stress_is_tau_plus_the_solvent_stress():
    L = np.array([[0.1, 2.0, 0.0], [0.3, -0.4, 0.0], [0.0, 0.0, 0.3]])
    es = extra_stress(np.arange(6.0), L, 0.5)
    S = L + L.T - (2.0 / 3.0) * np.trace(L) * np.eye(3)
    assert np.allclose(es, np.arange(6.0) + 0.5 * np.array([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2], S[2, 2]]))


def test_transient_extension_follows_the_closed_form():
    lam, etaP, etaS, rate, dt = 1.0, 0.8, 0.2, 0.2, 1e-3
    model = Model("Oldroyd-BLog", rho=1.0, etaS=etaS, etaP=etaP, lambda_=lam, stabilization="none")
    params = RheoTestParameters(UNIAXIAL, [rate], ramp=False)
    be = OracleBackend()
    rows = run_rheotest(model, params, dt, 2.0, nInIter=1, backend=be)
    assert len(rows) == 2000 and abs(rows[-1].x - 2.0) < 1e-12 and be.calls == 2000
    for r in (rows[499], rows[-1]):
        want = oldroydb_extension(lam, etaP, etaS, rate, r.x)
        assert np.max(np.abs(r.extraStress - want)) < 2e-3 * np.max(np.abs(want))


def test_transient_without_inner_iterations_does_nothing():
    """SIMPLE nInIter defaults to 0 in rheoTestFoam (createFields.H:139):
    no correct() is called and tau stays at its initial value."""
    model = Model("Oldroyd-BLog", etaS=0.2, etaP=0.8, lambda_=1.0)
    be = OracleBackend()
    rows = run_rheotest(model, RheoTestParameters(UNIAXIAL, [0.2]), 0.1, 0.5, backend=be)
    assert be.calls == 0 and len(rows) == 5
    assert np.allclose(rows[0].extraStress, extra_stress(np.zeros(6), UNIAXIAL * 0.2, 0.2))


def test_inner_iterations_share_the_old_time_theta():
    """nInIter = 3 iterates each step's update (theta.oldTime() fixed): the
    result is close to one correct() a step, not to three steps."""
    model = Model("GiesekusLog", etaS=0.2, etaP=0.8, lambda_=1.0, alpha=0.3)
    p = RheoTestParameters(UNIAXIAL, [0.3])
    r1 = run_rheotest(model, p, 0.01, 0.5, nInIter=1, backend=OracleBackend())
    r3 = run_rheotest(model, p, 0.01, 0.5, nInIter=3, backend=OracleBackend())
    r1x3 = run_rheotest(model, p, 0.03, 1.5, nInIter=1, backend=OracleBackend())
    a, b, c = r1[-1].extraStress, r3[-1].extraStress, r1x3[-1].extraStress
    assert np.max(np.abs(a - b)) < 0.05 * np.max(np.abs(b - c))


SHEAR = np.zeros((3, 3))
SHEAR[1, 0] = 1.0                     # d u_x / d y
SEED = np.array([1e-8, 0, 0, -1e-8, 0, 0])


def test_ramp_reaches_the_steady_states():
    """Oldroyd-B steady shear: tau_xy = etaP rate, N1 = 2 etaP lambda rate^2.
    The ramp's time step is lambda / rate and the log-form sources are
    explicit, so the steps are stable only where lambda rate is large
    enough (here from 1.5; in extension never, for any rate below the
    coil-stretch limit) -- the reference's choice of time step."""
    lam, etaP, etaS = 1.0, 0.8, 0.2
    model = Model("Oldroyd-BLog", etaS=etaS, etaP=etaP, lambda_=lam)
    rates = [1.5, 2.0, 3.0]
    params = RheoTestParameters(SHEAR, rates, ramp=True, maxIter=5000, relTol=1e-10)
    rows = run_rheotest(model, params, deltaT=None, endTime=None, theta0=SEED, backend=OracleBackend())
    assert [r.x for r in rows] == rates
    for r in rows:
        assert r.status == "Converged" and r.relError < 1e-10
        es = r.extraStress
        assert abs(es[1] - (etaP + etaS) * r.x) < 1e-7 * r.x
        assert abs((es[0] - es[3]) - 2 * etaP * lam * r.x ** 2) < 1e-6 * r.x ** 2


def test_ramp_gives_up_after_maxIter():
    model = Model("Oldroyd-BLog", etaS=0.2, etaP=0.8, lambda_=1.0)
    params = RheoTestParameters(SHEAR, [1.5, 2.0], ramp=True, maxIter=3, relTol=1e-12)
    be = OracleBackend()
    rows = run_rheotest(model, params, None, None, theta0=SEED, backend=be)
    # the check precedes the count (rheoTestFoam.C:75-85): the first rate ends
    # on its (maxIter + 2)-th step; the step that ends a rate counts as the
    # next rate's first, so later rates end on their (maxIter + 1)-th
    assert [r.status for r in rows] == ["Exceed_Niter", "Exceed_Niter"] and be.calls == (3 + 2) + (3 + 1)
    assert all(r.relError > 1e-8 for r in rows)


def _write(path, body, cls="dictionary"):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write(f"FoamFile\n{{\n    version 2.0;\n    format ascii;\n    class {cls};\n}}\n" + body)


def test_case_directory_and_report(tmp_path):
    root = str(tmp_path / "rt")
    _write(os.path.join(root, "constant", "constitutiveProperties"),
           "parameters\n{\n    type Oldroyd-BLog;\n    rho rho [1 -3 0 0 0 0 0] 1;\n"
           "    etaS etaS [1 -1 -1 0 0 0 0] 0.2;\n    etaP etaP [1 -1 -1 0 0 0 0] 0.8;\n"
           "    lambda lambda [0 0 1 0 0 0 0] 1;\n    stabilization none;\n}\n"
           "rheoTestFoamParameters\n{\n    ramp true;\n    gradU ( 0 0 0\n 1 0 0\n 0 0 0 );\n"
           "    gammaEpsilonDotL ( 1.5 2 );\n    relTol 1e-10;\n}\n")
    _write(os.path.join(root, "0", "theta"), "dimensions [0 0 0 0 0 0 0];\n"
           "internalField uniform (1e-8 0 0 -1e-8 0 0);\nboundaryField\n{\n}\n", cls="volSymmTensorField")
    _write(os.path.join(root, "system", "controlDict"), "application rheoTestFoam;\ndeltaT 0.001;\nendTime 5;\n")
    _write(os.path.join(root, "system", "fvSolution"),
           "solvers\n{\n    \"theta.*|tau.*\" { solver PBiCG; preconditioner DILU; tolerance 1e-10; relTol 0; }\n}\n"
           "SIMPLE { nInIter 5; }\n")
    inp = load_rheotest_case(root)
    assert inp["params"].ramp and inp["params"].rates == [1.5, 2.0] and inp["nInIter"] == 5
    assert np.allclose(inp["params"].gradU, SHEAR) and inp["solverTheta"].solver == "PBiCG"
    assert np.allclose(inp["theta0"], [1e-8, 0, 0, -1e-8, 0, 0])
    assert not any("PBiCG" in s for s in inp["substitutions"])
    rows = run_rheotest_case(root, backend=OracleBackend())
    text = open(os.path.join(root, "Report")).read().splitlines()
    assert text[0].startswith("******* Ramp mode") and text[1].split("\t")[-2:] == ["Status", "Relative_Error"]
    assert len(text) == 4 and text[2].split("\t")[0] == "1.5" and text[3].split("\t")[7] == "Converged"
    assert float(text[3].split("\t")[1]) == pytest.approx(rows[1].extraStress[0], rel=1e-5)
    t = report_text(rows[:1], RheoTestParameters(UNIAXIAL, [0.05], ramp=False)).splitlines()
    assert t[0] == "******* Transient mode: fixed ε̇|γ̇ = 0.05 **********"


def test_multimode_sums_the_modes():
    """Two Oldroyd-B modes in steady shear: tau_xy = (etaS1 + etaS2 + etaP1 +
    etaP2) rate, N1 = 2 (etaP1 lambda1 + etaP2 lambda2) rate^2; the ramp's
    time step uses lambdaMin and lambdaMax of the modes."""
    m1 = Model("Oldroyd-BLog", etaS=0.1, etaP=0.5, lambda_=0.8)
    m2 = Model("Oldroyd-BLog", etaS=0.05, etaP=0.3, lambda_=1.2)
    params = RheoTestParameters(SHEAR, [2.0, 3.0], ramp=True, relTol=1e-10)
    bes = [OracleBackend(), OracleBackend()]
    rows = run_rheotest([m1, m2], params, None, None, theta0=SEED, backend=bes)
    assert bes[0].o.case.deltaT == pytest.approx((0.8 + 1.2) * 0.5 / 3.0)
    for r in rows:
        es = r.extraStress
        assert r.status == "Converged"
        assert abs(es[1] - (0.1 + 0.05 + 0.5 + 0.3) * r.x) < 1e-7 * r.x
        assert abs((es[0] - es[3]) - 2 * (0.5 * 0.8 + 0.3 * 1.2) * r.x ** 2) < 1e-6 * r.x ** 2
    with pytest.raises(ValueError, match="backends"):
        run_rheotest([m1, m2], params, None, None, backend=OracleBackend())


def test_multimode_case_directory(tmp_path):
    from rheotool_gb300.foam_case import parse_dict
    from rheotool_gb300.rheotest import read_modes
    par = parse_dict("parameters\n{\n    type multiMode;\n    models\n    (\n"
                     "        M1 { type XPomPomLog; rho 1; etaS 0; etaP 280.4; lambdaB 0.0039; lambdaS 0.00056;"
                     " alpha 0.3; q 1; n 0; stabilization coupling; }\n"
                     "        M2 { type GiesekusLog; rho 1; etaS 0.1; etaP 810.4; lambda 0.051; alpha 0.3;"
                     " stabilization coupling; }\n    );\n}\n")["parameters"]
    modes = read_modes(par)
    assert [m.type for m in modes] == ["XPomPomLog", "GiesekusLog"]
    assert modes[0].lambda_ == 0.0039 and modes[0].lambdaS == 0.00056 and modes[1].alpha == 0.3
    from rheotool_gb300.foam_case import CaseError
    with pytest.raises(CaseError, match="models"):
        read_modes({"type": "multiMode"})
