"""rheoTestFoam on the GPU: the constitutive update under an imposed,
homogeneous velocity gradient.

rheoTestFoam (solvers/rheoTestFoam/rheoTestFoam.C:47-100, createFields.H)
imposes grad U = gradU * rate through the U boundary values of one cell, sets
phi = 0 and calls constEq.correct() nInIter times a time step.  It reports
extraStress = tauTotal() = tau + etaS (symm(L + L^T) - (2/3) tr(L) I)
(constitutiveEq.C:534-547) of the cell:

* transient mode (``ramp false``): the first rate of ``gammaEpsilonDotL``;
  one row (t, extraStress) a time step until endTime (timeWrite.H);
* ramp mode (``ramp true``): nInIter = 1 and, for each rate in turn,
  deltaT = (lambdaMin + lambdaMax) / 2 / rate; the rate is held until the
  relative change of extraStress between steps is below relTol or more than
  maxIter steps were taken, then one row (rate, extraStress, Converged or
  Exceed_Niter, relative change) is written and the next rate starts from
  the state reached (reStartOrEnd.H).  Converged means a change below 1e-8,
  whatever relTol is, as in the reference.

The library runs the homogeneous flow on an 8 x 8 cell box with phi = 0: the
cells are independent and identical, and grad U is passed to the update
directly (rt_constitutive_correct_iter), which is what the imposed boundary
values give fvc::grad(U) in the reference.  From theta = 0 exactly, a pure
shear leaves the log-conformation update at rest (the reference's as well):
give a small initial theta for shear flows.

The backend (``GpuBackend`` by default) is what steps the cell: ``setup``
(case and fields), ``fields``, ``correct`` (grad U, new time step or not) and
``tau`` (the first cell's tau).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Sequence

import numpy as np

from . import abi
from .case import Case, Fields, Model, SolverControl, cavity_case

SMALL = 1e-15   # OpenFOAM's SMALL for double precision


@dataclass
class RheoTestParameters:
    """constitutiveProperties' rheoTestFoamParameters (createFields.H:17-30)."""
    gradU: np.ndarray                  # (3, 3), L_ij = d U_j / d x_i, times each rate
    rates: Sequence[float]             # gammaEpsilonDotL
    ramp: bool = False
    maxIter: int = 5000
    relTol: float = 1e-8


@dataclass
class RheoTestRow:
    x: float                           # t (transient mode) or the rate (ramp mode)
    extraStress: np.ndarray            # (6,) xx, xy, xz, yy, yz, zz
    status: str = ""
    relError: float = float("nan")


class GpuBackend:
    """The library's context on one GPU (a new one, or ctx)."""

    def __init__(self, device: int = 0, ctx=None):
        from .runtime import Context
        self.own = ctx is None
        self.ctx = Context(device) if ctx is None else ctx

    def setup(self, case: Case, fields: Fields):
        self.ctx.setup_case(case, fields)

    def fields(self) -> Fields:
        return self.ctx.fields()

    def correct(self, L: np.ndarray, newTimeStep: bool):
        self.ctx.constitutive_correct(L, newTimeStep=newTimeStep)

    def tau(self) -> np.ndarray:
        return self.ctx.get_field(abi.RT_FIELD_TAU, (self.ctx.mesh.nCells, 6))[0][0]

    def close(self):
        if self.own:
            self.ctx.close()


def extra_stress(tau: np.ndarray, L: np.ndarray, etaS: float) -> np.ndarray:
    """tauTotal() of a viscoelastic model: tau + etaS (L + L^T - (2/3) tr(L) I)."""
    S = L + L.T - (2.0 / 3.0) * np.trace(L) * np.eye(3)
    return np.asarray(tau, dtype=np.float64) + etaS * np.array([S[0, 0], S[0, 1], S[0, 2], S[1, 1], S[1, 2],
                                                                  S[2, 2]])


def _full(s: np.ndarray) -> np.ndarray:
    return np.array([[s[0], s[1], s[2]], [s[1], s[3], s[4]], [s[2], s[4], s[5]]])


def homogeneous_case(model: Model, deltaT: float, solverTheta: Optional[SolverControl] = None,
                     theta0: Optional[np.ndarray] = None) -> tuple:
    """The 8 x 8 box of the homogeneous flow: (case, initial fields)."""
    case = cavity_case(8, model=model.type, dt=deltaT)
    case.model = model
    if solverTheta is not None:
        case.solverTheta = solverTheta
    f = Fields.zeros(case.mesh)
    if theta0 is not None:
        th = np.asarray(theta0, dtype=np.float64).reshape(6)
        mu, R = np.linalg.eigh(_full(th))          # ascending, as calcEig orders them
        f.theta[:] = th
        f.eigVals[:] = np.exp(mu)
        f.eigVecs[:] = R.reshape(9)
    return case, f


def run_rheotest(model: Model, params: RheoTestParameters, deltaT: float, endTime: float, nInIter: int = 0,
                 solverTheta: Optional[SolverControl] = None, theta0: Optional[np.ndarray] = None,
                 backend=None) -> List[RheoTestRow]:
    """The rows rheoTestFoam writes to its Report (see the module docstring)."""
    own = backend is None
    backend = GpuBackend() if own else backend
    try:
        G = np.asarray(params.gradU, dtype=np.float64).reshape(3, 3)
        rates = [float(r) for r in params.rates]
        if not rates:
            raise ValueError("gammaEpsilonDotL is empty")
        lam = model.lambda_           # lambdaMin = lambdaMax for a single-mode model
        dt = (lam + lam) * 0.5 / rates[0] if params.ramp else float(deltaT)
        case, f = homogeneous_case(model, dt, solverTheta, theta0)
        backend.setup(case, f)
        n = case.mesh.nCells
        rows: List[RheoTestRow] = []
        L = G * rates[0]
        if not params.ramp:
            nsteps = int(round(float(endTime) / dt))
            for s in range(1, nsteps + 1):
                for i in range(int(nInIter)):
                    backend.correct(np.tile(L.reshape(9), (n, 1)), i == 0)
                rows.append(RheoTestRow(s * dt, extra_stress(backend.tau(), L, model.etaS)))
            return rows
        idx, cnt, old = 0, 0, np.zeros((3, 3))
        while True:
            backend.correct(np.tile(L.reshape(9), (n, 1)), True)
            es = extra_stress(backend.tau(), L, model.etaS)
            T = _full(es)
            relError = float(np.linalg.norm(T - old) / (np.linalg.norm(T) + SMALL))
            if relError < params.relTol or cnt > params.maxIter:
                rows.append(RheoTestRow(rates[idx], es, "Converged" if relError < 1e-8 else "Exceed_Niter",
                                        relError))
                idx, cnt = idx + 1, 0
                if idx == len(rates):
                    return rows
                case.deltaT = (lam + lam) * 0.5 / rates[idx]
                backend.setup(case, backend.fields())
                L = G * rates[idx]
            old = T
            cnt += 1
    finally:
        if own:
            backend.close()


def report_text(rows: List[RheoTestRow], params: RheoTestParameters) -> str:
    """The Report file of rheoTestFoam (createFields.H:168-180, timeWrite.H,
    reStartOrEnd.H), values with six significant digits."""
    cols = "\t".join(f"extStress{c}" for c in ("XX", "XY", "XZ", "YY", "YZ", "ZZ"))
    g = lambda x: f"{x:.6g}"
    if params.ramp:
        out = ["******* Ramp mode: variable ε̇|γ̇ **********", f"ε̇|γ̇\t{cols}\tStatus\tRelative_Error"]
        out += ["\t".join([g(r.x)] + [g(v) for v in r.extraStress] + [r.status, g(r.relError)]) for r in rows]
    else:
        out = [f"******* Transient mode: fixed ε̇|γ̇ = {g(params.rates[0])} **********", f"t\t{cols}"]
        out += ["\t".join([g(r.x)] + [g(v) for v in r.extraStress]) + "\t" for r in rows]
    return "\n".join(out) + "\n"


def _numbers(v: Any) -> List[float]:
    from .foam_case import scalar
    if isinstance(v, (list, tuple)):
        return [scalar(x) for x in v]
    return [scalar(x) for x in str(v).replace("(", " ").replace(")", " ").split()]


def _switch(v: Any) -> bool:
    return str(v).strip().lower() in ("true", "on", "yes", "y", "1")


def load_rheotest_case(case_dir: str, substitute: bool = True) -> Dict[str, Any]:
    """The inputs of a rheoTestFoam case directory: the model
    (constant/constitutiveProperties ``parameters``), rheoTestFoamParameters,
    deltaT and endTime (system/controlDict), SIMPLE nInIter (default 0) and
    the theta solver (system/fvSolution), and the initial theta of cell 0
    (0/theta, zero when absent)."""
    from . import foam_io
    from .foam_case import CaseError, _solver, read_dict, read_model, scalar
    cp = read_dict(os.path.join(case_dir, "constant", "constitutiveProperties"))
    model = read_model(cp.get("parameters", cp))
    rp = cp.get("rheoTestFoamParameters")
    if not isinstance(rp, dict):
        raise CaseError("sub-dictionary rheoTestFoamParameters is undefined in constitutiveProperties")
    for key in ("gradU", "gammaEpsilonDotL"):
        if key not in rp:
            raise CaseError(f"keyword {key} is undefined in rheoTestFoamParameters")
    gradU = np.array(_numbers(rp["gradU"]))
    if gradU.size != 9:
        raise CaseError(f"rheoTestFoamParameters gradU: a tensor has 9 components, got {gradU.size}")
    ramp = _switch(rp.get("ramp", "false"))
    params = RheoTestParameters(gradU.reshape(3, 3), _numbers(rp["gammaEpsilonDotL"]), ramp,
                                int(scalar(rp.get("maxIter", "5000"))), scalar(rp.get("relTol", "1e-8")))
    ctrl = read_dict(os.path.join(case_dir, "system", "controlDict"))
    sol = read_dict(os.path.join(case_dir, "system", "fvSolution"))
    subs: List[str] = []
    solverTheta = _solver(sol.get("solvers", {}), "theta", subs, substitute)
    theta0 = None
    path = os.path.join(case_dir, "0", "theta")
    if os.path.exists(path):
        internal, _ = foam_io.read_field(path, n_internal=1)
        theta0 = np.asarray(internal, dtype=np.float64).reshape(-1, 6)[0]
    return dict(model=model, params=params, deltaT=scalar(ctrl.get("deltaT", "1")),
                endTime=scalar(ctrl.get("endTime", "1")),
                nInIter=int(scalar(sol.get("SIMPLE", {}).get("nInIter", "0"))), solverTheta=solverTheta,
                theta0=theta0, substitutions=subs)


def run_rheotest_case(case_dir: str, backend=None, substitute: bool = True) -> List[RheoTestRow]:
    """Run a rheoTestFoam case directory and write its Report file."""
    inp = load_rheotest_case(case_dir, substitute)
    rows = run_rheotest(inp["model"], inp["params"], inp["deltaT"], inp["endTime"], inp["nInIter"],
                        inp["solverTheta"], inp["theta0"], backend)
    with open(os.path.join(case_dir, "Report"), "w") as fh:
        fh.write(report_text(rows, inp["params"]))
    return rows


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="rheoTestFoam on the GPU: run a case directory, write its Report")
    ap.add_argument("case_dir")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    be = GpuBackend(a.device)
    try:
        rows = run_rheotest_case(a.case_dir, backend=be)
    finally:
        be.ctx.close()
    print(f"{len(rows)} rows written to {os.path.join(a.case_dir, 'Report')}")


if __name__ == "__main__":
    main()
