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

A multiMode model (multiMode.C: a list of models) runs each mode on its own
box; extraStress sums the modes' tau and etaS, and lambdaMin / lambdaMax of
the ramp's time step range over the modes (createFields.H:185-200).  In a
homogeneous flow the modes do not interact, so this is the reference's
multi-mode update; the flow solver takes single-mode models only.

A backend is what steps the cell of one mode: ``setup`` (case and fields),
``fields``, ``correct`` (grad U, new time step or not) and ``tau`` (the
first cell's tau).  ``GpuBackend`` (one library context) is the default.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Sequence, Union

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


def run_rheotest(model: Union[Model, Sequence[Model]], params: RheoTestParameters, deltaT: float,
                 endTime: float, nInIter: int = 0, solverTheta: Optional[SolverControl] = None,
                 theta0: Optional[np.ndarray] = None, backend=None) -> List[RheoTestRow]:
    """The rows rheoTestFoam writes to its Report (see the module docstring).
    model: one Model or the modes of a multiMode model; backend: one per
    mode (a list, or a single backend for a single mode), default a
    GpuBackend each."""
    modes = [model] if isinstance(model, Model) else list(model)
    if not modes:
        raise ValueError("multiMode: no models")
    own = backend is None
    backends = [GpuBackend() for _ in modes] if own else (list(backend) if isinstance(backend, (list, tuple))
                                                         else [backend])
    if len(backends) != len(modes):
        raise ValueError(f"{len(modes)} modes need as many backends, got {len(backends)}")
    try:
        G = np.asarray(params.gradU, dtype=np.float64).reshape(3, 3)
        rates = [float(r) for r in params.rates]
        if not rates:
            raise ValueError("gammaEpsilonDotL is empty")
        lamMax, lamMin = max(m.lambda_ for m in modes), min(m.lambda_ for m in modes)
        etaS = sum(m.etaS for m in modes)
        dt = (lamMin + lamMax) * 0.5 / rates[0] if params.ramp else float(deltaT)
        cases = []
        for m, be in zip(modes, backends):
            case, f = homogeneous_case(m, dt, solverTheta, theta0)
            be.setup(case, f)
            cases.append(case)
        n = cases[0].mesh.nCells
        rows: List[RheoTestRow] = []
        L = G * rates[0]

        def tau_total():
            return sum(be.tau() for be in backends)

        if not params.ramp:
            nsteps = int(round(float(endTime) / dt))
            for s in range(1, nsteps + 1):
                for be in backends:
                    for i in range(int(nInIter)):
                        be.correct(np.tile(L.reshape(9), (n, 1)), i == 0)
                rows.append(RheoTestRow(s * dt, extra_stress(tau_total(), L, etaS)))
            return rows
        idx, cnt, old = 0, 0, np.zeros((3, 3))
        while True:
            for be in backends:
                be.correct(np.tile(L.reshape(9), (n, 1)), True)
            es = extra_stress(tau_total(), L, etaS)
            T = _full(es)
            relError = float(np.linalg.norm(T - old) / (np.linalg.norm(T) + SMALL))
            if relError < params.relTol or cnt > params.maxIter:
                rows.append(RheoTestRow(rates[idx], es, "Converged" if relError < 1e-8 else "Exceed_Niter",
                                        relError))
                idx, cnt = idx + 1, 0
                if idx == len(rates):
                    return rows
                for case, be in zip(cases, backends):
                    case.deltaT = (lamMin + lamMax) * 0.5 / rates[idx]
                    be.setup(case, be.fields())
                L = G * rates[idx]
            old = T
            cnt += 1
    finally:
        if own:
            for be in backends:
                be.close()


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


def read_modes(par: Dict[str, Any]) -> Union[Model, List[Model]]:
    """The Model of a ``parameters`` dictionary, or the modes of a
    multiMode one (``models ( M1 { ... } M2 { ... } );``, multiMode.C:69-91)."""
    from .foam_case import CaseError, parse_dict, read_model
    if par.get("type") != "multiMode":
        return read_model(par)
    raw = par.get("models")
    if not isinstance(raw, str) or not raw.strip().startswith("("):
        raise CaseError("keyword models is undefined in the multiMode parameters")
    entries = parse_dict(raw.strip()[1:-1])
    modes = [read_model(d) for d in entries.values() if isinstance(d, dict)]
    if not modes:
        raise CaseError("multiMode: the models list is empty")
    return modes


def load_rheotest_case(case_dir: str, substitute: bool = True) -> Dict[str, Any]:
    """The inputs of a rheoTestFoam case directory: the model
    (constant/constitutiveProperties ``parameters``), rheoTestFoamParameters,
    deltaT and endTime (system/controlDict), SIMPLE nInIter (default 0) and
    the theta solver (system/fvSolution), and the initial theta of cell 0
    (0/theta, zero when absent)."""
    from . import foam_io
    from .foam_case import CaseError, _solver, read_dict, read_model, scalar
    cp = read_dict(os.path.join(case_dir, "constant", "constitutiveProperties"))
    model = read_modes(cp.get("parameters", cp))
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
    modes = load_rheotest_case(a.case_dir)["model"]
    bes = [GpuBackend(a.device) for _ in (modes if isinstance(modes, list) else [modes])]
    try:
        rows = run_rheotest_case(a.case_dir, backend=bes)
    finally:
        for be in bes:
            be.close()
    print(f"{len(rows)} rows written to {os.path.join(a.case_dir, 'Report')}")


if __name__ == "__main__":
    main()
