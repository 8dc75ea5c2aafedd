"""Run an OpenFOAM/rheoTool case directory through the library.

``load_case(case_dir)`` reads what rheoFoam reads for the segregated step:

* ``constant/polyMesh`` (``foam_io.read_polymesh``);
* ``constant/constitutiveProperties``: the ``parameters`` sub-dictionary
  (``type``, ``rho``, ``etaS``, ``etaP``, ``lambda`` ... ``stabilization``;
  dimensioned entries ``rho rho [1 -3 0 0 0 0 0] 0.01;`` give their number);
* ``system/fvSolution``: the ``solvers`` entries for p, U and theta (keys may
  be quoted regular expressions such as ``"(theta|tau)"``) and ``SIMPLE``
  (``nInIter``, ``pRefCell``, ``pRefValue``);
* ``system/fvSchemes``: ``div(phi,U)`` and ``div(phi,theta)`` (GaussDefCmpw
  with a limiter) and the ddt scheme;
* ``system/controlDict``: ``deltaT``, ``endTime``, ``writeInterval``;
* ``0/U``, ``0/p``, ``0/theta``, ``0/tau``: initial internal fields and the
  boundary conditions (fixedValue, zeroGradient, linearExtrapolation; empty
  and cyclic patches are part of the mesh).

A multiMode model (``type multiMode; models ( M1 { ... } M2 { ... } );``,
multiMode.C:69-91) reads each mode's ``0/thetaM1``, ``0/tauM1`` ... (the
fields rheoTool names after the mode's keyword) instead of ``0/theta`` and
``0/tau``; the modes must share rho, the stabilization and the boundary
conditions of theta and tau (the library sums their divTau as one).
``run_case`` writes ``tau`` (the modes' sum) and every mode's ``theta<K>``
and ``tau<K>``.

What the library does not implement is refused with a clear message unless
``substitute=True`` is given, in which case each substitution is recorded in
``loaded.substitutions``: rheoTool's external sparse solvers (``solverType eigenSolver``,
``petscSolver``, ``hypreSolver``) become PCG-DIC for p and PBiCGStab-DILU for
the others at their tolerance; ddt schemes other than Euler and
CrankNicolson become Euler; relaxation factors other than 1 are dropped (a
non-orthogonal mesh runs with the orthogonal laplacian only on request;
``nNonOrthogonalCorrectors`` is honoured, its explicit correction being zero
with that laplacian); a
``codedFixedValue`` patch (its code cannot run here) uses its ``value`` entry
unless ``bc_overrides`` gives the values.  ``run_case`` steps the case on the GPU
and writes OpenFOAM fields at the write times.

    python -m rheotool_gb300.foam_case CASE_DIR [--steps N] [--substitute] [--mixed] [--log]
"""
from __future__ import annotations

import argparse
import fnmatch
import os
import re
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Tuple

import numpy as np

from . import abi, foam_io
from .case import Case, Fields, Model, SolverControl, ThermoFunction

# ---------------------------------------------------------------------------
# dictionaries
# ---------------------------------------------------------------------------


def parse_dict(text: str) -> Dict[str, Any]:
    """OpenFOAM dictionary text -> nested dict of raw string values (the
    FoamFile header is skipped; comments removed)."""
    t = foam_io._strip(text)
    pos = 0

    def level(i: int) -> Tuple[Dict[str, Any], int]:
        d: Dict[str, Any] = {}
        n = len(t)
        while i < n:
            while i < n and t[i].isspace():
                i += 1
            if i >= n:
                break
            if t[i] == "}":
                return d, i + 1
            if t[i] == '"':
                e = t.index('"', i + 1)
                key = t[i + 1:e]
                i = e + 1
            else:
                s = i
                while i < n and not t[i].isspace() and t[i] not in "{;":
                    i += 1
                key = t[s:i]
            while i < n and t[i].isspace():
                i += 1
            if i < n and t[i] == "{":
                sub, i = level(i + 1)
                d[key] = sub
                continue
            s, depth = i, 0
            while i < n and not (t[i] == ";" and depth == 0):
                if t[i] == "(":
                    depth += 1
                elif t[i] == ")":
                    depth -= 1
                i += 1
            d[key] = t[s:i].strip()
            i += 1
        return d, i

    d, _ = level(pos)
    d.pop("FoamFile", None)
    return d


def read_dict(path: str) -> Dict[str, Any]:
    return parse_dict(foam_io._read_text(path))


def scalar(v: str) -> float:
    """The number of a plain or dimensioned scalar entry."""
    nums = re.findall(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?", v.split("]")[-1])
    if not nums:
        raise ValueError(f"no number in {v!r}")
    return float(nums[-1])


def lookup_pattern(d: Dict[str, Any], name: str) -> Optional[Any]:
    """An entry by exact name, else by a key that is a regular expression
    (OpenFOAM's quoted keys) or a glob matching it."""
    if name in d:
        return d[name]
    for k, v in d.items():
        try:
            if re.fullmatch(k, name):
                return v
        except re.error:
            pass
        if fnmatch.fnmatch(name, k):
            return v
    return None


# ---------------------------------------------------------------------------
# the case
# ---------------------------------------------------------------------------
LIMITERS = {"upwind", "cubista", "minmod", "smart", "waceb", "superbee"}


@dataclass
class LoadedCase:
    case: Case
    fields: Fields
    endTime: float
    writeInterval: float
    substitutions: List[str] = field(default_factory=list)
    mode_names: List[str] = field(default_factory=list)   # multiMode: the modes' keywords


# the keywords each model's constructor looks up without a default, beyond
# rho, etaS, etaP, lambda (lambdaD, lambdaB) and stabilization
# (GiesekusLog.C, PTTLog.C, FENE_PLog.C, FENE_CRLog.C, RoliePolyLog.C,
# XPomPomLog.C:114-122, WhiteMetznerCYLog.C:124-133)
MODEL_KEYS = {
    "GiesekusLog": ("alpha",),
    "PTTLog": ("epsilon", "zeta", "destructionFunctionType"),
    "FENE-PLog": ("L2",),
    "FENE-CRLog": ("L2",),
    "Rolie-PolyLog": ("lambdaR", "beta", "delta", "chiMax"),
    "XPomPomLog": ("lambdaS", "alpha", "q", "n"),
    "WhiteMetznerCYLog": ("m", "n", "K", "L", "a", "b"),
}
# the temperature functions each model builds (thermoFunction::New)
# each model's thermoFunction sub-dictionaries: (lambda, second relaxation
# time, etaP) (Oldroyd_BLog.C:118-119, RoliePolyLog.C:122-124,
# XPomPomLog.C:123-125)
THERMO_KEYS = {
    "Rolie-PolyLog": ("thermoLambdaD", "thermoLambdaR", "thermoEta"),
    "XPomPomLog": ("thermoLambdaB", "thermoLambdaS", "thermoEta"),
}
# the keywords of each thermoFunction type (thermoFunctions/<type>/<type>.C
# constructors)
THERMO_ARGS = {"Constant": (), "Arrhenius": ("alpha", "T0"), "ArrheniusModified": ("alpha", "T0"),
               "WLF": ("c1", "c2", "T0"), "VFT": ("A", "B", "T0")}


class CaseError(ValueError):
    pass


def _solver(d: Dict[str, Any], name: str, subs: List[str], substitute: bool) -> SolverControl:
    e = lookup_pattern(d, name)
    if e is None:
        raise CaseError(f"fvSolution: no solver entry for {name} (a case that solves U, p and tau coupled "
                        "through rheoTool's coupledSolvers is not supported)")
    sv = e.get("solver", "")
    stype = e.get("solverType", "openFoam")
    if stype != "openFoam":
        # rheoTool's external sparse solvers (sparseSolver.C:41): Eigen, PETSc, Hypre
        if not substitute:
            raise CaseError(f"fvSolution {name}: solverType {stype} ({sv}) is not implemented; pass "
                            "substitute=True for the library's Krylov solver at the same tolerance")
        new = ("PCG", "DIC") if name == "p" else ("PBiCGStab", "DILU")
        subs.append(f"{name}: solverType {stype} {sv} -> {new[0]}-{new[1]}")
        return SolverControl(new[0], new[1], scalar(e.get("tolerance", "1e-6")), scalar(e.get("relTol", "0")),
                             int(scalar(e.get("minIter", "0"))), int(scalar(e.get("maxIter", "1000"))))
    if sv not in ("PCG", "PBiCGStab", "PBiCG"):
        raise CaseError(f"fvSolution {name}: solver {sv!r} is not implemented (PCG, PBiCGStab, PBiCG)")
    pre = e.get("preconditioner", "none")
    if isinstance(pre, dict):
        pre = pre.get("preconditioner", "none")
    if pre not in ("DIC", "DILU", "diagonal", "none"):
        raise CaseError(f"fvSolution {name}: preconditioner {pre!r} is not implemented")
    return SolverControl(sv, pre, scalar(e.get("tolerance", "1e-6")), scalar(e.get("relTol", "0")),
                         int(scalar(e.get("minIter", "0"))), int(scalar(e.get("maxIter", "1000"))))


def _limiter(schemes: Dict[str, Any], key: str) -> str:
    v = lookup_pattern(schemes.get("divSchemes", {}), key)
    if v is None:
        v = schemes.get("divSchemes", {}).get("default", "none")
    words = v.split()
    if len(words) >= 2 and words[0] == "GaussDefCmpw" and words[1] in LIMITERS:
        return words[1]
    if words[:2] == ["Gauss", "upwind"]:
        return "upwind"
    raise CaseError(f"fvSchemes {key}: {v!r} is not implemented (GaussDefCmpw <limiter> or Gauss upwind)")


def read_mode_entries(par: Dict[str, Any]) -> Tuple[List[str], List[Model]]:
    """The modes of a ``parameters`` dictionary: ([], [model]) for a single
    model; for ``type multiMode`` the modes' keywords and models in list
    order (multiMode.C:69-91), which must share rho and the stabilization
    (the library takes one divTau of the summed tau with the summed
    viscosities)."""
    if par.get("type") != "multiMode":
        return [], [read_model(par)]
    raw = par.get("models")
    if not isinstance(raw, str) or not raw.strip().startswith("("):
        raise CaseError("keyword models is undefined in the multiMode parameters")
    entries = [(k, d) for k, d in parse_dict(raw.strip()[1:-1]).items() if isinstance(d, dict)]
    if not entries:
        raise CaseError("multiMode: the models list is empty")
    models = [read_model(d) for _, d in entries]
    for m in models[1:]:
        if m.rho != models[0].rho or m.stabilization != models[0].stabilization:
            raise CaseError("multiMode: the modes must share rho and stabilization (their divTau is summed as one)")
    return [k for k, _ in entries], models


def _bc_signature(bf: Dict[str, Any], mesh) -> List[Tuple[str, str, Any]]:
    """The boundary conditions of a field file, patch by patch (kind and value)."""
    out = []
    for p in mesh.patches:
        e = lookup_pattern(bf, p.name)
        if e is None:
            out.append((p.name, "", None))
            continue
        v = None if e["value"] is None else tuple(np.asarray(e["value"], dtype=np.float64).ravel().tolist())
        out.append((p.name, e["type"], v))
    return out


def read_model(par: Dict[str, Any]) -> Model:
    """The Model of a constitutiveProperties ``parameters`` dictionary, with
    the keywords each model's constructor reads and its FatalErrors as
    CaseError (newConstitutiveEq.C:32-61 and the models' constructors)."""
    typ = par.get("type", "")
    if typ not in abi.MODEL_NAMES:
        raise CaseError(f"Unknown constitutiveEq type {typ}; valid: {sorted(abi.MODEL_NAMES)}")
    lam_key = {"Rolie-PolyLog": "lambdaD", "XPomPomLog": "lambdaB"}.get(typ, "lambda")
    for key in ("rho", "etaS", "etaP", "stabilization", lam_key) + MODEL_KEYS.get(typ, ()):
        if key not in par:   # constitutiveEq's lookups (constitutiveEq.C:435-438 for stabilization)
            raise CaseError(f"keyword {key} is undefined in constitutiveProperties")
    mkw: Dict[str, Any] = dict(type=typ, rho=scalar(par["rho"]), etaS=scalar(par["etaS"]), etaP=scalar(par["etaP"]),
                               stabilization=par["stabilization"])
    mkw["lambda_"] = scalar(par[lam_key])
    for k in ("alpha", "epsilon", "zeta", "L2", "lambdaR", "beta", "delta", "chiMax", "lambdaS", "q", "n", "K",
              "a"):
        if k in par:
            mkw[k] = scalar(par[k])
    if typ == "WhiteMetznerCYLog":
        # WhiteMetznerCYLog.C:140-149: the log form only when m = n, K = L, a = b
        for x, y in (("m", "n"), ("K", "L"), ("a", "b")):
            if scalar(par[x]) != scalar(par[y]):
                raise CaseError("The Log version of the WhiteMetznerCY model can only be used if m=n and K=L and "
                                "a=b; use the stress version (WhiteMetznerCY)")
    names = THERMO_KEYS.get(typ, ("thermoLambda", None, "thermoEta"))
    for attr, th in zip(("thermoLambda", "thermoLambda2", "thermoEta"), names):
        # thermoFunction::New (newThermoFunction.C:33-61): no sub-dictionary
        # means the Constant (isothermal) function
        t = par.get(th) if th else None
        if not isinstance(t, dict):
            continue
        ttype = t.get("type")
        if ttype not in THERMO_ARGS:
            raise CaseError(f"Unknown thermoFunction type {ttype} ({th}); valid: {sorted(THERMO_ARGS)}")
        args = {}
        for key in THERMO_ARGS[ttype]:
            if key not in t:
                raise CaseError(f"keyword {key} is undefined in {th}")
            args[key] = scalar(t[key])
        mkw[attr] = ThermoFunction(ttype, **args)
    if "destructionFunctionType" in par:
        mkw["destructionFunctionType"] = par["destructionFunctionType"]
        dft = par["destructionFunctionType"]
        if typ == "PTTLog" and dft not in ("linear", "exponential", "generalized"):
            raise CaseError(f"PTTLog destructionFunctionType {dft}; valid: exponential, generalized, linear")
        if typ == "PTTLog" and dft == "generalized":
            # PTTLog.C:143-152: the Mittag-Leffler alpha and beta, both positive
            for key in ("alpha", "beta"):
                if key not in par:
                    raise CaseError(f"keyword {key} is undefined in constitutiveProperties")
            if scalar(par["alpha"]) <= 0 or scalar(par["beta"]) <= 0:
                raise CaseError("Both alpha and beta should be positive values for the Mittag-Leffler function "
                                "to converge.")
            for key, cast in (("rTolMittagLeffler", float), ("maxIterMittagLeffler", int)):
                if key in par:
                    mkw[key] = cast(scalar(par[key]))
    return Model(**mkw)


def load_case(case_dir: str, substitute: bool = False,
              bc_overrides: Optional[Dict[str, Dict[str, Tuple[str, Any]]]] = None,
              precision: int = abi.RT_PREC_FP64, thermo: bool = False) -> LoadedCase:
    subs: List[str] = []
    mesh = foam_io.read_polymesh(case_dir)
    q = foam_io.mesh_quality(mesh)
    if q["nonOrthogonality"] > 1e-6:
        # the laplacian and face gradients are the orthogonal ones (no
        # non-orthogonal correction): exact only on orthogonal meshes
        msg = f"mesh non-orthogonality {q['nonOrthogonality']:.3g} deg: orthogonal laplacian used"
        if not substitute:
            raise CaseError(msg + " (pass substitute=True to run it anyway)")
        subs.append(msg)
    cp = read_dict(os.path.join(case_dir, "constant", "constitutiveProperties"))
    mode_names, models = read_mode_entries(cp.get("parameters", cp))
    model = models[0]
    if not thermo:
        # rheoFoam has no temperature field: a thermoFunction other than
        # Constant needs the non-isothermal solver's T (thermoFunctions look it
        # up in the mesh, e.g. Arrhenius.C:56)
        for m in models:
            for attr in ("thermoLambda", "thermoLambda2", "thermoEta"):
                f = getattr(m, attr)
                if f.type != "Constant":
                    raise CaseError(f"{attr} type {f.type}: rheoFoam has no temperature field T (load with "
                                    "thermo=True and give T to Context.set_temperature for constitutive "
                                    "corrections)")

    sol = read_dict(os.path.join(case_dir, "system", "fvSolution"))
    solvers = sol.get("solvers", {})
    simple = sol.get("SIMPLE", {})
    nNonOrth = int(scalar(simple.get("nNonOrthogonalCorrectors", "0")))
    relax = sol.get("relaxationFactors", {})
    for group in ("fields", "equations"):
        for k, v in (relax.get(group, {}) or {}).items():
            if isinstance(v, str) and scalar(v) != 1.0:
                if not substitute:
                    raise CaseError(f"relaxationFactors {group} {k} {v}: only 1 (no relaxation) is implemented")
                subs.append(f"relaxationFactors {group} {k}: {v} -> 1")
    sch = read_dict(os.path.join(case_dir, "system", "fvSchemes"))
    ddt_words = sch.get("ddtSchemes", {}).get("default", "Euler").split()
    ddt, ddtPsi = ddt_words[0], 1.0
    if ddt == "CrankNicolson":
        # "CrankNicolson psi": the off-centering coefficient (1: Crank-Nicolson)
        ddtPsi = scalar(ddt_words[1]) if len(ddt_words) > 1 else 1.0
    elif ddt != "Euler":
        if not substitute:
            raise CaseError(f"fvSchemes ddt {ddt} is not implemented (Euler, CrankNicolson); pass substitute=True "
                            "for Euler")
        subs.append(f"ddt: {ddt} -> Euler")
        ddt = "Euler"
    ctrl = read_dict(os.path.join(case_dir, "system", "controlDict"))

    # boundary conditions and initial fields
    ncomp = {"U": 3, "p": 1, "theta": 6, "tau": 6}
    kinds = {"fixedValue", "zeroGradient", "linearExtrapolation"}
    bcs: Dict[str, Dict[str, Tuple[str, Any]]] = {p.name: {} for p in mesh.patches}
    f = Fields.zeros(mesh, len(models))
    for name, nc in ncomp.items():
        # multiMode: theta and tau per mode (theta<K>, tau<K>); the boundary
        # conditions are the first mode's, the others' must be the same
        files = [name + k for k in mode_names] if (mode_names and name in ("theta", "tau")) else [name]
        bf = None
        for i, fname in enumerate(files):
            internal, bfi = foam_io.read_field(os.path.join(case_dir, "0", fname), n_internal=mesh.nCells)
            arr = np.asarray(internal, dtype=np.float64).reshape(mesh.nCells, nc) if nc > 1 else np.asarray(internal)
            if len(files) > 1:
                getattr(f.modes[i], name)[:] = arr
                if name == "theta" and i == 0:
                    f.theta[:] = arr
                if name == "tau":
                    f.tau[:] += arr
            else:
                getattr(f, name)[:] = arr
            if bf is None:
                bf = bfi
            elif _bc_signature(bfi, mesh) != _bc_signature(bf, mesh):
                raise CaseError(f"0/{fname}: multiMode modes with different boundary conditions are not "
                                f"implemented (0/{files[0]} gives the others')")
        for p in mesh.patches:
            e = lookup_pattern(bf, p.name)
            if e is None:
                raise CaseError(f"0/{name}: no boundary condition for patch {p.name}")
            typ_b = e["type"]
            val = None
            if e["value"] is not None:
                v = np.asarray(e["value"], dtype=np.float64)
                val = np.broadcast_to(v.reshape(-1, nc) if v.size != nc else v.reshape(1, nc), (p.size, nc)).copy()
            ov = (bc_overrides or {}).get(p.name, {}).get(name)
            if ov is not None:
                bcs[p.name][name] = ov
                continue
            if typ_b == "codedFixedValue":
                if not substitute:
                    raise CaseError(f"0/{name} patch {p.name}: codedFixedValue cannot run here; give bc_overrides "
                                    "or pass substitute=True to use its value entry")
                subs.append(f"0/{name} {p.name}: codedFixedValue -> fixedValue (its value entry)")
                typ_b = "fixedValue"
            if typ_b not in kinds:
                raise CaseError(f"0/{name} patch {p.name}: boundary type {typ_b!r} is not implemented "
                                f"({sorted(kinds)})")
            if typ_b == "fixedValue":
                if val is None:
                    raise CaseError(f"0/{name} patch {p.name}: fixedValue without a value")
                bcs[p.name][name] = ("fixedValue", val)
            else:
                bcs[p.name][name] = (typ_b, None)
    case = Case(mesh, model, bcs, deltaT=scalar(ctrl.get("deltaT", "1e-3")),
                divU=_limiter(sch, "div(phi,U)"), divTheta=_limiter(sch, "div(phi,theta)"),
                solverU=_solver(solvers, "U", subs, substitute), solverP=_solver(solvers, "p", subs, substitute),
                solverTheta=_solver(solvers, "theta", subs, substitute),
                pRefCell=int(scalar(simple.get("pRefCell", "0"))), pRefValue=scalar(simple.get("pRefValue", "0")),
                precision=precision, name=os.path.basename(os.path.abspath(case_dir)),
                nInIter=int(scalar(simple.get("nInIter", "1"))), nNonOrthCorr=nNonOrth, ddt=ddt, ddtPsi=ddtPsi)
    case.moreModes = list(models[1:])
    # boundary values of the initial state (fixed values; the rest from the cells)
    holders = [f] + list(f.modes)
    for p in mesh.patches:
        sl = slice(p.start, p.start + p.size)
        for name, nc in ncomp.items():
            kind, val = case.bcs[p.name][name]
            for h in (holders if name in ("theta", "tau") else [f]):
                bnd = getattr(h, name + "b")
                cells = getattr(h, name)[mesh.bCell[sl]]
                if kind == "fixedValue" and val is not None:
                    v = np.asarray(val(mesh.bCf[sl]) if callable(val) else val, dtype=np.float64)
                    bnd[sl] = np.broadcast_to(v.reshape(-1, nc) if nc > 1 else v.reshape(-1), bnd[sl].shape)
                else:
                    bnd[sl] = cells
    if f.modes:   # the summed tau on the boundary too (multiMode::tau())
        f.taub[:] = sum(m.taub for m in f.modes)
    # initial face fluxes from U (createPhi)
    Uf = mesh.w[:, None] * (f.U[mesh.owner] - f.U[mesh.neighbour]) + f.U[mesh.neighbour]
    f.phi[:] = (mesh.Sf * Uf).sum(1)
    f.phib[:] = (mesh.bSf * f.Ub).sum(1)
    return LoadedCase(case, f, scalar(ctrl.get("endTime", "1")), scalar(ctrl.get("writeInterval", "1")), subs,
                      mode_names)


def run_case(case_dir: str, steps: Optional[int] = None, device: int = 0, log=None, **load_kw) -> LoadedCase:
    """Load the case, step it on the GPU to endTime (or `steps` steps) and
    write the fields at every write time and at the end.  log (a text
    stream, or None): the run's solver log in OpenFOAM's format, one step
    at a time (foam_log)."""
    import time as _time

    from .foam_log import FoamLog
    from .runtime import Context
    if load_kw.get("thermo"):
        raise CaseError("run_case steps rheoFoam, which has no temperature field: temperature-dependent "
                        "parameters apply to constitutive corrections (Context.set_temperature) only")
    lc = load_case(case_dir, **load_kw)
    case = lc.case
    dt = case.deltaT
    n = steps if steps is not None else int(round(lc.endTime / dt))
    every = max(1, int(round(lc.writeInterval / dt)))
    with Context(device) as ctx:
        ctx.setup_case(case, lc.fields)
        done = 0
        flog = FoamLog(case) if log is not None else None
        t0 = _time.perf_counter()
        while done < n:
            k = min(every, n - done)
            if flog is None:
                ctx.step(k)
            else:
                for j in range(k):
                    perf = ctx.step(1)
                    lines = flog.step((done + j + 1) * dt, perf, _time.perf_counter() - t0)
                    log.write("\n".join(lines) + "\n")
            done += k
            t = done * dt
            tdir = os.path.join(case_dir, f"{t:g}")
            got = ctx.fields()
            foam_io.write_fields(tdir, case.mesh, got)
            for k, m in zip(lc.mode_names, got.modes):   # multiMode: every mode's theta and tau
                for name, a, b, dims in (("theta", m.theta, m.thetab, "[0 0 0 0 0 0 0]"),
                                         ("tau", m.tau, m.taub, "[1 -1 -2 0 0 0 0]")):
                    bnd = {p.name: ("calculated", b[p.start:p.start + p.size]) for p in case.mesh.patches}
                    foam_io.write_field(os.path.join(tdir, name + k), "volSymmTensorField", name + k, a, bnd, dims,
                                        os.path.basename(tdir), 12)
    return lc


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("case_dir")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--substitute", action="store_true")
    ap.add_argument("--mixed", action="store_true", help="the mixed-precision form")
    ap.add_argument("--log", action="store_true", help="print the solver log in OpenFOAM's format")
    a = ap.parse_args(argv)
    import sys
    lc = run_case(a.case_dir, steps=a.steps, device=a.device, substitute=a.substitute,
                  precision=abi.RT_PREC_MIXED if a.mixed else abi.RT_PREC_FP64, log=sys.stdout if a.log else None)
    for s in lc.substitutions:
        print("substituted:", s)


if __name__ == "__main__":
    main()
