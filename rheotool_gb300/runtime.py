"""Host-side API over the C ABI (librheogpu.so).

``Context`` owns one device context: a mesh, a case and the device-resident
fields.  The higher-level classes mirror the two reference seams:

* ``ConstitutiveEq.New(name, case)`` + ``correct()`` / ``tau()`` —
  rheoTool's ``constitutiveEq`` run-time selection (``constitutiveEq.H:250-347``);
* ``LduSolver.New(fieldName, ctl)`` + ``solve(psi, source, cmpt)`` —
  OpenFOAM's ``lduMatrix::solver`` selected by ``solver``/``preconditioner``,
  returning a ``solverPerformance``-like record.

Every call goes to the CUDA library; a missing library or device is an error.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import abi
from .case import Case, Fields, SolverControl


class RheoGpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


class Context:
    """One device context (one stream, one mesh, one case)."""

    def __init__(self, device: int = 0):
        self.lib = abi.load_library()
        self._ctx = C.c_void_p()
        st = self.lib.rt_ctx_create(C.byref(self._ctx), int(device))
        if st != 0:
            raise RheoGpuError(st, "rt_ctx_create failed (no CUDA device?)")
        self.mesh = None
        self.case: Optional[Case] = None

    # ------------------------------------------------------------------
    def _check(self, st: int, what: str):
        if st != 0:
            msg = self.lib.rt_last_error(self._ctx)
            raise RheoGpuError(st, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if self._ctx:
            self.lib.rt_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------
    def upload_mesh(self, mesh):
        self.mesh = mesh
        from .case import Case as _Case  # noqa: F401
        md = _mesh_desc(mesh, self)
        self._check(self.lib.rt_mesh_upload(self._ctx, C.byref(md)), "rt_mesh_upload")
        ijk = getattr(mesh, "cellIJK", None)
        if ijk is not None and getattr(mesh, "shape", None) is not None:
            nx, ny, nz = mesh.shape
            a = np.ascontiguousarray(ijk, dtype=np.int32)
            self._check(self.lib.rt_mesh_set_ijk(self._ctx, nx, ny, nz, abi.iptr(a)), "rt_mesh_set_ijk")

    def set_option(self, option: int, value: int):
        self._check(self.lib.rt_set_option(self._ctx, int(option), int(value)), "rt_set_option")

    def set_sweep(self, mode: int):
        """abi.SWEEP_AUTO / SWEEP_LEVELS / SWEEP_SYSTOLIC for the DIC/DILU sweeps."""
        self.set_option(abi.RT_OPT_SWEEP, mode)

    def sweep_schedule(self) -> dict:
        """The tuned schedules of the one-component systolic sweeps."""
        a = np.zeros(6, np.int32)
        self._check(self.lib.rt_sweep_schedule(self._ctx, abi.iptr(a)), "rt_sweep_schedule")
        return {"fp64": {"candidate": int(a[0]), "P": int(a[1]), "NB": int(a[2])},
                "fp32": {"candidate": int(a[3]), "P": int(a[4]), "NB": int(a[5])}}

    def set_precision(self, precision: int):
        """abi.RT_PREC_FP64 / RT_PREC_MIXED for standalone ldu_solve calls
        (the time step takes its precision from the case control)."""
        self.set_option(abi.RT_OPT_PRECISION, precision)

    def setup_case(self, case: Case, fields: Optional[Fields] = None):
        if self.mesh is not case.mesh:
            self.upload_mesh(case.mesh)
        self.case = case
        _, bd, mp, ctl = case.descriptors()
        if len(case.models) > 1:
            self._check(self.lib.rt_case_setup_modes(self._ctx, C.byref(bd), case.mode_params(), len(case.models),
                                                     C.byref(ctl)), "rt_case_setup_modes")
        else:
            self._check(self.lib.rt_case_setup(self._ctx, C.byref(bd), C.byref(mp), C.byref(ctl)), "rt_case_setup")
        if fields is not None:
            self.set_fields(fields)

    @property
    def nModes(self) -> int:
        return len(self.case.models) if self.case is not None else 1

    def set_field(self, fid: int, internal=None, boundary=None):
        i = None if internal is None else _c(internal)
        b = None if boundary is None else _c(boundary)
        self._check(self.lib.rt_field_set(self._ctx, fid, abi.optr(i), abi.optr(b)), "rt_field_set")

    def get_field(self, fid: int, shape_in, shape_b=None):
        i = np.zeros(shape_in)
        b = None if shape_b is None else np.zeros(shape_b)
        self._check(self.lib.rt_field_get(self._ctx, fid, abi.dptr(i), abi.optr(b)), "rt_field_get")
        return i, b

    def set_fields(self, f: Fields):
        self.set_field(abi.RT_FIELD_U, f.U, f.Ub)
        self.set_field(abi.RT_FIELD_P, f.p, f.pb)
        self.set_field(abi.RT_FIELD_PHI, f.phi, f.phib)
        if f.modes:
            for i, m in enumerate(f.modes):
                for fid, a, b in ((abi.RT_FIELD_THETA, m.theta, m.thetab), (abi.RT_FIELD_TAU, m.tau, m.taub),
                                  (abi.RT_FIELD_EIGVALS, m.eigVals, None), (abi.RT_FIELD_EIGVECS, m.eigVecs, None)):
                    self._check(self.lib.rt_field_set_mode(self._ctx, fid, i, abi.optr(_c(a)),
                                                           abi.optr(None if b is None else _c(b))),
                                "rt_field_set_mode")
            self.set_field(abi.RT_FIELD_TAU, f.tau, f.taub)     # the summed tau
            return
        self.set_field(abi.RT_FIELD_THETA, f.theta, f.thetab)
        self.set_field(abi.RT_FIELD_TAU, f.tau, f.taub)
        self.set_field(abi.RT_FIELD_EIGVALS, f.eigVals)
        self.set_field(abi.RT_FIELD_EIGVECS, f.eigVecs)

    def fields(self) -> Fields:
        m = self.mesh
        N, nF, nB = m.nCells, m.nFaces, m.nBFaces
        U, Ub = self.get_field(abi.RT_FIELD_U, (N, 3), (nB, 3))
        p, pb = self.get_field(abi.RT_FIELD_P, (N,), (nB,))
        phi, phib = self.get_field(abi.RT_FIELD_PHI, (nF,), (nB,))
        th, thb = self.get_field(abi.RT_FIELD_THETA, (N, 6), (nB, 6))
        ta, tab = self.get_field(abi.RT_FIELD_TAU, (N, 6), (nB, 6))
        ev, _ = self.get_field(abi.RT_FIELD_EIGVALS, (N, 3))
        vv, _ = self.get_field(abi.RT_FIELD_EIGVECS, (N, 9))
        f = Fields(U, Ub, p, pb, phi, phib, th, thb, ta, tab, ev, vv)
        if self.nModes > 1:
            from .case import ModeFields
            for i in range(self.nModes):
                m = ModeFields.zeros(self.mesh)
                for fid, a, b in ((abi.RT_FIELD_THETA, m.theta, m.thetab), (abi.RT_FIELD_TAU, m.tau, m.taub),
                                  (abi.RT_FIELD_EIGVALS, m.eigVals, None), (abi.RT_FIELD_EIGVECS, m.eigVecs, None)):
                    self._check(self.lib.rt_field_get_mode(self._ctx, fid, i, abi.dptr(a), abi.optr(b)),
                                "rt_field_get_mode")
                f.modes.append(m)
        return f

    def mode_perf(self) -> List[List[abi.rt_solver_perf]]:
        """Every mode's theta solve records of the last correct() (multiMode)."""
        n = self.nModes
        perf = (abi.rt_solver_perf * (6 * n))()
        self._check(self.lib.rt_mode_perf(self._ctx, perf), "rt_mode_perf")
        return [list(perf[6 * i:6 * i + 6]) for i in range(n)]

    # ------------------------------------------------------------------
    def step(self, n: int = 1) -> abi.rt_step_perf:
        perf = abi.rt_step_perf()
        self._check(self.lib.rt_step(self._ctx, int(n), C.byref(perf)), "rt_step")
        return perf

    def constitutive_correct(self, gradU=None, newTimeStep: Optional[bool] = None) -> List[abi.rt_solver_perf]:
        """One constitutiveEq::correct().  newTimeStep None: a step of its own
        (rt_constitutive_correct); True / False: the first / a further inner
        iteration of a time step, solved against the theta kept by the first
        (rt_constitutive_correct_iter)."""
        perf = (abi.rt_solver_perf * 6)()
        g = None if gradU is None else _c(gradU)
        if newTimeStep is None:
            self._check(self.lib.rt_constitutive_correct(self._ctx, abi.optr(g), perf), "rt_constitutive_correct")
        else:
            self._check(self.lib.rt_constitutive_correct_iter(self._ctx, abi.optr(g), int(bool(newTimeStep)), perf),
                        "rt_constitutive_correct_iter")
        return list(perf)

    def set_temperature(self, T=None):
        """The cell temperatures T (nCells) for the case's thermo functions
        (each mode's thermoLambda, thermoLambda2, thermoEta): every later
        constitutive_correct shifts the relaxation times and etaP as a
        non-isothermal solver's constEq.correct() does (rt_set_temperature).
        None: the isothermal case again."""
        if T is None:
            self._check(self.lib.rt_set_temperature(self._ctx, None, None), "rt_set_temperature")
            return
        if self.case is None:
            raise ValueError("set up a case first")
        t = _c(T)
        self._check(self.lib.rt_set_temperature(self._ctx, self.case.thermo_descs(), abi.dptr(t)),
                    "rt_set_temperature")

    def ldu_solve(self, diag, upper, lower, source, psi, ctl) -> List[abi.rt_solver_perf]:
        """Solve nc = source.shape[0] systems sharing one matrix; psi (nc, N) is
        updated in place."""
        source = np.atleast_2d(_c(source))
        assert psi.dtype == np.float64 and psi.flags.c_contiguous
        psi2 = psi.reshape(source.shape)
        nc = source.shape[0]
        perf = (abi.rt_solver_perf * nc)()
        c = ctl.to_c() if hasattr(ctl, "to_c") else ctl
        st = self.lib.rt_ldu_solve(self._ctx, abi.dptr(_c(diag)), abi.dptr(_c(upper)), abi.dptr(_c(lower)),
                                   abi.dptr(source), abi.dptr(psi2), nc, C.byref(c), perf)
        if st not in (0, abi.RT_ENOCONV):
            self._check(st, "rt_ldu_solve")
        return list(perf)

    def residual(self, diag, upper, lower, source, psi) -> float:
        r = C.c_double()
        self._check(self.lib.rt_residual(self._ctx, abi.dptr(_c(diag)), abi.dptr(_c(upper)), abi.dptr(_c(lower)),
                                         abi.dptr(_c(source)), abi.dptr(_c(psi)), C.byref(r)), "rt_residual")
        return r.value

    def grad(self, psi, psib) -> np.ndarray:
        g = np.zeros((self.mesh.nCells, 3))
        self._check(self.lib.rt_op_grad(self._ctx, abi.dptr(_c(psi)), abi.dptr(_c(psib)), abi.dptr(g)), "rt_op_grad")
        return g

    def eig(self, theta):
        theta = _c(theta)
        n = theta.shape[0]
        ev = np.zeros((n, 3))
        vv = np.zeros((n, 9))
        self._check(self.lib.rt_op_eig(self._ctx, n, abi.dptr(theta), abi.dptr(ev), abi.dptr(vv)), "rt_op_eig")
        return ev, vv

    def sync(self):
        self._check(self.lib.rt_sync(self._ctx), "rt_sync")

    # ---- timing on the context stream ---------------------------------
    def timer_start(self):
        self._check(self.lib.rt_timer_start(self._ctx), "rt_timer_start")

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._check(self.lib.rt_timer_stop(self._ctx, C.byref(ms)), "rt_timer_stop")
        return ms.value

    def profile(self, on: bool):
        self._check(self.lib.rt_profile_enable(self._ctx, int(bool(on))), "rt_profile_enable")

    def profile_report(self) -> dict:
        """{name: (launches, device_ms, algorithmic_bytes)} since the last report."""
        buf = C.create_string_buffer(1 << 16)
        self._check(self.lib.rt_profile_report(self._ctx, buf, len(buf)), "rt_profile_report")
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms, by = line.split()
            out[name] = (int(n), float(ms), float(by))
        return out

    def kernel_count(self) -> int:
        n = C.c_int64()
        self._check(self.lib.rt_kernel_count(self._ctx, C.byref(n)), "rt_kernel_count")
        return n.value


def _mesh_desc(mesh, keeper) -> abi.rt_mesh_desc:
    keep = []

    def d(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return abi.dptr(a)

    def i(a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        keep.append(a)
        return abi.iptr(a)

    md = abi.rt_mesh_desc()
    md.nCells, md.nFaces, md.nBFaces, md.nPatches = mesh.nCells, mesh.nFaces, mesh.nBFaces, len(mesh.patches)
    md.owner, md.neighbour = i(mesh.owner), i(mesh.neighbour)
    md.Sf, md.magSf, md.Cf = d(mesh.Sf), d(mesh.magSf), d(mesh.Cf)
    md.weights, md.deltaCoeffs = d(mesh.w), d(mesh.deltaCoeffs)
    md.C, md.V = d(mesh.C), d(mesh.V)
    md.bCell, md.bSf, md.bmagSf, md.bCf, md.bDeltaCoeffs = (i(mesh.bCell), d(mesh.bSf), d(mesh.bmagSf),
                                                           d(mesh.bCf), d(mesh.bDelta))
    md.patchStart = i(np.array([p.start for p in mesh.patches] or [0]))
    md.patchSize = i(np.array([p.size for p in mesh.patches] or [0]))
    for k in range(3):
        md.solveDir[k] = int(mesh.solveDir[k])
    if getattr(mesh, "delta", None) is not None:
        md.delta = d(mesh.delta)
    if getattr(mesh, "coupled", None) is not None:
        md.coupled = i(mesh.coupled)
    keeper._mesh_keep = keep
    return md


# ---------------------------------------------------------------------------
# Reference-facing seams
# ---------------------------------------------------------------------------
class ConstitutiveEq:
    """GPU constitutive model behind rheoTool's constitutiveEq API.

    ``New(name, case)`` selects by ``case.model.type`` (``Oldroyd-BLog``,
    ``GiesekusLog``, ``PTTLog``, ``FENE-PLog``, ``FENE-CRLog``,
    ``Rolie-PolyLog``, ``XPomPomLog``, ``WhiteMetznerCYLog``), exactly as
    ``constitutiveEq::New`` does from ``constitutiveProperties``; an unknown
    type raises like the reference's FatalError (``newConstitutiveEq.C:47-58``).
    """

    def __init__(self, name: str, ctx: Context):
        self.name = name
        self.ctx = ctx

    @staticmethod
    def New(name: str, case: Case, ctx: Optional[Context] = None) -> "ConstitutiveEq":
        if case.model.type not in abi.MODEL_NAMES:
            raise ValueError(f"Unknown constitutiveEq type {case.model.type}\n\nValid constitutiveEqs are : "
                             f"{sorted(abi.MODEL_NAMES)}")
        ctx = ctx or Context()
        if ctx.case is not case:
            ctx.setup_case(case)
        return ConstitutiveEq(name, ctx)

    def correct(self, gradU=None):
        return self.ctx.constitutive_correct(gradU)

    def tau(self) -> np.ndarray:
        return self.ctx.get_field(abi.RT_FIELD_TAU, (self.ctx.mesh.nCells, 6))[0]

    def rho(self) -> float:
        return self.ctx.case.model.rho

    def isGNF(self) -> bool:
        return False


@dataclass
class SolverPerformance:
    solverName: str
    fieldName: str
    initialResidual: float
    finalResidual: float
    nIterations: int
    converged: bool
    singular: bool


class LduSolver:
    """lduMatrix::solver stand-in: PCG (+DIC/diagonal/none), PBiCGStab and
    PBiCG (+DILU/diagonal/none) on the context's mesh addressing."""

    def __init__(self, fieldName: str, ctl: SolverControl, ctx: Context):
        self.fieldName = fieldName
        self.ctl = ctl
        self.ctx = ctx

    @staticmethod
    def New(fieldName: str, ctl: SolverControl, ctx: Context) -> "LduSolver":
        if ctl.solver not in ("PCG", "PBiCGStab", "PBiCG"):
            raise ValueError(f"Unknown asymmetric matrix solver {ctl.solver}")
        return LduSolver(fieldName, ctl, ctx)

    def solve(self, diag, upper, lower, psi, source) -> List[SolverPerformance]:
        perf = self.ctx.ldu_solve(diag, upper, lower, source, psi, self.ctl)
        return [SolverPerformance(self.ctl.solver, self.fieldName, p.initialResidual, p.finalResidual,
                                  p.nIterations, bool(p.converged), bool(p.singular)) for p in perf]
