"""ctypes binding of the FP64 CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, as the oracle the library is compared against.  The
product (rheotool_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from rheotool_gb300 import abi
from rheotool_gb300.case import Case, Fields

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

_dp = C.POINTER(C.c_double)


class or_state(C.Structure):
    _fields_ = [(n, _dp) for n in ("U", "Ub", "p", "pb", "phi", "phib", "theta", "thetab",
                                   "tau", "taub", "eigVals", "eigVecs")]


class or_ddt(C.Structure):
    _fields_ = [("scheme", C.c_int), ("psi", C.c_double), ("nSteps", C.c_int), ("nThSteps", C.c_int)] + \
               [(n, _dp) for n in ("DU", "DUb", "Dphi", "Dphib", "Dth", "Us", "Ubs", "phis", "phibs", "ths")]


def build(force: bool = False) -> str:
    deps = (os.path.join(HERE, "oracle.c"), os.path.join(HERE, "..", "include", "rheogpu.h"))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(d) for d in deps):
        subprocess.check_call(["make", "-s", "-C", HERE, "-B" if force else "liboracle.so"])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        L.or_set_threads.argtypes = [C.c_int]
        L.or_grad.argtypes = [P(abi.rt_mesh_desc), _dp, _dp, _dp]
        L.or_ldu_solve.argtypes = [P(abi.rt_mesh_desc), _dp, _dp, _dp, _dp, _dp,
                                   P(abi.rt_solver_ctl), P(abi.rt_solver_perf)]
        L.or_ldu_solve.restype = C.c_int
        L.or_residual.argtypes = [P(abi.rt_mesh_desc), _dp, _dp, _dp, _dp, _dp]
        L.or_residual.restype = C.c_double
        L.or_eig.argtypes = [C.c_int, _dp, _dp, _dp]
        L.or_eig3.argtypes = [_dp, _dp, _dp]
        L.or_constitutive_correct.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc),
                                              P(abi.rt_model_params), P(abi.rt_case_ctl),
                                              P(or_state), _dp, P(abi.rt_solver_perf)]
        L.or_constitutive_correct.restype = C.c_int
        L.or_constitutive_correct_old.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc),
                                                  P(abi.rt_model_params), P(abi.rt_case_ctl),
                                                  P(or_state), _dp, _dp, P(abi.rt_solver_perf)]
        L.or_constitutive_correct_old.restype = C.c_int
        L.or_theta_source.argtypes = [P(abi.rt_model_params), C.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.or_tau_cells.argtypes = [P(abi.rt_model_params), C.c_int, _dp, _dp, _dp, _dp]
        L.or_step.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc), P(abi.rt_model_params),
                              P(abi.rt_case_ctl), P(or_state), C.c_int, P(abi.rt_step_perf)]
        L.or_step.restype = C.c_int
        L.or_init_fields.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc), P(or_state)]
        L.or_step_modes.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc), P(abi.rt_model_params), C.c_int,
                                    P(abi.rt_case_ctl), P(or_state), P(or_state), C.c_int, P(abi.rt_step_perf),
                                    P(abi.rt_solver_perf)]
        L.or_step_modes.restype = C.c_int
        L.or_constitutive_correct_modes.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc), P(abi.rt_model_params),
                                                    C.c_int, P(abi.rt_case_ctl), P(or_state), P(or_state), _dp,
                                                    P(abi.rt_solver_perf)]
        L.or_constitutive_correct_modes.restype = C.c_int
        L.or_step_ddt.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc), P(abi.rt_model_params), C.c_int,
                                  P(abi.rt_case_ctl), P(or_state), P(or_state), C.c_int, P(abi.rt_step_perf),
                                  P(abi.rt_solver_perf), P(or_ddt)]
        L.or_step_ddt.restype = C.c_int
        L.or_constitutive_correct_ddt.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc), P(abi.rt_model_params),
                                                  C.c_int, P(abi.rt_case_ctl), P(or_state), P(or_state), _dp, C.c_int,
                                                  P(abi.rt_solver_perf), P(or_ddt)]
        L.or_constitutive_correct_ddt.restype = C.c_int
        L.or_thermo_factor.argtypes = [P(abi.rt_thermo_fn), C.c_double]
        L.or_thermo_factor.restype = C.c_double
        L.or_thermo_factors.argtypes = [P(abi.rt_thermo_desc), C.c_int, _dp, _dp]
        L.or_constitutive_correct_thermo.argtypes = [P(abi.rt_mesh_desc), P(abi.rt_bc_desc), P(abi.rt_model_params),
                                                     C.c_int, P(abi.rt_case_ctl), P(or_state), P(or_state), _dp,
                                                     P(abi.rt_thermo_desc), _dp, P(abi.rt_solver_perf)]
        L.or_constitutive_correct_thermo.restype = C.c_int
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def _state(f: Fields) -> or_state:
    s = or_state()
    for name, _ in or_state._fields_:
        a = getattr(f, name)
        assert a.dtype == np.float64 and a.flags.c_contiguous, name
        setattr(s, name, a.ctypes.data_as(_dp))
    return s


def _mode_states(f: Fields):
    """or_state array of a multiMode state's modes (their U, p and phi
    pointers are the common fields')."""
    arr = (or_state * len(f.modes))()
    base = _state(f)
    for i, m in enumerate(f.modes):
        st = or_state()
        for name, _ in or_state._fields_:
            a = getattr(m, name, None)
            if a is None:
                setattr(st, name, getattr(base, name))
            else:
                assert a.dtype == np.float64 and a.flags.c_contiguous, name
                setattr(st, name, a.ctypes.data_as(_dp))
        arr[i] = st
    return arr


class Oracle:
    """FP64 CPU restatement of one case (same Case object as the GPU path)."""

    def __init__(self, case: Case, fields: Fields = None):
        self.case = case
        self.md, self.bd, self.mp, self.ctl = case.descriptors()
        self.nModes = len(case.models)
        self.models = case.mode_params()
        self.f = fields if fields is not None else Fields.zeros(case.mesh, self.nModes)
        if fields is None:
            lib().or_init_fields(C.byref(self.md), C.byref(self.bd), C.byref(_state(self.f)))
            if self.nModes > 1:
                # every mode starts from the boundary values of theta and tau;
                # the summed tau's boundary values are the modes' sum
                for m in self.f.modes:
                    m.thetab[...] = self.f.thetab
                    m.taub[...] = self.f.taub
                self.f.taub[...] = sum(m.taub for m in self.f.modes)
        self.modePerf = (abi.rt_solver_perf * (6 * self.nModes))()
        # Crank-Nicolson: the old-time derivatives and start-of-step fields
        self.cn = case.ddt == "CrankNicolson"
        if self.cn:
            m = case.mesh
            N, nF, nB = m.nCells, m.nFaces, m.nBFaces
            z = np.zeros
            self._ddt_arrays = {"DU": z(3 * N), "DUb": z(3 * nB), "Dphi": z(nF), "Dphib": z(nB),
                                "Dth": z(6 * N * self.nModes), "Us": z(3 * N), "Ubs": z(3 * nB), "phis": z(nF),
                                "phibs": z(nB), "ths": z(6 * N * self.nModes)}
            self.ddt = or_ddt(abi.RT_DDT_CRANKNICOLSON, case.ddtPsi, 0, 0,
                              *[self._ddt_arrays[n].ctypes.data_as(_dp) for n, _ in or_ddt._fields_[4:]])

    def step(self, n: int = 1) -> abi.rt_step_perf:
        perf = abi.rt_step_perf()
        if self.cn:
            modes = _mode_states(self.f) if self.nModes > 1 else None
            st = lib().or_step_ddt(C.byref(self.md), C.byref(self.bd), self.models, self.nModes,
                                   C.byref(self.ctl), C.byref(_state(self.f)), modes, int(n), C.byref(perf),
                                   self.modePerf, C.byref(self.ddt))
        elif self.nModes > 1:
            st = lib().or_step_modes(C.byref(self.md), C.byref(self.bd), self.models, self.nModes,
                                     C.byref(self.ctl), C.byref(_state(self.f)), _mode_states(self.f), int(n),
                                     C.byref(perf), self.modePerf)
        else:
            st = lib().or_step(C.byref(self.md), C.byref(self.bd), C.byref(self.mp), C.byref(self.ctl),
                               C.byref(_state(self.f)), int(n), C.byref(perf))
        if st != 0:
            raise RuntimeError(f"oracle step failed: {abi.STATUS_NAMES.get(st, st)}")
        self._mode0_view()
        return perf

    def _mode0_view(self):
        """A multiMode state shows mode 0's theta and eigen fields at the top
        level (tau there is the modes' sum)."""
        if self.nModes > 1:
            m0 = self.f.modes[0]
            for name in ("theta", "thetab", "eigVals", "eigVecs"):
                getattr(self.f, name)[...] = getattr(m0, name)

    def constitutive_correct(self, gradU: np.ndarray = None, thetaOld: np.ndarray = None, newTimeStep=None,
                             T: np.ndarray = None):
        """One correct(); thetaOld (nCells, 6): the old-time theta of the
        theta equation (an inner iteration of a step that started there),
        default the current theta.  T (nCells): cell temperatures for the
        modes' thermo functions (a non-isothermal solver's correct())."""
        perf = (abi.rt_solver_perf * 6)()
        g = None if gradU is None else np.ascontiguousarray(gradU, dtype=np.float64)
        gp = None if g is None else g.ctypes.data_as(_dp)
        if T is not None:
            if self.cn or thetaOld is not None:
                raise ValueError("temperature-dependent correct(): Euler, one call a step")
            t = np.ascontiguousarray(T, dtype=np.float64)
            modes = _mode_states(self.f) if self.nModes > 1 else None
            st = lib().or_constitutive_correct_thermo(C.byref(self.md), C.byref(self.bd), self.models, self.nModes,
                                                      C.byref(self.ctl), C.byref(_state(self.f)), modes, gp,
                                                      self.case.thermo_descs(), t.ctypes.data_as(_dp),
                                                      self.modePerf)
            if st != 0:
                raise RuntimeError(f"oracle constitutive correct failed: {st}")
            if self.nModes > 1:
                self._mode0_view()
            return list(self.modePerf[6 * (self.nModes - 1):])
        if self.cn:
            # Crank-Nicolson: a time step of its own unless newTimeStep is
            # False (a further inner iteration, against the theta kept at the
            # start of the step; thetaOld is not used)
            modes = _mode_states(self.f) if self.nModes > 1 else None
            st = lib().or_constitutive_correct_ddt(C.byref(self.md), C.byref(self.bd), self.models, self.nModes,
                                                   C.byref(self.ctl), C.byref(_state(self.f)), modes, gp,
                                                   int(newTimeStep is None or bool(newTimeStep)), self.modePerf,
                                                   C.byref(self.ddt))
            if st != 0:
                raise RuntimeError(f"oracle constitutive correct failed: {st}")
            self._mode0_view()
            return list(self.modePerf[6 * (self.nModes - 1):])
        if self.nModes > 1:
            if thetaOld is not None:
                raise ValueError("multiMode: inner iterations run inside step()")
            st = lib().or_constitutive_correct_modes(C.byref(self.md), C.byref(self.bd), self.models, self.nModes,
                                                     C.byref(self.ctl), C.byref(_state(self.f)),
                                                     _mode_states(self.f), gp, self.modePerf)
            if st != 0:
                raise RuntimeError(f"oracle constitutive correct failed: {st}")
            self._mode0_view()
            return list(self.modePerf[6 * (self.nModes - 1):])
        if thetaOld is None:
            st = lib().or_constitutive_correct(C.byref(self.md), C.byref(self.bd), C.byref(self.mp),
                                               C.byref(self.ctl), C.byref(_state(self.f)), gp, perf)
        else:
            t0 = np.ascontiguousarray(thetaOld, dtype=np.float64)
            st = lib().or_constitutive_correct_old(C.byref(self.md), C.byref(self.bd), C.byref(self.mp),
                                                   C.byref(self.ctl), C.byref(_state(self.f)), gp,
                                                   t0.ctypes.data_as(_dp), perf)
        if st != 0:
            raise RuntimeError(f"oracle constitutive correct failed: {st}")
        return list(perf)

    def grad(self, psi: np.ndarray, psib: np.ndarray) -> np.ndarray:
        g = np.zeros((self.case.mesh.nCells, 3))
        lib().or_grad(C.byref(self.md), abi.dptr(np.ascontiguousarray(psi, dtype=np.float64)),
                      abi.dptr(np.ascontiguousarray(psib, dtype=np.float64)), abi.dptr(g))
        return g

    def ldu_solve(self, diag, upper, lower, source, psi, ctl) -> abi.rt_solver_perf:
        """One-component lduMatrix::solver solve; psi is updated in place."""
        perf = abi.rt_solver_perf()
        c = ctl.to_c() if hasattr(ctl, "to_c") else ctl
        lib().or_ldu_solve(C.byref(self.md), abi.dptr(diag), abi.dptr(upper), abi.dptr(lower),
                           abi.dptr(source), abi.dptr(psi), C.byref(c), C.byref(perf))
        return perf

    def residual(self, diag, upper, lower, source, psi) -> float:
        return lib().or_residual(C.byref(self.md), abi.dptr(diag), abi.dptr(upper),
                                 abi.dptr(lower), abi.dptr(source), abi.dptr(psi))


def eig(theta: np.ndarray):
    """Per-cell calcEig of an (n, 6) symmTensor array -> (exp(mu) (n,3), vecs (n,9))."""
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    n = theta.shape[0]
    vals = np.zeros((n, 3))
    vecs = np.zeros((n, 9))
    lib().or_eig(n, abi.dptr(theta), abi.dptr(vals), abi.dptr(vecs))
    return vals, vecs


def eig3(s) -> tuple:
    s = np.ascontiguousarray(s, dtype=np.float64)
    mu = np.zeros(3)
    V = np.zeros(9)
    lib().or_eig3(abi.dptr(s), abi.dptr(mu), abi.dptr(V))
    return mu, V.reshape(3, 3)


def theta_source(mp: abi.rt_model_params, L, eigVecs, eigVals, theta):
    """The cell-local theta right-hand side of n cells (AoS arrays (n,9),
    (n,9), (n,3), (n,6)) -> (rhs (n,6), fP (n,))."""
    L, eigVecs, eigVals, theta = (np.ascontiguousarray(a, dtype=np.float64) for a in (L, eigVecs, eigVals, theta))
    n = theta.shape[0]
    rhs, fP = np.zeros((n, 6)), np.zeros(n)
    lib().or_theta_source(C.byref(mp), n, abi.dptr(L), abi.dptr(eigVecs), abi.dptr(eigVals), abi.dptr(theta),
                          abi.dptr(rhs), abi.dptr(fP))
    return rhs, fP


def tau_cells(mp: abi.rt_model_params, eigVecs, eigVals, fP):
    """tau (n,6) of n cells from eigVecs (n,9), eigVals (n,3) and fP (n,)."""
    eigVecs, eigVals, fP = (np.ascontiguousarray(a, dtype=np.float64) for a in (eigVecs, eigVals, fP))
    n = eigVals.shape[0]
    tau = np.zeros((n, 6))
    lib().or_tau_cells(C.byref(mp), n, abi.dptr(eigVecs), abi.dptr(eigVals), abi.dptr(fP), abi.dptr(tau))
    return tau
