"""ctypes mirror of ``include/rheogpu.h`` and the loader of ``librheogpu.so``.

The structures below are field-for-field copies of the C declarations; the
library itself is the CUDA build in this package directory.  Loading fails
loudly when the shared object is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBNAME = os.path.join(HERE, "librheogpu.so")

RT_OK, RT_EINVAL, RT_ENOCONV, RT_ENAN, RT_ETIMEOUT, RT_EOOM, RT_ECUDA, RT_ENOTREADY = range(8)
RT_BC_FIXED, RT_BC_ZEROGRAD, RT_BC_LINEXTRAP = 0, 1, 2
(RT_MODEL_OLDROYDB_LOG, RT_MODEL_GIESEKUS_LOG, RT_MODEL_PTT_LOG, RT_MODEL_FENEP_LOG, RT_MODEL_FENECR_LOG,
 RT_MODEL_ROLIEPOLY_LOG, RT_MODEL_XPOMPOM_LOG, RT_MODEL_WHITEMETZNERCY_LOG) = 0, 1, 2, 3, 4, 5, 6, 7
RT_PTT_LINEAR, RT_PTT_EXP, RT_PTT_GENERALIZED = 0, 1, 2
RT_STAB_NONE, RT_STAB_BSD, RT_STAB_COUPLING = 0, 1, 2
RT_SOLVER_PCG, RT_SOLVER_PBICGSTAB, RT_SOLVER_PBICG = 0, 1, 2
RT_PRECOND_NONE, RT_PRECOND_DIC, RT_PRECOND_DILU, RT_PRECOND_DIAGONAL = 0, 1, 2, 3
RT_LIM_NONE, RT_LIM_UPWIND, RT_LIM_CUBISTA, RT_LIM_MINMOD, RT_LIM_SMART, RT_LIM_WACEB, RT_LIM_SUPERBEE = -1, 0, 1, 2, 3, 4, 5
RT_PREC_FP64, RT_PREC_MIXED = 0, 1
RT_DDT_EULER, RT_DDT_CRANKNICOLSON = 0, 1
RT_FIELD_U, RT_FIELD_P, RT_FIELD_PHI, RT_FIELD_THETA, RT_FIELD_TAU, RT_FIELD_EIGVALS, RT_FIELD_EIGVECS = range(7)
RT_OPT_SWEEP = 1
RT_OPT_SWEEP_PLANES = 2
RT_OPT_PRECISION = 3
RT_OPT_MIXED_PARTS = 4
RT_OPT_MIXED_TIGHTEN = 5
RT_OPT_SWEEP_TUNE = 6
RT_OPT_SWEEP_RING = 7
RT_OPT_WAIT_LIMIT = 8
RT_OPT_STALL_TEST = 9
RT_OPT_MIXED_PRECOND = 10
RT_OPT_BATCH_PERSISTENT = 11
RT_OPT_SWEEP_COMPONENTS = 12
RT_OPT_MIXED_PRECOND_U = 13
RT_MAX_MODES = 16
SWEEP_AUTO, SWEEP_LEVELS, SWEEP_SYSTOLIC = 0, 1, 2

MODEL_NAMES = {
    "Oldroyd-BLog": RT_MODEL_OLDROYDB_LOG,
    "GiesekusLog": RT_MODEL_GIESEKUS_LOG,
    "PTTLog": RT_MODEL_PTT_LOG,
    "FENE-PLog": RT_MODEL_FENEP_LOG,
    "FENE-CRLog": RT_MODEL_FENECR_LOG,
    "Rolie-PolyLog": RT_MODEL_ROLIEPOLY_LOG,
    "XPomPomLog": RT_MODEL_XPOMPOM_LOG,
    "WhiteMetznerCYLog": RT_MODEL_WHITEMETZNERCY_LOG,
}
LIMITER_NAMES = {
    "none": RT_LIM_NONE, "upwind": RT_LIM_UPWIND, "cubista": RT_LIM_CUBISTA,
    "minmod": RT_LIM_MINMOD, "smart": RT_LIM_SMART, "waceb": RT_LIM_WACEB,
    "superbee": RT_LIM_SUPERBEE,
}
STATUS_NAMES = {0: "RT_OK", 1: "RT_EINVAL", 2: "RT_ENOCONV", 3: "RT_ENAN",
                4: "RT_ETIMEOUT", 5: "RT_EOOM", 6: "RT_ECUDA", 7: "RT_ENOTREADY"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class rt_mesh_desc(C.Structure):
    _fields_ = [
        ("nCells", C.c_int32), ("nFaces", C.c_int32), ("nBFaces", C.c_int32), ("nPatches", C.c_int32),
        ("owner", _ip), ("neighbour", _ip),
        ("Sf", _dp), ("magSf", _dp), ("Cf", _dp), ("weights", _dp), ("deltaCoeffs", _dp),
        ("C", _dp), ("V", _dp),
        ("bCell", _ip), ("bSf", _dp), ("bmagSf", _dp), ("bCf", _dp), ("bDeltaCoeffs", _dp),
        ("patchStart", _ip), ("patchSize", _ip),
        ("solveDir", C.c_int32 * 3),
        ("delta", _dp), ("coupled", _ip),
    ]


class rt_bc_desc(C.Structure):
    _fields_ = [
        ("U", _ip), ("p", _ip), ("theta", _ip), ("tau", _ip),
        ("Ub", _dp), ("pb", _dp), ("thetab", _dp), ("taub", _dp),
    ]


class rt_model_params(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("pttFunction", C.c_int32), ("stabilization", C.c_int32), ("pad_", C.c_int32),
        ("rho", C.c_double), ("etaS", C.c_double), ("etaP", C.c_double), ("lambda_", C.c_double),
        ("alpha", C.c_double), ("epsilon", C.c_double), ("zeta", C.c_double), ("L2", C.c_double),
        ("lambdaR", C.c_double), ("beta", C.c_double), ("delta", C.c_double), ("chiMax", C.c_double),
        ("lambdaS", C.c_double), ("q", C.c_double), ("n", C.c_double), ("K", C.c_double), ("a", C.c_double),
        ("rTolMittagLeffler", C.c_double), ("maxIterMittagLeffler", C.c_int32), ("pad2_", C.c_int32),
    ]


RT_THERMO_CONSTANT = 0
RT_THERMO_ARRHENIUS = 1
RT_THERMO_ARRHENIUS_MODIFIED = 2
RT_THERMO_WLF = 3
RT_THERMO_VFT = 4
THERMO_TYPES = {"Constant": RT_THERMO_CONSTANT, "Arrhenius": RT_THERMO_ARRHENIUS,
                "ArrheniusModified": RT_THERMO_ARRHENIUS_MODIFIED, "WLF": RT_THERMO_WLF, "VFT": RT_THERMO_VFT}


class rt_thermo_fn(C.Structure):
    _fields_ = [
        ("type", C.c_int32), ("pad_", C.c_int32),
        ("alpha", C.c_double), ("T0", C.c_double), ("c1", C.c_double), ("c2", C.c_double),
        ("A", C.c_double), ("B", C.c_double),
    ]


class rt_thermo_desc(C.Structure):
    _fields_ = [("lambda_", rt_thermo_fn), ("lambda2", rt_thermo_fn), ("eta", rt_thermo_fn)]


class rt_solver_ctl(C.Structure):
    _fields_ = [
        ("solver", C.c_int32), ("preconditioner", C.c_int32),
        ("tolerance", C.c_double), ("relTol", C.c_double),
        ("minIter", C.c_int32), ("maxIter", C.c_int32),
    ]


class rt_solver_perf(C.Structure):
    _fields_ = [
        ("initialResidual", C.c_double), ("finalResidual", C.c_double),
        ("nIterations", C.c_int32), ("converged", C.c_int32), ("singular", C.c_int32), ("pad_", C.c_int32),
    ]

    def as_dict(self):
        return dict(initialResidual=self.initialResidual, finalResidual=self.finalResidual,
                    nIterations=self.nIterations, converged=bool(self.converged),
                    singular=bool(self.singular))


class rt_case_ctl(C.Structure):
    _fields_ = [
        ("deltaT", C.c_double),
        ("divU", C.c_int32), ("divTheta", C.c_int32),
        ("pRefCell", C.c_int32), ("needReference", C.c_int32),
        ("pRefValue", C.c_double),
        ("solverU", rt_solver_ctl), ("solverP", rt_solver_ctl), ("solverTheta", rt_solver_ctl),
        ("precision", C.c_int32), ("nInIter", C.c_int32),
        ("bodyForce", C.c_double * 3),
        ("nNonOrthCorr", C.c_int32), ("ddtScheme", C.c_int32), ("ddtPsi", C.c_double),
    ]


class rt_step_perf(C.Structure):
    _fields_ = [
        ("U", rt_solver_perf * 3), ("p", rt_solver_perf), ("theta", rt_solver_perf * 6),
        ("contErrSumLocal", C.c_double), ("contErrGlobal", C.c_double),
    ]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def optr(a):
    """double* or NULL"""
    return None if a is None else dptr(a)


_lib = None


def load_library(path: str = LIBNAME):
    """Load librheogpu.so (built by ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "rt_ctx_create": ([P(vp), C.c_int32], C.c_int32),
        "rt_ctx_destroy": ([vp], C.c_int32),
        "rt_last_error": ([vp], C.c_char_p),
        "rt_status_string": ([C.c_int32], C.c_char_p),
        "rt_mesh_upload": ([vp, P(rt_mesh_desc)], C.c_int32),
        "rt_case_setup": ([vp, P(rt_bc_desc), P(rt_model_params), P(rt_case_ctl)], C.c_int32),
        "rt_case_setup_modes": ([vp, P(rt_bc_desc), P(rt_model_params), C.c_int32, P(rt_case_ctl)], C.c_int32),
        "rt_field_set_mode": ([vp, C.c_int32, C.c_int32, _dp, _dp], C.c_int32),
        "rt_field_get_mode": ([vp, C.c_int32, C.c_int32, _dp, _dp], C.c_int32),
        "rt_mode_perf": ([vp, P(rt_solver_perf)], C.c_int32),
        "rt_field_set": ([vp, C.c_int32, _dp, _dp], C.c_int32),
        "rt_field_get": ([vp, C.c_int32, _dp, _dp], C.c_int32),
        "rt_ldu_solve": ([vp, _dp, _dp, _dp, _dp, _dp, C.c_int32, P(rt_solver_ctl), P(rt_solver_perf)], C.c_int32),
        "rt_residual": ([vp, _dp, _dp, _dp, _dp, _dp, _dp], C.c_int32),
        "rt_residual_noalloc": ([vp, vp, vp, vp, vp, vp, _dp], C.c_int32),
        "rt_constitutive_correct": ([vp, _dp, P(rt_solver_perf)], C.c_int32),
        "rt_constitutive_correct_iter": ([vp, _dp, C.c_int32, P(rt_solver_perf)], C.c_int32),
        "rt_set_temperature": ([vp, P(rt_thermo_desc), _dp], C.c_int32),
        "rt_step": ([vp, C.c_int32, P(rt_step_perf)], C.c_int32),
        "rt_op_grad": ([vp, _dp, _dp, _dp], C.c_int32),
        "rt_op_eig": ([vp, C.c_int32, _dp, _dp, _dp], C.c_int32),
        "rt_sync": ([vp], C.c_int32),
        "rt_mesh_set_ijk": ([vp, C.c_int32, C.c_int32, C.c_int32, _ip], C.c_int32),
        "rt_set_option": ([vp, C.c_int32, C.c_int64], C.c_int32),
        "rt_timer_start": ([vp], C.c_int32),
        "rt_timer_stop": ([vp, P(C.c_double)], C.c_int32),
        "rt_profile_enable": ([vp, C.c_int32], C.c_int32),
        "rt_profile_report": ([vp, C.c_char_p, C.c_int32], C.c_int32),
        "rt_kernel_count": ([vp, P(C.c_int64)], C.c_int32),
        "rt_batch_layout": ([vp, C.c_int32, _ip, _ip, _ip, _ip, _ip], C.c_int32),
        "rt_batch_case_setup": ([vp, P(rt_bc_desc), P(rt_model_params), P(rt_case_ctl), _ip, _dp], C.c_int32),
        "rt_batch_step_perf": ([vp, P(rt_step_perf)], C.c_int32),
        "rt_device_bytes": ([P(C.c_int64)], C.c_int32),
        "rt_sweep_schedule": ([vp, _ip], C.c_int32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def header_symbols(header: str) -> list:
    """Names of the functions declared in a C header (``rt_...(``)."""
    import re
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rt_[a-z_0-9]+)\s*\(", txt)))
