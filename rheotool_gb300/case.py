"""Case description: mesh + boundary conditions + constitutive model + the
``fvSolution``/``fvSchemes``/``controlDict`` entries the time step reads.

The keys mirror rheoTool's dictionaries one to one:
``constant/constitutiveProperties`` (``type``, ``rho``, ``etaS``, ``etaP``,
``lambda``, ``alpha``, ``epsilon``, ``zeta``, ``L2``, ``lambdaR``/``lambdaD``,
``beta``, ``delta``, ``chiMax`` (Rolie-Poly), ``lambdaS``/``lambdaB``, ``q``,
``n`` (XPomPom), ``n``/``m``, ``K``/``L``, ``a``/``b`` (WhiteMetznerCY),
``rTolMittagLeffler``, ``maxIterMittagLeffler`` (generalized PTT), ``stabilization``,
``destructionFunctionType``; read in e.g. ``GiesekusLog.C:93-120`` and
``constitutiveEq::checkForStab``), ``system/fvSolution`` (``solver``,
``preconditioner``, ``tolerance``, ``relTol``, ``minIter``, ``maxIter``,
``pRefCell``, ``pRefValue``) and ``system/fvSchemes``
(``div(phi,U)``/``div(phi,theta)`` ``GaussDefCmpw <limiter>``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple, Union

import numpy as np

from . import abi
from .mesh import Mesh, cavity_mesh, contraction_mesh, channel_mesh, periodic_channel_mesh

BC_KINDS = {"fixedValue": abi.RT_BC_FIXED, "zeroGradient": abi.RT_BC_ZEROGRAD,
            "linearExtrapolation": abi.RT_BC_LINEXTRAP}
SOLVERS = {"PCG": abi.RT_SOLVER_PCG, "PBiCGStab": abi.RT_SOLVER_PBICGSTAB, "PBiCG": abi.RT_SOLVER_PBICG}
PRECONDS = {"none": abi.RT_PRECOND_NONE, "DIC": abi.RT_PRECOND_DIC,
            "DILU": abi.RT_PRECOND_DILU, "diagonal": abi.RT_PRECOND_DIAGONAL}
STABS = {"none": abi.RT_STAB_NONE, "BSD": abi.RT_STAB_BSD, "coupling": abi.RT_STAB_COUPLING}


@dataclass
class SolverControl:
    solver: str = "PBiCGStab"
    preconditioner: str = "DILU"
    tolerance: float = 1e-10
    relTol: float = 0.0
    minIter: int = 0
    maxIter: int = 1000

    def to_c(self) -> abi.rt_solver_ctl:
        return abi.rt_solver_ctl(SOLVERS[self.solver], PRECONDS[self.preconditioner],
                                 self.tolerance, self.relTol, self.minIter, self.maxIter)


@dataclass
class ThermoFunction:
    """One ``thermoFunction`` sub-dictionary of a model (``thermoLambda``,
    ``thermoEta``, ...; rheoTool's thermoFunctions/<type>): ``type`` one of
    Constant, Arrhenius (alpha, T0), ArrheniusModified (alpha, T0), WLF (c1,
    c2, T0), VFT (A, B, T0).  A model without the sub-dictionary has the
    Constant function (thermoFunctions/newThermoFunction.C:41)."""
    type: str = "Constant"
    alpha: float = 0.0
    T0: float = 0.0
    c1: float = 0.0
    c2: float = 0.0
    A: float = 0.0
    B: float = 0.0

    def to_c(self) -> abi.rt_thermo_fn:
        if self.type not in abi.THERMO_TYPES:
            raise ValueError(f"Unknown thermoFunction type {self.type}; valid: {sorted(abi.THERMO_TYPES)}")
        return abi.rt_thermo_fn(abi.THERMO_TYPES[self.type], 0, self.alpha, self.T0, self.c1, self.c2,
                                self.A, self.B)

    def factor(self, T: np.ndarray) -> np.ndarray:
        """The shift factor at temperatures T (the formulas the library and
        the oracle evaluate; for host-side checks)."""
        T = np.asarray(T, dtype=np.float64)
        if self.type == "Arrhenius":
            return np.exp(self.alpha * (1.0 / T - 1.0 / self.T0))
        if self.type == "ArrheniusModified":
            return np.exp(-self.alpha * (T - self.T0))
        if self.type == "WLF":
            return 10.0 ** (-self.c1 * (T - self.T0) / (self.c2 + (T - self.T0)))
        if self.type == "VFT":
            return 10.0 ** (self.B + self.A / (T - self.T0))
        if self.type == "Constant":
            return np.ones_like(T)
        raise ValueError(f"Unknown thermoFunction type {self.type}")


@dataclass
class Model:
    type: str = "Oldroyd-BLog"
    rho: float = 1.0
    etaS: float = 0.5
    etaP: float = 0.5
    lambda_: float = 1.0
    alpha: float = 0.0
    epsilon: float = 0.0
    zeta: float = 0.0
    L2: float = 100.0
    lambdaR: float = 1.0      # Rolie-PolyLog (its lambdaD is lambda_)
    beta: float = 0.0
    delta: float = -0.5
    chiMax: float = 0.0
    lambdaS: float = 1.0      # XPomPomLog (its lambdaB is lambda_)
    q: float = 1.0
    n: float = 0.0            # XPomPomLog stretch exponent, WhiteMetznerCYLog power index
    K: float = 0.0            # WhiteMetznerCYLog (the log form has L = K, b = a, m = n)
    a: float = 1.0
    rTolMittagLeffler: float = 1e-12   # PTTLog generalized (its alpha and beta are alpha, beta)
    maxIterMittagLeffler: int = 200
    stabilization: str = "coupling"
    destructionFunctionType: str = "linear"
    # non-isothermal parameter shifts: thermoLambda (Rolie-Poly thermoLambdaD,
    # XPomPom thermoLambdaB), the second relaxation time's (Rolie-Poly
    # thermoLambdaR, XPomPom thermoLambdaS) and thermoEta
    thermoLambda: ThermoFunction = field(default_factory=ThermoFunction)
    thermoLambda2: ThermoFunction = field(default_factory=ThermoFunction)
    thermoEta: ThermoFunction = field(default_factory=ThermoFunction)

    def thermo_c(self) -> abi.rt_thermo_desc:
        return abi.rt_thermo_desc(self.thermoLambda.to_c(), self.thermoLambda2.to_c(), self.thermoEta.to_c())

    def to_c(self) -> abi.rt_model_params:
        if self.type not in abi.MODEL_NAMES:
            raise ValueError(f"Unknown constitutiveEq type {self.type}; valid: "
                             f"{sorted(abi.MODEL_NAMES)}")
        ptts = {"linear": abi.RT_PTT_LINEAR, "exponential": abi.RT_PTT_EXP, "generalized": abi.RT_PTT_GENERALIZED}
        if self.type == "PTTLog" and self.destructionFunctionType not in ptts:
            raise ValueError(f"PTTLog destructionFunctionType {self.destructionFunctionType}; valid: "
                             f"{sorted(ptts)}")
        ptt = ptts.get(self.destructionFunctionType, abi.RT_PTT_LINEAR)
        return abi.rt_model_params(abi.MODEL_NAMES[self.type], ptt, STABS[self.stabilization], 0,
                                   self.rho, self.etaS, self.etaP, self.lambda_, self.alpha,
                                   self.epsilon, self.zeta, self.L2, self.lambdaR, self.beta,
                                   self.delta, self.chiMax, self.lambdaS, self.q, self.n, self.K, self.a,
                                   self.rTolMittagLeffler, int(self.maxIterMittagLeffler), 0)


Value = Union[float, Tuple[float, ...], Callable[[np.ndarray], np.ndarray]]


@dataclass
class Case:
    mesh: Mesh
    model: Model
    bcs: Dict[str, Dict[str, Tuple[str, Optional[Value]]]]   # patch -> field -> (kind, value)
    deltaT: float = 1e-3
    divU: str = "cubista"
    divTheta: str = "cubista"
    solverU: SolverControl = field(default_factory=lambda: SolverControl("PBiCGStab", "DILU", 1e-10))
    solverP: SolverControl = field(default_factory=lambda: SolverControl("PCG", "DIC", 1e-8, maxIter=800))
    solverTheta: SolverControl = field(default_factory=lambda: SolverControl("PBiCGStab", "DILU", 1e-10))
    pRefCell: int = 0
    pRefValue: float = 0.0
    precision: int = abi.RT_PREC_FP64
    name: str = "case"
    bodyForce: Tuple[float, float, float] = (0.0, 0.0, 0.0)   # per unit mass, in UEqn
    nInIter: int = 1          # SIMPLE.nInIter: inner iterations per time step
    nNonOrthCorr: int = 0     # SIMPLE.nNonOrthogonalCorrectors
    ddt: str = "Euler"        # ddtSchemes default: "Euler" or "CrankNicolson"
    ddtPsi: float = 1.0       # CrankNicolson off-centering coefficient
    # multiMode (multiMode.C:69-91): the modes after the first (``model``);
    # every mode has its own theta, tau and eigen fields, tau is their sum
    moreModes: List[Model] = field(default_factory=list)

    @property
    def models(self) -> List[Model]:
        """The modes of the constitutive model (one for a single-mode model)."""
        return [self.model] + list(self.moreModes)

    def thermo_descs(self):
        """ctypes array of every mode's rt_thermo_desc."""
        ms = self.models
        arr = (abi.rt_thermo_desc * len(ms))()
        for i, m in enumerate(ms):
            arr[i] = m.thermo_c()
        return arr

    def mode_params(self):
        """ctypes array of every mode's rt_model_params."""
        ms = self.models
        arr = (abi.rt_model_params * len(ms))()
        for i, m in enumerate(ms):
            arr[i] = m.to_c()
        return arr

    # ------------------------------------------------------------------
    def _field_bc(self, fld: str, ncomp: int):
        m = self.mesh
        kinds = np.zeros(len(m.patches), np.int32)
        vals = np.zeros((m.nBFaces, ncomp))
        for p, patch in enumerate(m.patches):
            kind, val = self.bcs[patch.name][fld]
            kinds[p] = BC_KINDS[kind]
            if val is None:
                continue
            sl = slice(patch.start, patch.start + patch.size)
            if callable(val):
                vals[sl] = np.asarray(val(m.bCf[sl])).reshape(patch.size, ncomp)
            else:
                vals[sl] = np.broadcast_to(np.asarray(val, dtype=np.float64), (patch.size, ncomp))
        return kinds, np.ascontiguousarray(vals)

    @property
    def needReference(self) -> bool:
        return all(self.bcs[p.name]["p"][0] != "fixedValue" for p in self.mesh.patches)

    def descriptors(self):
        """(rt_mesh_desc, rt_bc_desc, rt_model_params, rt_case_ctl); the numpy
        arrays behind the pointers are kept alive on ``self``."""
        m = self.mesh
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
        md.nCells, md.nFaces, md.nBFaces, md.nPatches = m.nCells, m.nFaces, m.nBFaces, len(m.patches)
        md.owner, md.neighbour = i(m.owner), i(m.neighbour)
        md.Sf, md.magSf, md.Cf = d(m.Sf), d(m.magSf), d(m.Cf)
        md.weights, md.deltaCoeffs = d(m.w), d(m.deltaCoeffs)
        md.C, md.V = d(m.C), d(m.V)
        md.bCell, md.bSf, md.bmagSf, md.bCf, md.bDeltaCoeffs = i(m.bCell), d(m.bSf), d(m.bmagSf), d(m.bCf), d(m.bDelta)
        md.patchStart = i(np.array([p.start for p in m.patches]))
        md.patchSize = i(np.array([p.size for p in m.patches]))
        for k in range(3):
            md.solveDir[k] = int(m.solveDir[k])
        if m.delta is not None:
            md.delta = d(m.delta)
        if m.coupled is not None:
            md.coupled = i(m.coupled)

        kU, Ub = self._field_bc("U", 3)
        kP, pb = self._field_bc("p", 1)
        kT, thb = self._field_bc("theta", 6)
        kTa, tab = self._field_bc("tau", 6)
        bd = abi.rt_bc_desc(i(kU), i(kP), i(kT), i(kTa), d(Ub), d(pb.reshape(-1)), d(thb), d(tab))
        mp = self.model.to_c()
        ctl = abi.rt_case_ctl()
        ctl.deltaT = self.deltaT
        ctl.divU = abi.LIMITER_NAMES[self.divU]
        ctl.divTheta = abi.LIMITER_NAMES[self.divTheta]
        ctl.pRefCell = self.pRefCell
        ctl.needReference = int(self.needReference)
        ctl.pRefValue = self.pRefValue
        ctl.solverU = self.solverU.to_c()
        ctl.solverP = self.solverP.to_c()
        ctl.solverTheta = self.solverTheta.to_c()
        ctl.precision = self.precision
        ctl.nInIter = int(self.nInIter)
        ctl.nNonOrthCorr = int(self.nNonOrthCorr)
        if self.ddt not in ("Euler", "CrankNicolson"):
            raise ValueError(f"ddt scheme {self.ddt!r}: Euler or CrankNicolson")
        ctl.ddtScheme = abi.RT_DDT_CRANKNICOLSON if self.ddt == "CrankNicolson" else abi.RT_DDT_EULER
        ctl.ddtPsi = float(self.ddtPsi)
        for k in range(3):
            ctl.bodyForce[k] = float(self.bodyForce[k])
        self._keep = keep
        return md, bd, mp, ctl


# ---------------------------------------------------------------------------
# Workload builders
# ---------------------------------------------------------------------------
WALL_VE = {"U": ("fixedValue", (0.0, 0.0, 0.0)), "p": ("zeroGradient", None),
           "theta": ("zeroGradient", None), "tau": ("linearExtrapolation", 0.0)}


def lid_profile(Cf: np.ndarray) -> np.ndarray:
    """Steady lid velocity U = (16 x^2 (1-x)^2, 0, 0)."""
    x = Cf[:, 0]
    u = np.zeros((Cf.shape[0], 3))
    u[:, 0] = 16.0 * x ** 2 * (1.0 - x) ** 2
    return u


def cavity_case(n: int = 64, model: str = "Oldroyd-BLog", Wi: float = 0.5, beta: float = 0.5,
                Re: float = 0.01, dt: float = 1e-3, mesh: Optional[Mesh] = None, **model_kw) -> Case:
    """Lid-driven cavity: U_lid = 16x^2(1-x)^2, lambda = Wi (U = L = 1),
    etaS = beta, etaP = 1 - beta, rho = Re (eta0 = 1); Euler, GaussDefCmpw
    cubista, p PCG-DIC 1e-8, U/theta PBiCGStab-DILU 1e-10."""
    mesh = cavity_mesh(n) if mesh is None else mesh
    mdl = Model(model, rho=Re, etaS=beta, etaP=1.0 - beta, lambda_=Wi, **model_kw)
    bcs = {
        "movingLid": dict(WALL_VE, U=("fixedValue", lid_profile)),
        "fixedWalls": dict(WALL_VE),
    }
    return Case(mesh, mdl, bcs, deltaT=dt, name=f"cavity{n}_{model}")


def contraction_case(mesh: Optional[Mesh] = None, model: str = "GiesekusLog", Wi: float = 2.0,
                     beta: float = 1.0 / 9.0, rho: float = 0.01, alpha: float = 0.1,
                     U_in: float = 0.25, dt: float = 5e-3, **model_kw) -> Case:
    """3-D 4:1 planar contraction, Giesekus-Log alpha = 0.1, beta = 1/9,
    Wi = lambda U_d / H = 2 with U_d = 4 U_in = 1 and H = 1."""
    mesh = mesh if mesh is not None else contraction_mesh()
    U_d = 4.0 * U_in
    mdl = Model(model, rho=rho, etaS=beta, etaP=1.0 - beta, lambda_=Wi * 1.0 / U_d,
                alpha=alpha, **model_kw)
    bcs = {
        "inlet": {"U": ("fixedValue", (U_in, 0.0, 0.0)), "p": ("zeroGradient", None),
                  "theta": ("fixedValue", 0.0), "tau": ("fixedValue", 0.0)},
        "outlet": {"U": ("zeroGradient", None), "p": ("fixedValue", 0.0),
                   "theta": ("zeroGradient", None), "tau": ("zeroGradient", None)},
        "walls": dict(WALL_VE),
    }
    return Case(mesh, mdl, bcs, deltaT=dt, name=f"contraction{mesh.nCells}_{model}")


def channel_case(mesh: Optional[Mesh] = None, model: str = "Oldroyd-BLog", U_in: float = 1.0,
                 dt: float = 1e-2, lambda_: float = 0.1, beta: float = 0.5, rho: float = 0.01,
                 **model_kw) -> Case:
    mesh = mesh if mesh is not None else channel_mesh()
    mdl = Model(model, rho=rho, etaS=beta, etaP=1.0 - beta, lambda_=lambda_, **model_kw)
    bcs = {
        "inlet": {"U": ("fixedValue", (U_in, 0.0, 0.0)), "p": ("zeroGradient", None),
                  "theta": ("fixedValue", 0.0), "tau": ("fixedValue", 0.0)},
        "outlet": {"U": ("zeroGradient", None), "p": ("fixedValue", 0.0),
                   "theta": ("zeroGradient", None), "tau": ("zeroGradient", None)},
        "walls": dict(WALL_VE),
    }
    return Case(mesh, mdl, bcs, deltaT=dt, name=f"channel_{model}")


def periodic_channel_case(mesh: Optional[Mesh] = None, model: str = "PTTLog", Wi: float = 2.0,
                          beta: float = 1.0 / 9.0, rho: float = 0.01, U_mean: float = 1.0,
                          H: float = 1.0, dt: float = 5e-3, epsilon: float = 0.25, **model_kw) -> Case:
    """Channel periodic in x and z between walls at y = +-H, driven by a
    uniform streamwise body force (the mean pressure gradient).  The force is
    the one that gives a Newtonian fluid of the same total viscosity the mean
    velocity U_mean: g = 3 (etaS + etaP) U_mean / (rho H^2).  lambda = Wi H /
    U_mean.  The default model is the linear PTT (epsilon 0.25, zeta 0).  The
    walls are the only patch, so p needs a reference cell."""
    mesh = mesh if mesh is not None else periodic_channel_mesh()
    eta0 = 1.0
    kw = dict(model_kw)
    if model == "PTTLog":
        kw.setdefault("epsilon", epsilon)
    mdl = Model(model, rho=rho, etaS=beta * eta0, etaP=(1.0 - beta) * eta0, lambda_=Wi * H / U_mean, **kw)
    bcs = {"walls": dict(WALL_VE)}
    g = 3.0 * eta0 * U_mean / (rho * H * H)
    return Case(mesh, mdl, bcs, deltaT=dt, name=f"periodicChannel{mesh.nCells}_{model}_Wi{Wi:g}",
                bodyForce=(g, 0.0, 0.0))


def lognormal_conformation(n: int, sigma: float = 0.1, seed: int = 20261203):
    """Per-cell log-conformation theta = Q diag(sigma z) Q^T with z ~ N(0, 1)^3
    and Q a Haar-random rotation (QR of a Gaussian matrix, signs fixed), so
    that A = exp(theta) = I + a lognormal perturbation, always SPD.  Returns
    theta (n, 6; xx xy xz yy yz zz), eigVals = exp(mu) ascending (n, 3) and
    eigVecs (n, 9; row-major, eigenvectors as columns), the state calcEig
    leaves behind."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mu = sigma * rng.standard_normal((n, 3))
    G = rng.standard_normal((n, 3, 3))
    Q, R = np.linalg.qr(G)
    Q = Q * np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
    order = np.argsort(mu, axis=1)
    mu = np.take_along_axis(mu, order, axis=1)
    Q = np.take_along_axis(Q, order[:, None, :], axis=2)
    T = np.einsum("nij,nj,nkj->nik", Q, mu, Q)
    theta = np.stack([T[:, 0, 0], T[:, 0, 1], T[:, 0, 2], T[:, 1, 1], T[:, 1, 2], T[:, 2, 2]], axis=1)
    return np.ascontiguousarray(theta), np.exp(mu), np.ascontiguousarray(Q.reshape(n, 9))


def periodic_channel_state(case: "Case", sigma: float = 0.1, seed: int = 20261203) -> "Fields":
    """Initial state of the periodic channel: the laminar Newtonian profile
    u = 1.5 U_mean (1 - y^2/H^2) (with its face fluxes), p = 0, and the
    lognormal log-conformation of `lognormal_conformation` with the matching
    eigen-decomposition and tau = etaP/(lambda (1 - zeta)) (A - I)
    (Oldroyd-B, Giesekus and PTT; zeta = 0 but for PTT).  Boundary values of
    theta and tau are the wall cells' values."""
    m = case.mesh
    md = case.model
    if md.type == "FENE-PLog":
        raise ValueError("the lognormal initial state is defined for Oldroyd-B, Giesekus and PTT")
    N = m.nCells
    f = Fields.zeros(m)
    H = float(np.abs(m.bCf[:, 1]).max())
    g = case.bodyForce[0]
    U_mean = g * md.rho * H * H / (3.0 * (md.etaS + md.etaP))
    y = m.C[:, 1]
    f.U[:, 0] = 1.5 * U_mean * (1.0 - (y / H) ** 2)
    Uf = m.w[:, None] * (f.U[m.owner] - f.U[m.neighbour]) + f.U[m.neighbour]
    f.phi[:] = (m.Sf * Uf).sum(1)
    th, ev, vv = lognormal_conformation(N, sigma, seed)
    f.theta[:] = th
    f.eigVals[:] = ev
    f.eigVecs[:] = vv
    R = vv.reshape(N, 3, 3)
    A = np.einsum("nij,nj,nkj->nik", R, ev, R)
    zeta = md.zeta if md.type == "PTTLog" else 0.0
    c = md.etaP / (md.lambda_ * (1.0 - zeta))
    T = c * (A - np.eye(3)[None])
    f.tau[:] = np.stack([T[:, 0, 0], T[:, 0, 1], T[:, 0, 2], T[:, 1, 1], T[:, 1, 2], T[:, 2, 2]], axis=1)
    f.thetab[:] = f.theta[m.bCell]
    f.taub[:] = f.tau[m.bCell]
    return f


@dataclass
class Fields:
    """Host copy of the state of a case (OpenFOAM AoS layout)."""
    U: np.ndarray
    Ub: np.ndarray
    p: np.ndarray
    pb: np.ndarray
    phi: np.ndarray
    phib: np.ndarray
    theta: np.ndarray
    thetab: np.ndarray
    tau: np.ndarray
    taub: np.ndarray
    eigVals: np.ndarray
    eigVecs: np.ndarray
    # multiMode: every mode's constitutive fields (empty for a single-mode
    # model); theta, eigVals and eigVecs above are then mode 0's and tau,
    # taub the modes' sum (multiMode::tau())
    modes: List["ModeFields"] = field(default_factory=list)

    @staticmethod
    def zeros(mesh: Mesh, nModes: int = 1) -> "Fields":
        N, nF, nB = mesh.nCells, mesh.nFaces, mesh.nBFaces
        z = lambda *s: np.zeros(s)
        f = Fields(U=z(N, 3), Ub=z(nB, 3), p=z(N), pb=z(nB), phi=z(nF), phib=z(nB),
                   theta=z(N, 6), thetab=z(nB, 6), tau=z(N, 6), taub=z(nB, 6),
                   eigVals=np.ones((N, 3)), eigVecs=np.tile(np.eye(3).reshape(9), (N, 1)))
        if nModes > 1:
            f.modes = [ModeFields.zeros(mesh) for _ in range(nModes)]
        return f

    def copy(self) -> "Fields":
        return Fields(**{k: (v.copy() if isinstance(v, np.ndarray) else [m.copy() for m in v])
                         for k, v in self.__dict__.items()})


@dataclass
class ModeFields:
    """One mode's constitutive fields of a multiMode model."""
    theta: np.ndarray
    thetab: np.ndarray
    tau: np.ndarray
    taub: np.ndarray
    eigVals: np.ndarray
    eigVecs: np.ndarray

    @staticmethod
    def zeros(mesh: Mesh) -> "ModeFields":
        N, nB = mesh.nCells, mesh.nBFaces
        return ModeFields(np.zeros((N, 6)), np.zeros((nB, 6)), np.zeros((N, 6)), np.zeros((nB, 6)),
                          np.ones((N, 3)), np.tile(np.eye(3).reshape(9), (N, 1)))

    def copy(self) -> "ModeFields":
        return ModeFields(**{k: v.copy() for k, v in self.__dict__.items()})
