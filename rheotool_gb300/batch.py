"""Batched form: many independent cases of uneven size stepped together.

The cases are uploaded as one device mesh, the disjoint union of their
meshes (cells, internal faces and boundary faces concatenated case by case,
so the union keeps OpenFOAM's upper-triangular face order).  Every kernel of
the time step then runs once per stage for all cases, each cell with its own
case's model, and every Krylov solve is per case (own scalars, own stopping
point), so a case gives the same result in a batch as alone, to the round-off
of a different reduction grouping.  When every case is a structured 2-D box,
the DIC/DILU sweeps run one CTA per case.

No reference counterpart: rheoFoam runs one case per process; the case
definitions, models and solver controls are the reference's.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import abi
from .case import Case, Fields, cavity_case
from .mesh import Mesh, Patch, cavity_mesh
from .runtime import Context, _mesh_desc


def union_mesh(meshes: Sequence[Mesh]):
    """Disjoint union of meshes -> (mesh, cellStart, faceStart, bFaceStart)."""
    sd = meshes[0].solveDir
    for m in meshes:
        if not np.array_equal(m.solveDir, sd):
            raise ValueError("all cases of a batch must have the same empty directions")
    cs = np.zeros(len(meshes) + 1, np.int64)
    fs = np.zeros(len(meshes) + 1, np.int64)
    bs = np.zeros(len(meshes) + 1, np.int64)
    for i, m in enumerate(meshes):
        cs[i + 1] = cs[i] + m.nCells
        fs[i + 1] = fs[i] + m.nFaces
        bs[i + 1] = bs[i] + m.nBFaces
    cat = lambda name: np.concatenate([getattr(m, name) for m in meshes])
    patches: List[Patch] = []
    for i, m in enumerate(meshes):
        for p in m.patches:
            patches.append(Patch(f"{i}:{p.name}", int(bs[i] + p.start), p.size))
    u = Mesh(
        nCells=int(cs[-1]),
        owner=np.concatenate([m.owner + cs[i] for i, m in enumerate(meshes)]).astype(np.int32),
        neighbour=np.concatenate([m.neighbour + cs[i] for i, m in enumerate(meshes)]).astype(np.int32),
        Sf=cat("Sf"), magSf=cat("magSf"), Cf=cat("Cf"), w=cat("w"), deltaCoeffs=cat("deltaCoeffs"),
        C=cat("C"), V=cat("V"),
        bCell=np.concatenate([m.bCell + cs[i] for i, m in enumerate(meshes)]).astype(np.int32),
        bSf=cat("bSf"), bmagSf=cat("bmagSf"), bCf=cat("bCf"), bDelta=cat("bDelta"),
        bPatch=np.concatenate([m.bPatch for m in meshes]).astype(np.int32),
        patches=patches, solveDir=sd, shape=None, cellIJK=cat("cellIJK").astype(np.int32),
        name=f"batch{len(meshes)}",
    )
    return u, cs.astype(np.int32), fs.astype(np.int32), bs.astype(np.int32)


@dataclass
class CasePerf:
    U: list
    p: object
    theta: list


class BatchContext:
    """Steps a list of cases as one device mesh.

    The cases share the time step, the discretisation (limiters) and the
    solver controls; each has its own mesh, boundary conditions and model."""

    def __init__(self, cases: Sequence[Case], ctx: Optional[Context] = None, device: int = 0):
        self.cases = list(cases)
        c0 = self.cases[0]
        for c in self.cases[1:]:
            for key in ("deltaT", "divU", "divTheta", "solverU", "solverP", "solverTheta", "precision"):
                if getattr(c, key) != getattr(c0, key):
                    raise ValueError(f"cases of a batch must share {key}")
        self.ctx = ctx if ctx is not None else Context(device)
        self.mesh, self.cellStart, self.faceStart, self.bStart = union_mesh([c.mesh for c in self.cases])
        lib, h = self.ctx.lib, self.ctx._ctx
        md = _mesh_desc(self.mesh, self)
        self.ctx._check(lib.rt_mesh_upload(h, C.byref(md)), "rt_mesh_upload")
        self.ctx.mesh = self.mesh
        one = self.cases[0].mesh
        if len(self.cases) == 1 and one.shape is not None and getattr(one, "cellIJK", None) is not None:
            # a batch of one case runs the single-case path: give it the case's
            # structured description, so that its sweeps are the systolic ones
            nx, ny, nz = one.shape
            a = np.ascontiguousarray(one.cellIJK, dtype=np.int32)
            self.ctx._check(lib.rt_mesh_set_ijk(h, nx, ny, nz, abi.iptr(a)), "rt_mesh_set_ijk")
        dims = np.array([c.mesh.shape if c.mesh.shape is not None else (0, 0, 0) for c in self.cases],
                        dtype=np.int32).reshape(-1)
        ijk = np.ascontiguousarray(self.mesh.cellIJK, dtype=np.int32)
        self.ctx._check(lib.rt_batch_layout(h, len(self.cases), abi.iptr(self.cellStart), abi.iptr(self.faceStart),
                                            abi.iptr(self.bStart), abi.iptr(dims), abi.iptr(ijk)),
                        "rt_batch_layout")
        self.setup()

    def setup(self):
        """(Re)initialise every case's state (rt_batch_case_setup)."""
        lib, h = self.ctx.lib, self.ctx._ctx
        keep = []

        def i32(a):
            a = np.ascontiguousarray(a, dtype=np.int32)
            keep.append(a)
            return abi.iptr(a)

        def f64(a):
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return abi.dptr(a)

        kinds = {f: [] for f in ("U", "p", "theta", "tau")}
        vals = {f: [] for f in ("U", "p", "theta", "tau")}
        for c in self.cases:
            for f, nc in (("U", 3), ("p", 1), ("theta", 6), ("tau", 6)):
                k, v = c._field_bc(f, nc)
                kinds[f].append(k)
                vals[f].append(v)
        cat = lambda f: np.concatenate(vals[f]) if vals[f] else np.zeros((0,))
        bd = abi.rt_bc_desc(i32(np.concatenate(kinds["U"])), i32(np.concatenate(kinds["p"])),
                            i32(np.concatenate(kinds["theta"])), i32(np.concatenate(kinds["tau"])),
                            f64(cat("U")), f64(cat("p").reshape(-1)), f64(cat("theta")), f64(cat("tau")))
        models = (abi.rt_model_params * len(self.cases))(*[c.model.to_c() for c in self.cases])
        _, _, _, ctl = self.cases[0].descriptors()
        ref = np.array([self.cellStart[i] + c.pRefCell if c.needReference else -1
                        for i, c in enumerate(self.cases)], np.int32)
        refv = np.array([c.pRefValue for c in self.cases], np.float64)
        self.ctx._check(lib.rt_batch_case_setup(h, C.byref(bd), models, C.byref(ctl), abi.iptr(ref), abi.dptr(refv)),
                        "rt_batch_case_setup")

    def step(self, n: int = 1) -> abi.rt_step_perf:
        """n steps of every case; returns the aggregate record (worst case)."""
        return self.ctx.step(n)

    def case_perf(self) -> List[abi.rt_step_perf]:
        perf = (abi.rt_step_perf * len(self.cases))()
        self.ctx._check(self.ctx.lib.rt_batch_step_perf(self.ctx._ctx, perf), "rt_batch_step_perf")
        return list(perf)

    def set_case_fields(self, states: dict):
        """Give some cases their fields (case index -> Fields): the others keep
        the state they have (after setup: their initial state).  The serving
        loop carries running cases into a new layout this way."""
        if not states:
            return
        f = self.ctx.fields()
        for i, g in states.items():
            c0, c1 = self.cellStart[i], self.cellStart[i + 1]
            f0, f1 = self.faceStart[i], self.faceStart[i + 1]
            b0, b1 = self.bStart[i], self.bStart[i + 1]
            for name, lo, hi in (("U", c0, c1), ("Ub", b0, b1), ("p", c0, c1), ("pb", b0, b1), ("phi", f0, f1),
                                 ("phib", b0, b1), ("theta", c0, c1), ("thetab", b0, b1), ("tau", c0, c1),
                                 ("taub", b0, b1), ("eigVals", c0, c1), ("eigVecs", c0, c1)):
                getattr(f, name)[lo:hi] = getattr(g, name)
        self.ctx.set_fields(f)

    def fields(self) -> List[Fields]:
        """Each case's fields."""
        f = self.ctx.fields()
        out = []
        for i in range(len(self.cases)):
            c0, c1 = self.cellStart[i], self.cellStart[i + 1]
            f0, f1 = self.faceStart[i], self.faceStart[i + 1]
            b0, b1 = self.bStart[i], self.bStart[i + 1]
            out.append(Fields(U=f.U[c0:c1], Ub=f.Ub[b0:b1], p=f.p[c0:c1], pb=f.pb[b0:b1], phi=f.phi[f0:f1],
                              phib=f.phib[b0:b1], theta=f.theta[c0:c1], thetab=f.thetab[b0:b1],
                              tau=f.tau[c0:c1], taub=f.taub[b0:b1], eigVals=f.eigVals[c0:c1],
                              eigVecs=f.eigVecs[c0:c1]))
        return out

    @property
    def nCells(self) -> int:
        return int(self.cellStart[-1])


# ---------------------------------------------------------------------------
# The parametric cavity sweep: independent 2-D cavities of uneven size
# ---------------------------------------------------------------------------
def cavity_sweep(n_cases: int = 512, n_min: int = 32, n_max: int = 192, seed: int = 20261203,
                 dt: float = 1e-3, precision: int = abi.RT_PREC_MIXED) -> List[Case]:
    """Synthetic parametric sweep: side n ~ U{n_min..n_max}, model ~ U{Oldroyd-B,
    Giesekus alpha = 0.1, FENE-P L2 = 100}, Wi ~ logU(0.1, 4), beta ~ U(0.1, 0.9),
    Re = 0.01, Euler dt, cubista, p PCG-DIC 1e-8, U/theta PBiCGStab-DILU 1e-10."""
    rng = np.random.default_rng(seed)
    cases = []
    meshes = {}
    for _ in range(n_cases):
        n = int(rng.integers(n_min, n_max + 1))
        model = ("Oldroyd-BLog", "GiesekusLog", "FENE-PLog")[int(rng.integers(0, 3))]
        Wi = float(np.exp(rng.uniform(np.log(0.1), np.log(4.0))))
        beta = float(rng.uniform(0.1, 0.9))
        kw = {"alpha": 0.1} if model == "GiesekusLog" else {"L2": 100.0} if model == "FENE-PLog" else {}
        if n not in meshes:
            meshes[n] = cavity_mesh(n)
        c = cavity_case(n, model=model, Wi=Wi, beta=beta, Re=0.01, dt=dt, mesh=meshes[n], **kw)
        c.precision = precision
        cases.append(c)
    return cases
