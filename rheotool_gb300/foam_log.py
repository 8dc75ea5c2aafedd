"""Solver logs in OpenFOAM's format, for diffing a GPU run's log with a
rheoFoam log line by line.

rheoFoam prints, per time step:
- ``Time = <t>``;
- one ``Solving for`` line per solved component of U, p and theta;
- the continuity errors;
- the execution time.

A ``Solving for`` line reads ``<preconditioner><solver>:  Solving for
<field><component>, Initial residual = <r0>, Final residual = <r>, No
Iterations <n>``. It is OpenFOAM's SolverPerformance print; the names are the
field's name with pTraits' component names, as rheoTool's own sparse solvers
also form them (libs/sparseMatrixSolvers/segregated/petscSolver/
petscSolver.C:480-481). The continuity line is OpenFOAM's continuityErrs.H,
with the cumulative error summed over the steps a log has seen.

The library records the last solve of each field in a step (rt_step_perf).
With nNonOrthogonalCorrectors or nInIter above their defaults, rheoFoam
prints one line per corrector or inner iteration, and this log prints the
last one only.
"""
from __future__ import annotations

from typing import List, Sequence

from . import abi

VECTOR = ("x", "y", "z")
SYMM_TENSOR = ("xx", "xy", "xz", "yy", "yz", "zz")


def solver_name(ctl) -> str:
    """OpenFOAM's name of a solver with its preconditioner (DICPCG,
    DILUPBiCGStab, DILUPBiCG; the preconditioner is left out when none)."""
    pre = "" if ctl.preconditioner == "none" else ctl.preconditioner
    return pre + ctl.solver


def solving_line(name: str, field: str, perf) -> str:
    return (f"{name}:  Solving for {field}, Initial residual = {perf.initialResidual:g}, "
            f"Final residual = {perf.finalResidual:g}, No Iterations {perf.nIterations}")


class FoamLog:
    """The log of a case's time steps, one call of ``step`` per step;
    ``lines`` holds every line so far."""

    def __init__(self, case):
        self.case = case
        self.cumulative = 0.0
        self.lines: List[str] = []

    def step(self, time: float, perf: abi.rt_step_perf, execution_s: float = None) -> List[str]:
        c = self.case
        out = ["", f"Time = {time:g}", ""]
        u = solver_name(c.solverU)
        for k in range(3):
            if perf.U[k].nIterations >= 0 and c.mesh.solveDir[k]:
                out.append(solving_line(u, "U" + VECTOR[k], perf.U[k]))
        out.append(solving_line(solver_name(c.solverP), "p", perf.p))
        self.cumulative += perf.contErrGlobal
        out.append(f"time step continuity errors : sum local = {perf.contErrSumLocal:g}, "
                   f"global = {perf.contErrGlobal:g}, cumulative = {self.cumulative:g}")
        th = solver_name(c.solverTheta)
        for k in range(6):
            if perf.theta[k].nIterations >= 0:
                out.append(solving_line(th, "theta" + SYMM_TENSOR[k], perf.theta[k]))
        if execution_s is not None:
            out.append(f"ExecutionTime = {execution_s:g} s")
        self.lines.extend(out)
        return out

    def text(self) -> str:
        return "\n".join(self.lines) + "\n"


def step_log(case, times: Sequence[float], perfs: Sequence[abi.rt_step_perf]) -> str:
    """The log of several steps at once."""
    log = FoamLog(case)
    for t, p in zip(times, perfs):
        log.step(t, p)
    return log.text()
