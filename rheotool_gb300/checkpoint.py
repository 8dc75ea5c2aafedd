"""Checkpoint and resume of a running case.

A checkpoint is a snapshot of every device-resident field of a context's
case: U, p, phi, theta, tau, eigVals and eigVecs with their boundary values,
and every mode's theta, tau and eigen fields of a multiMode model.  It is
written as one ``.npz`` with the case's sizes and the step and time reached.
Set a context up with the same case and these fields, and the run continues
bit for bit as if it had not stopped: between Euler time steps these fields
are the whole state of the step.

The reference writes time directories for the same purpose, `startFrom
latestTime` in controlDict to resume (runTime.write(), solvers/rheoFoam/
rheoFoam.C:164; the Log models' AUTO_WRITE fields, e.g.
Oldroyd-B/Oldroyd-BLog/Oldroyd_BLog.C:52-113).  Those are written in ASCII at
writePrecision (`foam_io.write_fields` writes them too); this snapshot is
binary so that the resumed run is exact.

Not covered:
- Crank-Nicolson runs: they also carry the old-time derivatives of U, phi and
  theta, which the C ABI does not expose, so they are refused.
- Batched contexts: a batch carries its cases' fields through
  ``BatchContext.set_case_fields``.
"""
from __future__ import annotations

from typing import Any, Dict, Tuple

import numpy as np

from .case import Case, Fields, ModeFields

FORMAT = 1
_FIELDS = ("U", "Ub", "p", "pb", "phi", "phib", "theta", "thetab", "tau", "taub", "eigVals", "eigVecs")
_MODE_FIELDS = ("theta", "thetab", "tau", "taub", "eigVals", "eigVecs")


def _check_case(case: Case) -> None:
    if case.ddt != "Euler":
        raise ValueError(f"checkpoint: ddt {case.ddt} carries old-time derivatives the C ABI does not expose; "
                         "only Euler runs resume exactly")


def save_fields(path: str, case: Case, fields: Fields, step: int = 0, time: float = 0.0) -> None:
    """Write the snapshot of `fields` (the state of `case` after `step` steps,
    at `time`) to `path` (.npz)."""
    _check_case(case)
    m = case.mesh
    arrays: Dict[str, Any] = {
        "format": np.int64(FORMAT), "step": np.int64(step), "time": np.float64(time),
        "sizes": np.array([m.nCells, m.nFaces, m.nBFaces, len(case.models)], dtype=np.int64),
        "models": np.array([mm.type for mm in case.models]),
    }
    for name in _FIELDS:
        arrays[name] = np.ascontiguousarray(getattr(fields, name), dtype=np.float64)
    for i, mf in enumerate(fields.modes):
        for name in _MODE_FIELDS:
            arrays[f"mode{i}_{name}"] = np.ascontiguousarray(getattr(mf, name), dtype=np.float64)
    with open(path, "wb") as fh:
        np.savez(fh, **arrays)


def load_fields(path: str, case: Case) -> Tuple[Fields, Dict[str, Any]]:
    """Read a snapshot for `case`: (fields, {"step", "time"}).  A snapshot of
    another mesh size or other models is refused (ValueError)."""
    _check_case(case)
    with np.load(path, allow_pickle=False) as z:
        if int(z["format"]) != FORMAT:
            raise ValueError(f"checkpoint format {int(z['format'])}, this library reads {FORMAT}")
        m = case.mesh
        want = [m.nCells, m.nFaces, m.nBFaces, len(case.models)]
        got = [int(v) for v in z["sizes"]]
        if got != want:
            raise ValueError(f"checkpoint of cells/faces/boundary faces/modes {got}, the case has {want}")
        models = [str(t) for t in z["models"]]
        if models != [mm.type for mm in case.models]:
            raise ValueError(f"checkpoint of models {models}, the case has {[mm.type for mm in case.models]}")
        f = Fields(**{name: z[name].copy() for name in _FIELDS})
        if len(case.models) > 1:
            f.modes = [ModeFields(**{name: z[f"mode{i}_{name}"].copy() for name in _MODE_FIELDS})
                       for i in range(len(case.models))]
        meta = {"step": int(z["step"]), "time": float(z["time"])}
    return f, meta


def save(ctx, path: str, step: int = 0, time: float = 0.0) -> None:
    """Snapshot the case a runtime.Context is running (after `step` steps,
    at `time`)."""
    if ctx.case is None:
        raise ValueError("checkpoint: the context has no case")
    _check_case(ctx.case)
    save_fields(path, ctx.case, ctx.fields(), step, time)


def resume(ctx, case: Case, path: str) -> Dict[str, Any]:
    """Set `case` up on a runtime.Context from the snapshot at `path`; returns
    {"step", "time"} of the snapshot."""
    fields, meta = load_fields(path, case)
    ctx.setup_case(case, fields)
    return meta
