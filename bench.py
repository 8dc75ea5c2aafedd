#!/usr/bin/env python
"""bench.py — throughput of the rheoFoam segregated time step on GB300.

Workload (one "step" = one rheoFoam time step: UEqn, SIMPLEC pEqn with a
PCG-DIC pressure solve, GiesekusLog constitutive update with six
PBiCGStab-DILU theta solves): 3-D planar 4:1 contraction, 1,000,000 hex cells,
Giesekus-Log alpha = 0.1, Wi = 2, beta = 1/9, synthetic mesh and inputs (no
dataset exists for it).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--precision fp64|mixed]

Prints one JSON line.  `value` is device-timed (CUDA events on the library's
stream) whole-job cell-steps/s of the selected form with all fields resident
in HBM: by default the FP64 plain form, the reference's own precision.  The
mixed-precision form (FP32 Krylov iterations and sweeps, FP64 residual
replacement; FP32 constitutive algebra with FP64 fallbacks) is timed in the
same run on the same case and steps (`mixed_precision`), with each field's
relative L2 difference from the FP64 form (`field_error_vs_fp64`).  `e2e` is
the same metric over the same steps from the same state, through the C ABI
with pinned host buffers (each step uploads U, p, phi and downloads U, p,
phi, tau; theta stays resident, as it does between rheoFoam time steps).
`roofline` is for the operation with the largest device time, measured live
with CUDA events; `cpu_baseline` is the FP64 CPU oracle on a bounded sample
of the same workload.  `--impl reference` times the reference algorithm on
the host cores over the same mesh and steps: the reference itself (rheoTool
on OpenFOAM v9) cannot be built here, so its FP64 CPU restatement (oracle/)
runs instead; its Krylov iterations, sweeps and face loops are sequential, as
one OpenFOAM process runs them, so it runs on one core.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s (1M-cell Giesekus)"
UNIT = "cell-steps/s"
WORKLOAD = ("3-D planar 4:1 contraction, 1,000,000 hex cells (266x100x50 bounding grid, graded), "
            "GiesekusLog alpha=0.1, Wi=2, beta=1/9, rho=0.01, dt=5e-3, Euler, GaussDefCmpw cubista, "
            "p PCG-DIC 1e-8, U/theta PBiCGStab-DILU 1e-10")
SAMPLE_DIMS = dict(nx_up=67, nx_down=66, ny_in=25, ny_out=13, nz=25)   # 126,675 cells


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--small", action="store_true", help="126,675-cell sample instead of 1M (testing)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="form timed for `value` (the other is timed beside it unless --no-plain)")
    ap.add_argument("--no-plain", action="store_true", help="skip the second form")
    ap.add_argument("--no-floor", action="store_true",
                    help="skip the FP64 run with 100x tighter tolerances (the solver-tolerance floor)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched cavity sweep")
    ap.add_argument("--no-serve", action="store_true", help="skip the served request stream")
    ap.add_argument("--batch-cases", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--serve-requests", type=int, default=24)
    ap.add_argument("--serve-steps", type=int, default=10)
    ap.add_argument("--serve3d-requests", type=int, default=8)
    ap.add_argument("--serve3d-steps", type=int, default=100)
    ap.add_argument("--precision-sweep", action="store_true",
                    help="instead of the throughput line: the precision sweep on the periodic PTT channel")
    ap.add_argument("--sweep-dims", default="400x100x100", help="periodic channel cells nx x ny x nz")
    ap.add_argument("--sweep-steps", type=int, default=3)
    ap.add_argument("--no-sweep", action="store_true", help="skip the precision sweep key of the default line")
    ap.add_argument("--no-check", action="store_true", help="skip the mixed-vs-converged-FP64 check on the headline")
    ap.add_argument("--check-steps", type=int, default=4)
    ap.add_argument("--mixed-precond", type=int, default=None,
                    help="RT_OPT_MIXED_PRECOND of the mixed form (Jacobi sweeps of its pressure DIC; 0 exact)")
    return ap.parse_args()


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_case(small: bool):
    from rheotool_gb300.case import contraction_case
    from rheotool_gb300.mesh import contraction_mesh
    if small:
        return contraction_case(contraction_mesh(**SAMPLE_DIMS))
    return contraction_case()


def rank_max(ms: float, pg) -> float:
    """The slowest rank's time (every rank gets it), then a barrier; `pg` is
    torch.distributed with a process group, or None for one rank."""
    if pg is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    pg.barrier()
    return float(t[0])


def whole_job_value(cells: int, steps: int, world: int, ms_max: float) -> float:
    """Cell-steps/s of the whole job: every rank steps its own replica of the
    case, so the units are cells x steps x ranks over the slowest rank's time."""
    return cells * steps * world / (ms_max * 1e-3)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(index)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_baseline(seconds: float, warm: int = 1):
    """FP64 CPU oracle on the 126,675-cell sample, one core (its Krylov
    sweeps, face loops and cell loops all run on one thread)."""
    from oracle import pyoracle
    pyoracle.set_threads(1)
    case = make_case(True)
    o = pyoracle.Oracle(case)
    if warm:
        o.step(warm)
    n, t0 = 0, time.perf_counter()
    while True:
        o.step(1)
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    cells = case.mesh.nCells
    return {"value": cells * n / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"same contraction/Giesekus case at {cells:,} cells (1/8 of the 1M mesh), "
                      f"{n} time steps after {warm} warm-up step(s), FP64 oracle on one core, {dt:.1f} s"}


def run_batched(args):
    """Batched form: the parametric cavity sweep (independent 2-D cavities,
    side 32..192, Oldroyd-B / Giesekus / FENE-P, Wi 0.1..4) as one device
    mesh in the mixed form, against the FP64 plain path running a sample of
    the same cases one at a time."""
    import numpy as np
    from rheotool_gb300 import abi
    from rheotool_gb300.batch import BatchContext, cavity_sweep
    from rheotool_gb300.runtime import Context
    cases = cavity_sweep(args.batch_cases, 32, 192, precision=abi.RT_PREC_MIXED)
    bt = BatchContext(cases)
    bt.step(2)
    bt.ctx.sync()
    k0 = bt.ctx.kernel_count()
    bt.ctx.timer_start()
    bt.step(args.batch_steps)
    ms = bt.ctx.timer_stop()
    launches = bt.ctx.kernel_count() - k0
    cells = bt.nCells
    value = cells * args.batch_steps / (ms * 1e-3)
    perf = bt.case_perf()
    bt.ctx.close()
    # the plain path: 16 of the cases, one context each, FP64, same protocol
    import copy
    sample = [copy.copy(cases[i]) for i in range(0, len(cases), max(1, len(cases) // 16))][:16]
    tot_ms, tot_cells = 0.0, 0
    for c in sample:
        c.precision = abi.RT_PREC_FP64
        ctx = Context(0)
        ctx.setup_case(c)
        ctx.step(2)
        ctx.sync()
        ctx.timer_start()
        ctx.step(3)
        tot_ms += ctx.timer_stop()
        tot_cells += c.mesh.nCells * 3
        ctx.close()
    plain = tot_cells / (tot_ms * 1e-3)
    return {"workload": f"{len(cases)} independent 2-D cavities, side 32..192 (uniform), "
                        "models Oldroyd-B / Giesekus alpha=0.1 / FENE-P L2=100, Wi log-uniform 0.1..4, "
                        "beta 0.1..0.9, Re 0.01, dt 1e-3; mixed-precision form, one device mesh",
            "cases": len(cases), "cells": cells, "steps": args.batch_steps, "value": value,
            "unit": UNIT, "ms_per_step": ms / args.batch_steps, "gpu_launches": launches,
            "time_to_solution_200_steps_s": 200 * ms / args.batch_steps * 1e-3,
            "p_iterations_max": max(p.p.nIterations for p in perf),
            "plain_fp64_one_case_at_a_time": {"value": plain, "unit": UNIT,
                                              "sample": f"{len(sample)} of the cases, 3 timed steps each"},
            "speedup_vs_plain_fp64": value / plain}


def run_served(args):
    """Served form: a Poisson request stream (50 requests/s) of 2-D cavity and
    2-D contraction cases (16k..65k cells), each a fixed number of steps,
    served by the continuous-batching loop in the mixed form; the same stream
    served one request at a time by the FP64 plain path for comparison."""
    import copy
    import numpy as np
    from rheotool_gb300 import abi
    from rheotool_gb300.case import cavity_case, contraction_case
    from rheotool_gb300.mesh import cavity_mesh, contraction_mesh
    from rheotool_gb300.serve import poisson_run
    rng = np.random.default_rng(20261203)
    meshes = {("cav", n): cavity_mesh(n) for n in (128, 160, 192, 224, 256)}
    for nx, ny in ((60, 20), (90, 30), (120, 40)):
        meshes[("con", nx)] = contraction_mesh(nx, nx, 2 * ny, ny, two_d=True)
    keys = list(meshes)
    cases = []
    for i in range(args.serve_requests):
        key = keys[int(rng.integers(0, len(keys)))]
        m = meshes[key]
        if key[0] == "cav":
            c = cavity_case(m.shape[0], model="GiesekusLog", Wi=float(rng.uniform(0.5, 2.0)), dt=1e-3, mesh=m,
                            alpha=0.1)
        else:
            c = contraction_case(m, dt=2e-3)
        c.precision = abi.RT_PREC_MIXED
        cases.append(c)
    served = poisson_run(cases, args.serve_steps, rate=50.0, slots=4, batch_cells=40000, batch_max=8,
                         quantum=5, hbm_budget=64 << 30)
    plain_cases = []
    for c in cases:
        c2 = copy.copy(c)
        c2.precision = abi.RT_PREC_FP64
        plain_cases.append(c2)
    plain = poisson_run(plain_cases, args.serve_steps, rate=50.0, slots=1, batch_cells=0, quantum=5,
                        hbm_budget=64 << 30)
    strip = lambda d: {k: v for k, v in d.items() if k != "requests_list"}
    out = {"workload": f"{len(cases)} requests, Poisson 50/s, 2-D cavity (128..256 side) and 2-D contraction "
                       f"(7k..29k cells) Giesekus cases, {args.serve_steps} steps each; mixed form, 4 slots, "
                       "small cases batched (requests join and leave running batches)",
           "served": strip(served), "plain_fp64_one_request_at_a_time": strip(plain),
           "speedup_p50": plain["p50_s"] / served["p50_s"] if served["p50_s"] else None,
           "speedup_throughput": served["cell_steps_per_s"] / plain["cell_steps_per_s"]}
    if args.serve3d_requests > 0:
        out["served_3d"] = run_served_3d(args)
    return out


def run_served_3d(args):
    """Served form on the serving config's sizes: a Poisson stream (50
    requests/s) of 3-D 4:1 contraction Giesekus cases of 16k..1M cells (size
    log-uniform, seeded), each a fixed number of steps (100 by default), in
    the mixed form on 4 slots; p50/p99 time to solution and aggregate
    cell-steps/s."""
    import numpy as np
    from rheotool_gb300 import abi
    from rheotool_gb300.case import contraction_case
    from rheotool_gb300.mesh import contraction_mesh
    from rheotool_gb300.serve import poisson_run
    rng = np.random.default_rng(20261204)
    cases = []
    for i in range(args.serve3d_requests):
        target = float(np.exp(rng.uniform(np.log(16e3), np.log(1e6))))
        f = (target / 1e6) ** (1.0 / 3.0)
        dims = dict(nx_up=max(4, round(134 * f)), nx_down=max(4, round(132 * f)), ny_in=max(4, round(50 * f)),
                    ny_out=max(2, round(25 * f)), nz=max(2, round(50 * f)))
        c = contraction_case(contraction_mesh(**dims))
        c.precision = abi.RT_PREC_MIXED
        cases.append(c)
    served = poisson_run(cases, args.serve3d_steps, rate=50.0, slots=4, batch_cells=0, quantum=10,
                         hbm_budget=96 << 30)
    cells = [c.mesh.nCells for c in cases]
    return {"workload": f"{len(cases)} requests, Poisson 50/s, 3-D planar 4:1 contraction GiesekusLog Wi 2, "
                        f"{min(cells):,}..{max(cells):,} cells (log-uniform in 16k..1M, seeded), "
                        f"{args.serve3d_steps} steps each; mixed form, 4 slots",
            "cells": cells, **{k: v for k, v in served.items() if k != "requests_list"}}


def run_precision_sweep(args):
    """Precision sweep: a channel periodic in x and z (4,000,000 cells by
    default), linear PTT-Log (epsilon 0.25, zeta 0, beta 1/9), Wi in {0.5, 2,
    8}, laminar velocity profile and a seeded lognormal initial conformation
    (theta = Q diag(0.1 z) Q^T, z ~ N(0, 1)^3, Q Haar-random; seed 20261203).
    For each Wi the same steps run in three forms from the same state: the
    FP64 plain form, the mixed form (FP32 Krylov iterations and sweeps, FP64
    residual replacement; FP32 constitutive algebra with FP64 eigen-solve
    fallback and exp back-transformation), and the FP64 form with every
    Krylov tolerance 100x tighter.  Reported per field: relative L2 of mixed
    vs FP64, of FP64 vs the tight FP64 (the solver-tolerance floor) and of
    mixed vs the tight FP64; and the device-timed cell-steps/s of each form."""
    import copy
    import numpy as np
    from rheotool_gb300 import abi
    from rheotool_gb300.case import SolverControl, periodic_channel_case, periodic_channel_state
    from rheotool_gb300.mesh import periodic_channel_mesh
    from rheotool_gb300.runtime import Context
    nx, ny, nz = (int(v) for v in args.sweep_dims.lower().split("x"))
    mesh = periodic_channel_mesh(nx, ny, nz)
    N = mesh.nCells
    names = ("U", "p", "phi", "theta", "tau")
    ctx = Context(0)
    result = {}
    for Wi in (0.5, 2.0, 8.0):
        case = periodic_channel_case(mesh, Wi=Wi)
        f0 = periodic_channel_state(case, sigma=0.1, seed=20261203)
        runs = {}
        for form in ("fp64", "mixed", "fp64_tight"):
            c = copy.copy(case)
            c.precision = abi.RT_PREC_MIXED if form == "mixed" else abi.RT_PREC_FP64
            if form == "fp64_tight":
                c.solverU, c.solverP, c.solverTheta = [
                    SolverControl(x.solver, x.preconditioner, x.tolerance * 1e-2, x.relTol, x.minIter,
                                  max(5 * x.maxIter, 4000)) for x in (case.solverU, case.solverP, case.solverTheta)]
            ctx.setup_case(c, f0.copy())
            ctx.sync()
            ctx.timer_start()
            perf = ctx.step(args.sweep_steps)
            ms = ctx.timer_stop()
            runs[form] = (ctx.fields(), ms, perf)
        err = lambda a, b: {n: float(np.linalg.norm(getattr(a, n) - getattr(b, n))
                                     / max(np.linalg.norm(getattr(b, n)), 1e-300)) for n in names}
        f64, fmx, ftt = runs["fp64"][0], runs["mixed"][0], runs["fp64_tight"][0]
        result[f"Wi={Wi:g}"] = {
            "mixed_vs_fp64": err(fmx, f64), "fp64_vs_fp64_tight": err(f64, ftt),
            "mixed_vs_fp64_tight": err(fmx, ftt),
            "cell_steps_per_s": {k: N * args.sweep_steps / (v[1] * 1e-3) for k, v in runs.items()},
            "p_iterations_last_step": {k: v[2].p.nIterations for k, v in runs.items()},
            "theta_max_abs": float(np.abs(f64.theta).max()),
        }
    ctx.close()
    return {"metric": "per-field relative L2 error of the mixed form vs the FP64 form (precision sweep)",
            "config": {"workload": f"3-D channel periodic in x and z, {nx}x{ny}x{nz} = {N:,} cells, walls at y=+-1, "
                                   "body-force driven (mean velocity 1), PTT-Log linear epsilon=0.25 zeta=0, "
                                   "beta=1/9, rho=0.01, dt=5e-3, Euler, GaussDefCmpw cubista, p PCG-DIC 1e-8, "
                                   "U/theta PBiCGStab-DILU 1e-10; theta0 = Q diag(0.1 z) Q^T seeded lognormal",
                       "steps": args.sweep_steps, "cells": N},
            "data": "synthetic", "results": result}


def lognormal_contraction_state(case, sigma=0.1, seed=20261203):
    """The contraction's initial fields with the seeded lognormal
    log-conformation of the precision sweep (theta = Q diag(sigma z) Q^T, z ~
    N(0, 1)^3, Q Haar-random): every cell's conformation eigenvalues apart,
    tau = etaP/lambda (A - I); U = 0, phi from the inlet."""
    import numpy as np
    from rheotool_gb300.case import Fields, lognormal_conformation
    m, md = case.mesh, case.model
    f = Fields.zeros(m)
    for p in m.patches:   # boundary values: fixed values from the BCs, the rest from the cells
        sl = slice(p.start, p.start + p.size)
        for name, nc in (("U", 3), ("p", 1), ("theta", 6), ("tau", 6)):
            kind, val = case.bcs[p.name][name]
            if kind == "fixedValue" and val is not None:
                getattr(f, name + "b")[sl] = np.broadcast_to(np.asarray(val, dtype=np.float64),
                                                             getattr(f, name + "b")[sl].shape)
    f.phib[:] = (m.bSf * f.Ub).sum(1)
    th, ev, vv = lognormal_conformation(m.nCells, sigma, seed)
    f.theta[:], f.eigVals[:], f.eigVecs[:] = th, ev, vv
    R = vv.reshape(-1, 3, 3)
    T = md.etaP / md.lambda_ * (np.einsum("nij,nj,nkj->nik", R, ev, R) - np.eye(3))
    f.tau[:] = np.stack([T[:, 0, 0], T[:, 0, 1], T[:, 0, 2], T[:, 1, 1], T[:, 1, 2], T[:, 2, 2]], axis=1)
    for p in m.patches:
        sl = slice(p.start, p.start + p.size)
        if case.bcs[p.name]["theta"][0] == "zeroGradient":
            f.thetab[sl] = f.theta[m.bCell[sl]]
    return f


def run_precision_check(args, case):
    """The mixed form against converged FP64 fields on the headline case
    itself.  From theta = 0 the contraction is ill-conditioned at round-off
    level (degenerate conformation eigenvalues: a 1e-16 inlet perturbation
    moves the FP64 theta by ~1e-2 within a few steps), so the comparison
    starts from the seeded lognormal conformation, where every cell's
    eigenvalues are apart.  Three runs of `steps` steps from that state: FP64
    with every Krylov tolerance x1e-2 ('tight'), FP64 with x1e-4 ('tighter';
    tight vs tighter is the floor: how converged the tight FP64 fields are)
    and the mixed form with every tolerance x1e-2 and no further tightening."""
    import copy
    import numpy as np
    from rheotool_gb300 import abi
    from rheotool_gb300.runtime import Context
    steps = args.check_steps
    f0 = lognormal_contraction_state(case)
    names = ("U", "p", "phi", "theta", "tau")
    runs = {}
    for key, prec, fac in (("fp64_tight", abi.RT_PREC_FP64, 1e-2), ("fp64_tighter", abi.RT_PREC_FP64, 1e-4),
                           ("mixed_tight", abi.RT_PREC_MIXED, 1e-2)):
        c = copy.copy(case)
        c.precision = prec
        c.solverU, c.solverP, c.solverTheta = [copy.copy(x) for x in (case.solverU, case.solverP, case.solverTheta)]
        for sctl in (c.solverU, c.solverP, c.solverTheta):
            sctl.tolerance *= fac
            sctl.maxIter = max(5 * sctl.maxIter, 5000)
        ctx = Context(0)
        ctx.set_option(abi.RT_OPT_MIXED_TIGHTEN, 0)
        ctx.setup_case(c, f0.copy())
        perf = ctx.step(steps)
        runs[key] = (ctx.fields(), {"p": perf.p.nIterations, "U": [perf.U[k].nIterations for k in range(3)],
                                    "p_converged": bool(perf.p.converged)})
        ctx.close()
    err = lambda a, b: {n: float(np.linalg.norm(getattr(a, n) - getattr(b, n))
                                 / max(np.linalg.norm(getattr(b, n)), 1e-300)) for n in names}
    return {"what": f"relative L2 after {steps} steps of the headline case from the seeded lognormal conformation "
                    "(sigma 0.1, seed 20261203)",
            "floor_fp64_tight_vs_tighter": err(runs["fp64_tight"][0], runs["fp64_tighter"][0]),
            "mixed_tight_vs_fp64_tighter": err(runs["mixed_tight"][0], runs["fp64_tighter"][0]),
            "mixed_tight_vs_fp64_tight": err(runs["mixed_tight"][0], runs["fp64_tight"][0]),
            "iterations_last_step": {k: v[1] for k, v in runs.items()}}


def run_reference(args, rank):
    """The reference algorithm on the host: the FP64 oracle on the same mesh
    (1,000,000 cells unless --small) and the same steps as the GPU arm's
    `value` (W untimed warm-up steps, then K timed), with every host thread
    it can use: its cell-local constitutive loops (source, eigen-
    decomposition, tau) run on all host cores; its Krylov sweeps and face
    loops are sequential, as one OpenFOAM process runs them."""
    if rank != 0:
        return
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    case = make_case(args.small)
    o = pyoracle.Oracle(case)
    if args.warmup:
        o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    cells = case.mesh.nCells
    v = cells * args.steps / dt
    workload = (WORKLOAD if not args.small else WORKLOAD.replace("1,000,000", f"{cells:,}")) + ", FP64 plain form"
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": workload, "cells": cells},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"the whole {cells:,}-cell case, steps {args.warmup + 1}..{args.warmup + args.steps} "
                                   "(the GPU arm's timed steps); rheoTool/OpenFOAM v9 is not buildable here, its FP64 "
                                   f"restatement runs with its cell-local constitutive loops on {threads} threads and "
                                   "its Krylov sweeps and face loops sequential, as one OpenFOAM process runs them"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.precision_sweep:
        if rank == 0:
            print(json.dumps(run_precision_sweep(args)), flush=True)
        return
    import numpy as np
    from rheotool_gb300 import abi
    from rheotool_gb300.runtime import Context

    pg = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        tdist.init_process_group("gloo")
        pg = tdist

    case = make_case(args.small)
    N, F, NB = case.mesh.nCells, case.mesh.nFaces, case.mesh.nBFaces
    prec = abi.RT_PREC_MIXED if args.precision == "mixed" else abi.RT_PREC_FP64
    other = abi.RT_PREC_FP64 if prec == abi.RT_PREC_MIXED else abi.RT_PREC_MIXED

    def timed(ctx, precision, clocks):
        case.precision = precision
        if precision == abi.RT_PREC_MIXED and args.mixed_precond is not None:
            ctx.set_option(abi.RT_OPT_MIXED_PRECOND, args.mixed_precond)
        ctx.setup_case(case)
        if args.warmup:
            ctx.step(args.warmup)
        ctx.sync()
        if pg:
            pg.barrier()
        clk = Clocks(local) if clocks else None
        k0 = ctx.kernel_count()
        ctx.timer_start()
        perf = ctx.step(args.steps)
        ms = ctx.timer_stop()
        launches = ctx.kernel_count() - k0
        clocks = clk.stop() if clk else None
        ms = rank_max(ms, pg)
        return ms, perf, launches, clocks

    def iters(perf):
        return {"p": perf.p.nIterations, "U": [perf.U[k].nIterations for k in range(3)],
                "theta": [perf.theta[k].nIterations for k in range(6)]}

    ctx = Context(local)
    ms, perf, launches, clocks = timed(ctx, prec, True)
    schedule = ctx.sweep_schedule()
    total_cells = N * args.steps * world
    value = whole_job_value(N, args.steps, world, ms)

    # ---- the other form on the same case, same steps; field differences ---
    second = None
    field_err = None
    floor = None
    names = ("U", "p", "phi", "theta", "tau")

    def rel_err(got, ref):
        return {n: float(np.linalg.norm(getattr(got, n) - getattr(ref, n))
                         / max(np.linalg.norm(getattr(ref, n)), 1e-300)) for n in names}

    if not args.no_plain:
        ctx2 = Context(local)
        ms2, perf2, launches2, _ = timed(ctx2, other, False)
        a, b = ctx.fields(), ctx2.fields()
        ref, got = (b, a) if prec == abi.RT_PREC_MIXED else (a, b)
        field_err = rel_err(got, ref)
        second = {"precision": "fp64" if other == abi.RT_PREC_FP64 else "mixed",
                  "value": total_cells / (ms2 * 1e-3), "ms_per_step": ms2 / args.steps,
                  "gpu_launches": launches2, "iterations_last_step": iters(perf2)}
        ctx2.close()
        case.precision = prec
        if not args.no_floor:
            # The FP64 form again with every Krylov tolerance 100x tighter: how far
            # the FP64 fields at the case's own tolerances are from converged
            # solves (the floor below which no two tolerance-stopped forms can
            # agree), and how far each form is from those converged fields.
            import copy
            saved = case.solverU, case.solverP, case.solverTheta
            tight = []
            for s_ in saved:
                t = copy.copy(s_)
                t.tolerance *= 1e-2
                t.maxIter = max(5 * s_.maxIter, 4000)
                tight.append(t)
            case.solverU, case.solverP, case.solverTheta = tight
            ctx3 = Context(local)
            ms3, perf3, _, _ = timed(ctx3, abi.RT_PREC_FP64, False)
            c = ctx3.fields()
            ctx3.close()
            case.solverU, case.solverP, case.solverTheta = saved
            case.precision = prec
            fp64_f, mixed_f = (b, a) if prec == abi.RT_PREC_MIXED else (a, b)
            floor = {"what": "relative L2 field differences after the same steps from the same state; "
                             "'tight' = FP64 form with every Krylov tolerance x1e-2",
                     "fp64_vs_fp64_tight": rel_err(fp64_f, c),
                     "mixed_vs_fp64_tight": rel_err(mixed_f, c),
                     "iterations_last_step_tight": iters(perf3), "ms_per_step_tight": ms3 / args.steps}

    # ---- roofline of the dominant operation (live CUDA events) ------------
    roof = None
    prof = {}
    if not args.no_profile:
        ctx.profile(True)
        ctx.step(2)
        prof = ctx.profile_report()
        ctx.profile(False)
        leaves = {k: v for k, v in prof.items() if not k.startswith("solve_") and v[2] > 0}
        if leaves:
            name = max(leaves, key=lambda k: leaves[k][1])
            n, tms, by = leaves[name]
            peak, src = peaks()
            achieved = (by / n) / (tms / n * 1e-3) / 1e9
            traffic = None
            tp = os.path.join(ROOT, "profiles", "traffic.json")
            if os.path.exists(tp):
                try:
                    tj = json.load(open(tp))
                    if name in tj:
                        traffic = tj[name]["dram_bytes_per_cell"] * N
                except Exception:
                    traffic = None
            roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)",
                    "traffic": traffic, "algorithmic_bytes_per_launch": by / n,
                    "launches_per_2_steps": n, "avg_launch_ms": tms / n,
                    "share_of_profiled_time": tms / max(sum(v[1] for k, v in prof.items()
                                                            if not k.startswith("solve_")), 1e-30)}

    # ---- end to end through the C ABI with host buffers -------------------
    # The same steps as `value` from the same state: a fresh case setup, W
    # warm-up steps, then K timed steps, each uploading U, p and phi from
    # pinned host memory, stepping once and downloading U, p, phi and tau.
    e2e = None
    if not args.no_e2e:
        try:
            import torch
            pin = lambda shape: torch.zeros(shape, dtype=torch.float64, pin_memory=True).numpy()
        except Exception:
            pin = lambda shape: np.zeros(shape)
        U, Ub, p, pb = pin((N, 3)), pin((NB, 3)), pin(N), pin(NB)
        phi, phib, tau = pin(F), pin(NB), pin((N, 6))
        up = ((abi.RT_FIELD_U, U, Ub), (abi.RT_FIELD_P, p, pb), (abi.RT_FIELD_PHI, phi, phib))
        case.precision = prec
        ctx.setup_case(case)
        for fid, a_, b_ in up:
            ctx.lib.rt_field_get(ctx._ctx, fid, abi.dptr(a_), abi.dptr(b_))
        for _ in range(args.warmup):
            for fid, a_, b_ in up:
                ctx.lib.rt_field_set(ctx._ctx, fid, abi.dptr(a_), abi.dptr(b_))
            ctx.step(1)
            for fid, a_, b_ in up:
                ctx.lib.rt_field_get(ctx._ctx, fid, abi.dptr(a_), abi.dptr(b_))
        ctx.sync()
        if pg:
            pg.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for fid, a_, b_ in up:
                st = ctx.lib.rt_field_set(ctx._ctx, fid, abi.dptr(a_), abi.dptr(b_))
                assert st == 0
            ctx.step(1)
            for fid, a_, b_ in up:
                st = ctx.lib.rt_field_get(ctx._ctx, fid, abi.dptr(a_), abi.dptr(b_))
                assert st == 0
            ctx.lib.rt_field_get(ctx._ctx, abi.RT_FIELD_TAU, abi.dptr(tau), None)
        dt = rank_max((time.perf_counter() - t0) * 1e3, pg) * 1e-3
        h2d = 8 * (3 * N + 3 * NB + N + NB + F + NB)
        d2h = h2d + 8 * 6 * N
        e2e = {"value": N * args.steps * world / dt, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": args.steps, "warmup": args.warmup,
               "path": "rt_field_set(U,p,phi) + rt_step(1) + rt_field_get(U,p,phi,tau) per step, pinned host "
                       "buffers, host wall clock; the same steps as value from the same initial state "
                       "(theta stays resident between steps, as between rheoFoam time steps)"}

    ctx.close()
    batched = None if (args.no_batch or args.small) else run_batched(args)
    served = None if (args.no_serve or args.small) else run_served(args)
    sweep = None if (args.no_sweep or args.small or rank != 0) else run_precision_sweep(args)
    check = None if (args.no_check or rank != 0) else run_precision_check(args, case)

    cpu = None
    if not args.no_cpu and rank == 0:
        cpu = cpu_baseline(args.cpu_seconds)

    if rank == 0:
        mixed = prec == abi.RT_PREC_MIXED
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64 (FP32 Krylov iterations and sweeps, FP64 residual replacement, FP64 assembly)"
                     if mixed else "f64",
            "data": "synthetic",
            "config": {"workload": (WORKLOAD if not args.small else WORKLOAD.replace("1,000,000", f"{N:,}"))
                                   + (", mixed-precision form" if mixed else ", FP64 plain form"),
                       "cells": N, "faces": F, "parallelism": f"replicas x{world} (independent cases)",
                       "l2": "inputs larger than L2: the step touches ~2 GB of fields and matrices per step",
                       "iterations_last_step": iters(perf),
                       "sweep_schedule_autotuned": schedule},
            "clocks": clocks, "gpu_launches": launches, "roofline": roof, "e2e": e2e, "cpu_baseline": cpu,
        }
        if second is not None:
            key = "plain_fp64" if mixed else "mixed_precision"
            second["speedup_mixed_vs_fp64"] = (value / second["value"]) if mixed else (second["value"] / value)
            second["field_error_vs_fp64"] = field_err
            line[key] = second
        if floor is not None:
            line["solver_tolerance_floor"] = floor
        line["profile_ms_2_steps"] = {k: round(v[1], 3) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}
        if prof:
            peak, _ = peaks()
            ops = {}
            for k, (n, tms, by) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
                if k.startswith("solve_") or by <= 0 or n == 0:
                    continue
                gbs = (by / n) / (tms / n * 1e-3) / 1e9
                ops[k] = {"launches": n, "avg_ms": round(tms / n, 5), "bytes_per_launch": by / n,
                          "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
            line["roofline_per_operation"] = ops
        if batched is not None:
            line["batched"] = batched
        if served is not None:
            line["served"] = served
        if sweep is not None:
            line["precision_sweep"] = sweep
        if check is not None:
            line["precision_check_headline"] = check
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
