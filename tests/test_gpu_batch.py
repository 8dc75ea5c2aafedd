"""Batched form: many independent cases of uneven size stepped as one device
mesh, through the C ABI.

Each case of a batch must give what it gives alone.  In FP64 the batch runs
the plain solvers' arithmetic per case, so each case's fields match the FP64
oracle at the plain path's bar (1e-9 relative L2, or the oracle's own
round-off sensitivity where a case is ill-conditioned).  In the mixed form a
case in a batch and the same case alone differ only by the grouping of their
reductions, so both satisfy the mixed form's bar against the oracle.
"""
import numpy as np
import pytest

from rheotool_gb300 import abi
from rheotool_gb300.batch import BatchContext, cavity_sweep, union_mesh
from rheotool_gb300.case import cavity_case, contraction_case
from rheotool_gb300.mesh import contraction_mesh

from test_gpu_parity import TOL_STEP, oracle_run, rel, step_bar

pytestmark = pytest.mark.gpu

NAMES = ("U", "p", "phi", "theta", "tau")


def small_sweep(precision):
    cases = cavity_sweep(n_cases=6, n_min=8, n_max=20, seed=7, dt=5e-3, precision=precision)
    return cases


def test_batch_fp64_matches_oracle_per_case():
    cases = small_sweep(abi.RT_PREC_FP64)
    bt = BatchContext(cases)
    try:
        bt.step(4)
        got = bt.fields()
        perf = bt.case_perf()
    finally:
        bt.ctx.close()
    for i, c in enumerate(cases):
        ref = oracle_run(c, 4)
        errs = {n: rel(getattr(got[i], n), getattr(ref, n)) for n in NAMES}
        if all(e < TOL_STEP for e in errs.values()):
            continue
        bar = step_bar(c, 4, ref, NAMES)
        for n in NAMES:
            assert errs[n] < bar[n], (i, c.model.type, n, errs[n], bar[n])
    assert all(p.p.converged for p in perf)


def test_batch_case_equals_case_alone_fp64(ctx):
    """Iteration counts and fields of each case: in the batch as alone."""
    cases = small_sweep(abi.RT_PREC_FP64)
    bt = BatchContext(cases)
    try:
        bt.step(3)
        got = bt.fields()
        perf = bt.case_perf()
    finally:
        bt.ctx.close()
    for i, c in enumerate(cases):
        ctx.setup_case(c)
        pa = ctx.step(3)
        alone = ctx.fields()
        assert abs(perf[i].p.nIterations - pa.p.nIterations) <= 1, (i, perf[i].p.nIterations, pa.p.nIterations)
        for k in range(2):
            assert abs(perf[i].U[k].nIterations - pa.U[k].nIterations) <= 1
        for n in NAMES:
            assert rel(getattr(got[i], n), getattr(alone, n)) < 1e-8, (i, n)


def test_batch_mixed_within_mixed_bar():
    from test_gpu_mixed import TOL_MIXED, _tightened
    import copy
    cases = small_sweep(abi.RT_PREC_MIXED)
    bt = BatchContext(cases)
    try:
        bt.step(4)
        got = bt.fields()
    finally:
        bt.ctx.close()
    for i, c in enumerate(cases):
        ref = oracle_run(c, 4)
        tight = copy.copy(c)
        tight.solverU, tight.solverP, tight.solverTheta = (_tightened(c.solverU), _tightened(c.solverP),
                                                            _tightened(c.solverTheta))
        ref_t = oracle_run(tight, 4)
        for n in NAMES:
            floor = rel(getattr(ref_t, n), getattr(ref, n))
            err = rel(getattr(got[i], n), getattr(ref, n))
            assert err < max(TOL_MIXED, 3.0 * floor), (i, n, err, floor)


def test_batch_level_sweeps_for_unstructured_cases():
    """A batch whose cases carry no 2-D box layout (here 3-D contractions)
    uses the level-scheduled sweeps over the union: same per-case results."""
    meshes = [contraction_mesh(8, 6, 6, 4, 3, 4.0, 4.0), contraction_mesh(10, 8, 6, 4, 4, 4.0, 4.0)]
    cases = [contraction_case(m) for m in meshes]
    for c in cases:
        c.precision = abi.RT_PREC_FP64
    bt = BatchContext(cases)
    try:
        bt.step(2)
        got = bt.fields()
    finally:
        bt.ctx.close()
    for i, c in enumerate(cases):
        ref = oracle_run(c, 2)
        for n in NAMES:
            assert rel(getattr(got[i], n), getattr(ref, n)) < TOL_STEP, (i, n)


def test_batch_layout_rejects_a_face_across_cases(ctx):
    from rheotool_gb300.runtime import RheoGpuError, _mesh_desc
    import ctypes as C
    cases = small_sweep(abi.RT_PREC_FP64)[:2]
    u, cs, fs, bs = union_mesh([c.mesh for c in cases])
    md = _mesh_desc(u, ctx)
    ctx._check(ctx.lib.rt_mesh_upload(ctx._ctx, C.byref(md)), "rt_mesh_upload")
    bad = cs.copy()
    bad[1] += 1                       # the first face of case 1 now joins two cases
    st = ctx.lib.rt_batch_layout(ctx._ctx, 2, abi.iptr(bad), abi.iptr(fs), abi.iptr(bs), None, None)
    assert st == abi.RT_EINVAL
    ctx.mesh = None


@pytest.mark.parametrize("precision", [abi.RT_PREC_FP64, abi.RT_PREC_MIXED])
def test_batch_persistent_solves_equal_launch_sequence(precision):
    """The batched pressure and momentum solves as one persistent CTA per
    case (all its iterations in one launch) take the per-iteration launch
    sequence's scalar decisions with one-pass reductions per case (the launch
    path sums 256-cell blocks first): iteration counts close, fields equal
    within the parity bars (1e-9 FP64, 1e-6 mixed, or the case's round-off
    sensitivity bar where it is larger)."""
    cases = cavity_sweep(n_cases=10, n_min=16, n_max=96, seed=9, dt=2e-3, precision=precision)
    out = {}
    for persistent in (0, 1):
        bt = BatchContext(cases)
        try:
            bt.ctx.set_option(abi.RT_OPT_BATCH_PERSISTENT, 2 if persistent else 0)
            bt.ctx.set_option(abi.RT_OPT_MIXED_PRECOND, 0)   # the same preconditioners on both paths
            bt.ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, 0)
            bt.step(3)
            out[persistent] = (bt.fields(), [(p.p.nIterations, p.U[0].nIterations, p.U[1].nIterations)
                                             for p in bt.case_perf()])
        finally:
            bt.ctx.close()
    # PCG within one iteration; BiCGStab's residual is not monotone, so a
    # round-off change moves its crossing of the tolerance by a few
    for a, b in zip(out[0][1], out[1][1]):
        assert abs(a[0] - b[0]) <= 1, (a, b)
        assert all(abs(i - j) <= max(5, 0.2 * i) for i, j in zip(a[1:], b[1:])), (a, b)
    assert max(i[0] for i in out[1][1]) > 20 and max(i[1] for i in out[1][1]) > 2
    plain = TOL_STEP if precision == abi.RT_PREC_FP64 else 1e-6
    for i, c in enumerate(cases):
        errs = {n: rel(getattr(out[1][0][i], n), getattr(out[0][0][i], n)) for n in NAMES}
        if all(e < plain for e in errs.values()):
            continue
        # round-off amplified by the case itself (conformation eigenvalues
        # degenerate at rest): the oracle's own sensitivity bar
        bar = step_bar(c, 3, oracle_run(c, 3), NAMES)
        for n in NAMES:
            assert errs[n] < max(plain, bar[n]), (i, n, errs[n], bar[n])


def test_batch_of_one_case_equals_the_case_alone(ctx):
    """A batch layout holding a single case (what a serving batch shrinks to
    when its other requests have left) runs the single-case path with the
    case's own pressure reference: the same bits as the case alone."""
    case = cavity_case(12, model="GiesekusLog", Wi=2.0, dt=5e-3, alpha=0.1)
    bt = BatchContext([case])
    try:
        bt.step(6)
        got = bt.fields()[0]
    finally:
        bt.ctx.close()
    ctx.setup_case(case)
    ctx.step(6)
    alone = ctx.fields()
    for n in NAMES:
        assert np.array_equal(getattr(got, n), getattr(alone, n)), n


def test_batch_of_256_row_cases_on_both_paths():
    """Cases of 256 rows (eight j-blocks: the largest per-case sweep, whose
    rings take the most shared memory) step through the launch sequence and
    through the persistent solvers, and the two agree."""
    cases = [cavity_case(256, model="GiesekusLog", Wi=1.0, dt=1e-3, alpha=0.1), cavity_case(40, dt=1e-3)]
    for c in cases:
        c.precision = abi.RT_PREC_MIXED
    out = []
    for mode in (0, 2):
        bt = BatchContext(cases)
        try:
            bt.ctx.set_option(abi.RT_OPT_BATCH_PERSISTENT, mode)
            bt.step(2)
            out.append((bt.fields(), [p.p.nIterations for p in bt.case_perf()]))
        finally:
            bt.ctx.close()
    assert min(out[0][1]) > 0 and min(out[1][1]) > 0
    for i in range(len(cases)):
        for n in NAMES:
            assert rel(getattr(out[1][0][i], n), getattr(out[0][0][i], n)) < 1e-6, (i, n)


def test_batch_persistent_multigrid_solves():
    """The mixed form's batched pressure and momentum solves with each case's
    multigrid V-cycle (RT_OPT_MIXED_PRECOND -2 and RT_OPT_MIXED_PRECOND_U -2,
    the defaults, in the persistent solvers; the momentum matrix is
    non-symmetric) against the exact DIC / DILU of the launch sequence: far
    fewer pressure iterations, fewer momentum iterations, fields within the
    mixed bar of each other."""
    cases = cavity_sweep(n_cases=10, n_min=16, n_max=96, seed=9, dt=2e-3, precision=abi.RT_PREC_MIXED)
    out = {}
    for mode in ("sweeps", "mg"):
        bt = BatchContext(cases)
        try:
            bt.ctx.set_option(abi.RT_OPT_BATCH_PERSISTENT, 2 if mode == "mg" else 0)
            bt.ctx.set_option(abi.RT_OPT_MIXED_PRECOND, -2 if mode == "mg" else 0)
            bt.ctx.set_option(abi.RT_OPT_MIXED_PRECOND_U, -2 if mode == "mg" else 0)
            bt.step(3)
            perf = bt.case_perf()
            assert all(p.p.converged and p.U[0].converged and p.U[1].converged for p in perf)
            out[mode] = (bt.fields(), [p.p.nIterations for p in perf],
                         [p.U[0].nIterations + p.U[1].nIterations for p in perf])
        finally:
            bt.ctx.close()
    assert sum(out["mg"][1]) < 0.5 * sum(out["sweeps"][1]), (out["mg"][1], out["sweeps"][1])
    assert sum(out["mg"][2]) < sum(out["sweeps"][2]), (out["mg"][2], out["sweeps"][2])
    for i, c in enumerate(cases):
        errs = {n: rel(getattr(out["mg"][0][i], n), getattr(out["sweeps"][0][i], n)) for n in NAMES}
        if all(e < 1e-6 for e in errs.values()):
            continue
        bar = step_bar(c, 3, oracle_run(c, 3), NAMES)
        for n in NAMES:
            assert errs[n] < max(1e-6, bar[n]), (i, n, errs[n], bar[n])
