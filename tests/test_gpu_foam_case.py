"""An OpenFOAM/rheoTool case directory run on the GPU through
foam_case.run_case (the loader, the time loop, the field writer), against the
FP64 oracle stepping the same loaded case.

The directory takes the tutorials' own choices that the library runs as
written: the Cavity tutorial's ddtSchemes default "CrankNicolson 1"
(of90/tutorials/rheoFoam/Cavity/Oldroyd-BLog/system/fvSchemes:18) and the
Contraction41 tutorials' solvers, PCG-DIC for p and PBiCG-DILU for U and
theta (of90/tutorials/rheoFoam/Contraction41/Oldroyd-BLog/system/
fvSolution:18-51), with a non-orthogonal corrector.
"""
import os

import numpy as np
import pytest

from rheotool_gb300 import foam_io
from rheotool_gb300.foam_case import load_case, run_case

from test_foam_case import _cavity_dir, _write
from test_gpu_parity import TOL_STEP, rel

pytestmark = pytest.mark.gpu


def _tutorial_dir(root):
    _cavity_dir(root, n=12, solverU="PBiCG", ddt="CrankNicolson 1")
    _write(os.path.join(root, "system", "fvSolution"), "dictionary", "fvSolution",
           "solvers\n{\n    p { solver PCG; preconditioner DIC; tolerance 1e-10; relTol 0; maxIter 800; }\n"
           "    U { solver PBiCG; preconditioner { preconditioner DILU; } tolerance 1e-10; relTol 0; minIter 1; "
           "maxIter 1000; }\n"
           "    \"(theta|tau)\" { solver PBiCG; preconditioner { preconditioner DILU; } tolerance 1e-12; relTol 0; "
           "minIter 0; maxIter 1000; }\n}\n"
           "SIMPLE\n{\n    nInIter 1;\n    nNonOrthogonalCorrectors 1;\n    pRefCell 0;\n    pRefValue 0;\n}\n"
           "relaxationFactors\n{\n    fields { p 1; }\n    equations { U 1; theta 1; }\n}\n")
    _write(os.path.join(root, "system", "controlDict"), "dictionary", "controlDict",
           "application rheoFoam;\ndeltaT 1e-3;\nendTime 0.006;\nwriteInterval 0.003;\n")
    return root


def test_case_directory_runs_on_the_gpu_as_written(tmp_path):
    from oracle.pyoracle import Oracle
    root = _tutorial_dir(str(tmp_path / "cavityCN"))
    lc = load_case(root)                       # nothing refused, nothing substituted
    assert lc.substitutions == []
    c = lc.case
    assert (c.ddt, c.ddtPsi, c.nNonOrthCorr) == ("CrankNicolson", 1.0, 1)
    assert (c.solverU.solver, c.solverTheta.solver, c.solverP.solver) == ("PBiCG", "PBiCG", "PCG")
    run_case(root)                             # 6 steps, fields written at 0.003 and 0.006
    ref = Oracle(c, lc.fields.copy())
    mesh = c.mesh
    for t in ("0.003", "0.006"):
        ref.step(3)
        d = os.path.join(root, t)
        assert os.path.isdir(d), t
        for name, nc in (("U", 3), ("p", 1), ("theta", 6), ("tau", 6)):
            internal, _ = foam_io.read_field(os.path.join(d, name), n_internal=mesh.nCells)
            got = np.asarray(internal, dtype=np.float64).reshape(getattr(ref.f, name).shape)
            # written with 12 significant digits (writePrecision 12 of the tutorials)
            assert rel(got, getattr(ref.f, name)) < max(TOL_STEP, 1e-11), (t, name, rel(got, getattr(ref.f, name)))


def test_multimode_case_directory_runs_on_the_gpu(tmp_path):
    """A multiMode case directory (two modes, each with its own 0/theta<K>
    and 0/tau<K>) run by run_case on the GPU: the summed tau and every mode's
    theta and tau written at the write times equal the oracle's."""
    from oracle.pyoracle import Oracle
    from test_foam_case import multimode_cavity_dir
    root = multimode_cavity_dir(str(tmp_path / "mm"), n=12)
    lc = load_case(root)
    assert lc.mode_names == ["M1", "M2"]
    run_case(root)                             # 3 steps, fields written at 0.001, 0.002, 0.003
    ref = Oracle(lc.case, lc.fields.copy())
    mesh = lc.case.mesh
    for t in ("0.001", "0.002", "0.003"):
        ref.step(1)
        d = os.path.join(root, t)
        checks = [("U", 3, ref.f.U), ("p", 1, ref.f.p), ("tau", 6, ref.f.tau)]
        for i, k in enumerate(lc.mode_names):
            checks += [("theta" + k, 6, ref.f.modes[i].theta), ("tau" + k, 6, ref.f.modes[i].tau)]
        for name, nc, want in checks:
            internal, _ = foam_io.read_field(os.path.join(d, name), n_internal=mesh.nCells)
            got = np.asarray(internal, dtype=np.float64).reshape(want.shape)
            assert rel(got, want) < max(TOL_STEP, 1e-11), (t, name, rel(got, want))
