"""Loading an OpenFOAM case directory (polyMesh, 0/, constant/, system/) into
the library's Case on the CPU: a lid-driven cavity written as OpenFOAM files
loads into the same case the builder makes (mesh, model, BCs, solver
controls, schemes) and the oracle steps both to the same fields; what the
library does not implement is refused unless substitutions are allowed."""
import os

import numpy as np
import pytest

from rheotool_gb300 import foam_io
from rheotool_gb300.case import cavity_case, lid_profile
from rheotool_gb300.foam_case import CaseError, load_case, parse_dict, run_case, scalar
from rheotool_gb300.mesh import YP, graded_nodes

HDR = 'FoamFile\n{{\n    version 2.0;\n    format ascii;\n    class {cls};\n    object {obj};\n}}\n'


def _write(path, cls, obj, body):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write(HDR.format(cls=cls, obj=obj) + body)


def _cavity_dir(root, n=8, solverU="PBiCGStab", ddt="Euler", lid="fixedValue"):
    xs = graded_nodes(0.0, 1.0, n)
    foam_io.write_structured_polymesh(os.path.join(root, "constant", "polyMesh"), xs, xs, np.array([-0.5, 0.5]),
                                      lambda d, i, j, k, Cf: np.zeros(i.size, np.int64) if d == YP
                                      else np.ones(i.size, np.int64),
                                      ["movingLid", "fixedWalls"], ["wall", "wall"], empty_z=True)
    mesh = foam_io.read_polymesh(root)
    lidU = lid_profile(mesh.bCf[mesh.patch("movingLid").start:][:mesh.patch("movingLid").size])
    lidv = "nonuniform List<vector> {}\n(\n{}\n)".format(len(lidU), "\n".join(
        f"({u[0]!r} {u[1]!r} {u[2]!r})" for u in lidU.tolist()))
    lidbc = (f"movingLid {{ type fixedValue; value {lidv}; }}" if lid == "fixedValue"
             else "movingLid { type codedFixedValue; value uniform (0 0 0); name movLid; }")
    _write(os.path.join(root, "0", "U"), "volVectorField", "U",
           "dimensions [0 1 -1 0 0 0 0];\ninternalField uniform (0 0 0);\nboundaryField\n{\n"
           f"    {lidbc}\n    fixedWalls {{ type fixedValue; value uniform (0 0 0); }}\n"
           "    frontAndBack { type empty; }\n}\n")
    _write(os.path.join(root, "0", "p"), "volScalarField", "p",
           "dimensions [0 2 -2 0 0 0 0];\ninternalField uniform 0;\nboundaryField\n{\n"
           "    \"(movingLid|fixedWalls)\" { type zeroGradient; }\n    frontAndBack { type empty; }\n}\n")
    _write(os.path.join(root, "0", "theta"), "volSymmTensorField", "theta",
           "dimensions [0 0 0 0 0 0 0];\ninternalField uniform (0 0 0 0 0 0);\nboundaryField\n{\n"
           "    movingLid { type zeroGradient; }\n    fixedWalls { type zeroGradient; }\n"
           "    frontAndBack { type empty; }\n}\n")
    _write(os.path.join(root, "0", "tau"), "volSymmTensorField", "tau",
           "dimensions [1 -1 -2 0 0 0 0];\ninternalField uniform (0 0 0 0 0 0);\nboundaryField\n{\n"
           "    movingLid { type linearExtrapolation; value uniform (0 0 0 0 0 0); }\n"
           "    fixedWalls { type linearExtrapolation; value uniform (0 0 0 0 0 0); }\n"
           "    frontAndBack { type empty; }\n}\n")
    _write(os.path.join(root, "constant", "constitutiveProperties"), "dictionary", "constitutiveProperties",
           "parameters\n{\n    type Oldroyd-BLog;\n    rho rho [1 -3 0 0 0 0 0] 0.01;\n"
           "    etaS etaS [1 -1 -1 0 0 0 0] 0.5;\n    etaP etaP [1 -1 -1 0 0 0 0] 0.5;\n"
           "    lambda lambda [0 0 1 0 0 0 0] 0.5;\n    stabilization coupling;\n}\n")
    _write(os.path.join(root, "system", "fvSolution"), "dictionary", "fvSolution",
           "solvers\n{\n    p { solver PCG; preconditioner DIC; tolerance 1e-8; relTol 0; maxIter 800; }\n"
           f"    U {{ solver {solverU}; preconditioner {{ preconditioner DILU; }} tolerance 1e-10; relTol 0; }}\n"
           "    \"(theta|tau)\" { solver PBiCGStab; preconditioner DILU; tolerance 1e-10; relTol 0; }\n}\n"
           "SIMPLE\n{\n    nInIter 1;\n    pRefCell 0;\n    pRefValue 0;\n}\n")
    _write(os.path.join(root, "system", "fvSchemes"), "dictionary", "fvSchemes",
           f"ddtSchemes {{ default {ddt}; }}\ndivSchemes\n{{\n    default none;\n"
           "    div(phi,U) GaussDefCmpw cubista;\n    div(phi,theta) GaussDefCmpw cubista;\n}\n")
    _write(os.path.join(root, "system", "controlDict"), "dictionary", "controlDict",
           "application rheoFoam;\ndeltaT 1e-3;\nendTime 0.003;\nwriteInterval 0.001;\n")
    return root


def test_parse_dict_and_scalars():
    d = parse_dict('FoamFile { version 2.0; }\n// c\nsolvers { "(U|theta)" { solver PBiCGStab; '
                   'preconditioner { preconditioner DILU; } } }\nrho rho [1 -3 0 0 0 0 0] 0.01;\nx 2e-3;')
    assert d["solvers"]["(U|theta)"]["preconditioner"]["preconditioner"] == "DILU"
    assert scalar(d["rho"]) == 0.01 and scalar(d["x"]) == 2e-3


def test_cavity_case_directory_loads_like_the_builder(tmp_path):
    from oracle.pyoracle import Oracle
    root = _cavity_dir(str(tmp_path / "cavity"))
    lc = load_case(root)
    ref = cavity_case(8)
    c = lc.case
    assert c.model.type == "Oldroyd-BLog" and c.model.rho == 0.01 and c.model.lambda_ == 0.5
    assert c.model.stabilization == "coupling" and c.divU == "cubista" and c.nInIter == 1
    assert (c.solverP.solver, c.solverP.preconditioner, c.solverP.tolerance, c.solverP.maxIter) == \
        ("PCG", "DIC", 1e-8, 800)
    assert (c.solverU.solver, c.solverU.preconditioner, c.solverTheta.solver) == ("PBiCGStab", "DILU", "PBiCGStab")
    assert c.deltaT == 1e-3 and lc.endTime == 0.003 and not lc.substitutions
    a, b = Oracle(ref), Oracle(c, lc.fields.copy())
    a.step(3)
    b.step(3)
    for name in ("U", "p", "phi", "theta", "tau"):
        x, y = getattr(b.f, name), getattr(a.f, name)
        assert np.linalg.norm(x - y) <= 1e-11 * max(np.linalg.norm(y), 1e-300), name


def test_unimplemented_entries_are_refused_or_substituted(tmp_path):
    root = _cavity_dir(str(tmp_path / "c1"), solverU="PBiCG", ddt="backward", lid="coded")
    with pytest.raises(CaseError, match="backward|codedFixedValue"):
        load_case(root)
    lc = load_case(root, substitute=True)
    text = " ".join(lc.substitutions)
    assert "backward -> Euler" in text and "codedFixedValue" in text
    assert lc.case.solverU.solver == "PBiCG"          # the tutorials' solver, run as written
    # the Cavity tutorial's Crank-Nicolson runs as written
    root2 = _cavity_dir(str(tmp_path / "c2"), ddt="CrankNicolson 0.9")
    lc2 = load_case(root2)
    assert (lc2.case.ddt, lc2.case.ddtPsi) == ("CrankNicolson", 0.9) and not lc2.substitutions
    lc2 = load_case(root, substitute=True, bc_overrides={"movingLid": {"U": ("fixedValue", lid_profile)}})
    assert callable(lc2.case.bcs["movingLid"]["U"][1])


def test_rheotool_external_solvers_and_relaxation(tmp_path):
    """The Cavity tutorial's form: p and U through rheoTool's eigenSolver
    (Eigen BiCGSTAB + ILUT) and relaxation factors of 1 are accepted as
    written only with substitutions; factors other than 1 are refused."""
    root = _cavity_dir(str(tmp_path / "c2"))
    path = os.path.join(root, "system", "fvSolution")
    _write(path, "dictionary", "fvSolution",
           "solvers\n{\n    \"(p|U)\"\n    {\n        solverType eigenSolver;\n        solver BiCGSTAB;\n"
           "        tolerance 1e-12;\n        maxIter 1000;\n        preconditioner { preconditioner ILUT; }\n    }\n"
           "    \"(theta|tau)\" { solver PBiCGStab; preconditioner { preconditioner DILU; } tolerance 1e-10; }\n}\n"
           "SIMPLE { nInIter 1; nNonOrthogonalCorrectors 0; pRefCell 0; pRefValue 0; }\n"
           "relaxationFactors { fields { p 1; } equations { U 1; } }\n")
    with pytest.raises(CaseError, match="eigenSolver"):
        load_case(root)
    lc = load_case(root, substitute=True)
    assert (lc.case.solverP.solver, lc.case.solverP.preconditioner, lc.case.solverP.tolerance) == ("PCG", "DIC", 1e-12)
    assert (lc.case.solverU.solver, lc.case.solverU.preconditioner) == ("PBiCGStab", "DILU")
    assert any("eigenSolver" in x for x in lc.substitutions)
    assert not any("relaxation" in x for x in lc.substitutions)
    with open(path) as f:
        text = f.read().replace("equations { U 1; }", "equations { U 0.7; }")
    with open(path, "w") as f:
        f.write(text)
    with pytest.raises(CaseError, match="relaxationFactors"):
        load_case(root)
    lc2 = load_case(root, substitute=True)
    assert any("relaxationFactors equations U: 0.7 -> 1" in x for x in lc2.substitutions)


def _props(root, body):
    _write(os.path.join(root, "constant", "constitutiveProperties"), "dictionary", "constitutiveProperties",
           "parameters\n{\n" + body + "\n}\n")


def test_model_keywords_as_the_reference_reads_them(tmp_path):
    """XPomPomLog and WhiteMetznerCYLog read their constructors' keywords
    (lambdaB for lambda; WhiteMetznerCYLog only with m = n, K = L, a = b);
    a missing keyword, a temperature function other than Constant, a
    generalized PTT function without positive alpha and beta and an unknown
    destruction function are refused as the reference would abort."""
    root = _cavity_dir(str(tmp_path / "m"))
    base = "rho 1; etaS 0.1; etaP 0.9; stabilization coupling;"
    _props(root, "type XPomPomLog; " + base + " lambdaB 0.5; lambdaS 0.2; alpha 0.15; q 2; n 0;")
    m = load_case(root).case.model
    assert (m.type, m.lambda_, m.lambdaS, m.alpha, m.q, m.n) == ("XPomPomLog", 0.5, 0.2, 0.15, 2.0, 0.0)
    _props(root, "type WhiteMetznerCYLog; " + base + " lambda 0.5; m 0.4; n 0.4; K 1; L 1; a 2; b 2;")
    m = load_case(root).case.model
    assert (m.type, m.lambda_, m.n, m.K, m.a) == ("WhiteMetznerCYLog", 0.5, 0.4, 1.0, 2.0)
    _props(root, "type WhiteMetznerCYLog; " + base + " lambda 0.5; m 0.5; n 0.4; K 1; L 1; a 2; b 2;")
    with pytest.raises(CaseError, match="m=n"):
        load_case(root)
    _props(root, "type XPomPomLog; " + base + " lambdaB 0.5; lambdaS 0.2; alpha 0.15; q 2;")
    with pytest.raises(CaseError, match="keyword n is undefined"):
        load_case(root)
    _props(root, "type GiesekusLog; " + base + " lambda 0.5; alpha 0.1;"
           " thermoLambda { type Arrhenius; alpha 3000; T0 320; }")
    with pytest.raises(CaseError, match="thermoLambda type Arrhenius"):
        load_case(root)
    # a non-isothermal case: the thermoFunction sub-dictionaries by the
    # model's own names
    m = load_case(root, thermo=True).case.model
    assert (m.thermoLambda.type, m.thermoLambda.alpha, m.thermoLambda.T0) == ("Arrhenius", 3000.0, 320.0)
    assert m.thermoEta.type == "Constant" and m.thermoLambda2.type == "Constant"
    _props(root, "type Rolie-PolyLog; " + base + " lambdaD 0.5; lambdaR 0.1; beta 0; delta -0.5; chiMax 5;"
           " thermoLambdaR { type WLF; c1 8.86; c2 101.6; T0 300; } thermoEta { type VFT; A 500; B -1; T0 150; }")
    m = load_case(root, thermo=True).case.model
    assert (m.thermoLambda2.type, m.thermoLambda2.c1, m.thermoLambda2.c2) == ("WLF", 8.86, 101.6)
    assert (m.thermoEta.type, m.thermoEta.A, m.thermoEta.B, m.thermoEta.T0) == ("VFT", 500.0, -1.0, 150.0)
    _props(root, "type GiesekusLog; " + base + " lambda 0.5; alpha 0.1; thermoEta { type WLF; c1 8.86; T0 300; }")
    with pytest.raises(CaseError, match="keyword c2 is undefined in thermoEta"):
        load_case(root, thermo=True)
    _props(root, "type GiesekusLog; " + base + " lambda 0.5; alpha 0.1; thermoEta { type Eyring; }")
    with pytest.raises(CaseError, match="Unknown thermoFunction type Eyring"):
        load_case(root, thermo=True)
    with pytest.raises(CaseError, match="no temperature field"):
        run_case(root, thermo=True)
    _props(root, "type PTTLog; " + base + " lambda 0.5; epsilon 0.25; zeta 0; alpha 0.8; beta 1.2;"
           " destructionFunctionType generalized; maxIterMittagLeffler 150;")
    m = load_case(root).case.model
    assert (m.destructionFunctionType, m.alpha, m.beta, m.maxIterMittagLeffler) == ("generalized", 0.8, 1.2, 150)
    _props(root, "type PTTLog; " + base + " lambda 0.5; epsilon 0.25; zeta 0; alpha 0.8; beta 0;"
           " destructionFunctionType generalized;")
    with pytest.raises(CaseError, match="should be positive"):
        load_case(root)
    _props(root, "type PTTLog; " + base + " lambda 0.5; epsilon 0.25; zeta 0; destructionFunctionType quadratic;")
    with pytest.raises(CaseError, match="quadratic"):
        load_case(root)


MULTIMODE_PARAMETERS = (
    "parameters\n{\n    type multiMode;\n    models\n    (\n"
    "        M1\n        {\n            type Oldroyd-BLog;\n            rho rho [1 -3 0 0 0 0 0] 0.01;\n"
    "            etaS etaS [1 -1 -1 0 0 0 0] 0.25;\n            etaP etaP [1 -1 -1 0 0 0 0] 0.3;\n"
    "            lambda lambda [0 0 1 0 0 0 0] 0.5;\n            stabilization coupling;\n        }\n"
    "        M2\n        {\n            type GiesekusLog;\n            rho rho [1 -3 0 0 0 0 0] 0.01;\n"
    "            etaS etaS [1 -1 -1 0 0 0 0] 0.25;\n            etaP etaP [1 -1 -1 0 0 0 0] 0.2;\n"
    "            lambda lambda [0 0 1 0 0 0 0] 0.1;\n            alpha alpha [0 0 0 0 0 0 0] 0.2;\n"
    "            stabilization coupling;\n        }\n    );\n}\n")


def multimode_cavity_dir(root, n=8, **kw):
    """The cavity case directory with a two-mode multiMode model laid out as
    rheoTool's multiMode tutorials are (Channel2D_VE/multiMode: 0/thetaM1,
    0/tauM1, 0/thetaM2, 0/tauM2 instead of 0/theta and 0/tau)."""
    _cavity_dir(root, n=n, **kw)
    _write(os.path.join(root, "constant", "constitutiveProperties"), "dictionary", "constitutiveProperties",
           MULTIMODE_PARAMETERS)
    for name in ("theta", "tau"):
        src = os.path.join(root, "0", name)
        text = open(src).read()
        for k in ("M1", "M2"):
            with open(src + k, "w") as fh:
                fh.write(text.replace(f"object      {name};", f"object      {name}{k};")
                         .replace(f"object {name};", f"object {name}{k};"))
        os.remove(src)
    return root


def test_multimode_case_directory_loads_like_the_builder(tmp_path):
    """A multiMode case directory: the modes in list order with their own
    fields, stepping as the same model built directly."""
    import copy
    from oracle.pyoracle import Oracle
    root = multimode_cavity_dir(str(tmp_path / "mm"))
    lc = load_case(root)
    c = lc.case
    assert lc.mode_names == ["M1", "M2"] and [m.type for m in c.models] == ["Oldroyd-BLog", "GiesekusLog"]
    assert len(lc.fields.modes) == 2 and not lc.substitutions
    ref = cavity_case(8)
    ref.model = copy.copy(c.models[0])
    ref.moreModes = [copy.copy(c.models[1])]
    a, b = Oracle(ref), Oracle(c, lc.fields.copy())
    a.step(3)
    b.step(3)
    for name in ("U", "p", "phi", "tau"):
        x, y = getattr(b.f, name), getattr(a.f, name)
        assert np.linalg.norm(x - y) <= 1e-11 * max(np.linalg.norm(y), 1e-300), name
    for mx, my in zip(b.f.modes, a.f.modes):
        assert np.linalg.norm(mx.theta - my.theta) <= 1e-11 * max(np.linalg.norm(my.theta), 1e-300)


def test_multimode_modes_must_share_rho_and_stabilization(tmp_path):
    root = multimode_cavity_dir(str(tmp_path / "mm2"))
    path = os.path.join(root, "constant", "constitutiveProperties")
    _write(path, "dictionary", "constitutiveProperties",
           MULTIMODE_PARAMETERS.replace("stabilization coupling;\n        }\n    );", "stabilization BSD;\n        }\n    );"))
    with pytest.raises(CaseError, match="share rho and stabilization"):
        load_case(root)
