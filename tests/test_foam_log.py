"""The OpenFOAM-format solver log (foam_log) from a step's records."""
from rheotool_gb300 import abi
from rheotool_gb300.case import cavity_case
from rheotool_gb300.foam_log import FoamLog, solver_name


def perf_record():
    p = abi.rt_step_perf()
    for k, (r0, r, n) in enumerate(((1.0, 2.5e-11, 4), (0.75, 1.25e-11, 5), (0.0, 0.0, -1))):
        p.U[k].initialResidual, p.U[k].finalResidual, p.U[k].nIterations = r0, r, n
    p.p.initialResidual, p.p.finalResidual, p.p.nIterations = 1.0, 9.5e-9, 123
    for k in range(6):
        solved = k in (0, 1, 3)
        p.theta[k].initialResidual = 0.5 if solved else 0.0
        p.theta[k].finalResidual = 1e-12 if solved else 0.0
        p.theta[k].nIterations = 2 if solved else -1
    p.contErrSumLocal, p.contErrGlobal = 1.5e-9, -2e-20
    return p


def test_solver_names_are_openfoams():
    c = cavity_case(4)
    assert solver_name(c.solverP) == "DICPCG"
    assert solver_name(c.solverU) == "DILUPBiCGStab"


def test_step_lines():
    c = cavity_case(4)                          # 2-D: Uz not solved
    log = FoamLog(c)
    lines = log.step(0.005, perf_record())
    assert lines[:3] == ["", "Time = 0.005", ""]
    assert lines[3] == "DILUPBiCGStab:  Solving for Ux, Initial residual = 1, Final residual = 2.5e-11, No Iterations 4"
    assert lines[4] == ("DILUPBiCGStab:  Solving for Uy, Initial residual = 0.75, Final residual = 1.25e-11, "
                        "No Iterations 5")
    assert lines[5] == "DICPCG:  Solving for p, Initial residual = 1, Final residual = 9.5e-09, No Iterations 123"
    assert lines[6] == "time step continuity errors : sum local = 1.5e-09, global = -2e-20, cumulative = -2e-20"
    assert [l.split(",")[0] for l in lines[7:]] == ["DILUPBiCGStab:  Solving for thetaxx",
                                                    "DILUPBiCGStab:  Solving for thetaxy",
                                                    "DILUPBiCGStab:  Solving for thetayy"]
    log.step(0.01, perf_record())
    assert log.lines[-4].endswith("cumulative = -4e-20")
    assert log.text().count("Time = ") == 2


def test_run_case_writes_one_log_block_a_step(tmp_path, monkeypatch):
    """run_case's time loop with a log steps one step at a time and writes
    one block per step (the context replaced by a stand-in that returns the
    initial fields and a fixed record: the loop and the log are host logic)."""
    import io
    import os

    from rheotool_gb300 import runtime
    from rheotool_gb300.foam_case import run_case
    from test_gpu_foam_case import _tutorial_dir

    calls = []

    class Stand:
        def __init__(self, device):
            pass

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def setup_case(self, case, fields):
            self.f = fields

        def step(self, n):
            calls.append(n)
            return perf_record()

        def fields(self):
            return self.f

    monkeypatch.setattr(runtime, "Context", Stand)
    root = _tutorial_dir(str(tmp_path / "cavity"))
    out = io.StringIO()
    run_case(root, log=out)
    text = out.getvalue()
    assert calls == [1] * 6
    assert [l for l in text.splitlines() if l.startswith("Time = ")] == [
        f"Time = {t:g}" for t in (0.001, 0.002, 0.003, 0.004, 0.005, 0.006)]
    assert text.count("DILUPBiCG:  Solving for Ux") == 6 and text.count("DICPCG:  Solving for p") == 6
    assert os.path.isdir(os.path.join(root, "0.003")) and os.path.isdir(os.path.join(root, "0.006"))
