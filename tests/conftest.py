import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and librheogpu.so")
    config.addinivalue_line("markers", "slow: long-running oracle cases")


@pytest.fixture(scope="session")
def ctx():
    from rheotool_gb300.runtime import Context
    c = Context(0)
    yield c
    c.close()


def pytest_terminal_summary(terminalreporter):
    """The bar each full-step GPU parity case passed at (plain 1e-9, or the
    round-off sensitivity bar of ill-conditioned cases), with its errors."""
    for name, mod in list(sys.modules.items()):
        if name.endswith("test_gpu_parity") and getattr(mod, "BAR_LOG", None):
            terminalreporter.write_sep("-", "step parity bars")
            for label, kind, errs, bar in mod.BAR_LOG:
                e = " ".join(f"{n}={v:.1e}" for n, v in errs.items())
                b = "" if bar is None else " bar " + " ".join(f"{n}={v:.1e}" for n, v in bar.items())
                terminalreporter.write_line(f"{label}: {kind}: {e}{b}")
