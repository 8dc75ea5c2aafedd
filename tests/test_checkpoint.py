"""Checkpoint snapshots on the CPU: the .npz round trip is exact (single- and
multiMode), and snapshots of another case are refused."""
import numpy as np
import pytest

from rheotool_gb300 import checkpoint
from rheotool_gb300.case import Fields, cavity_case

from test_gpu_parity import multimode_case


def random_fields(case, rng):
    f = Fields.zeros(case.mesh, len(case.models))
    for name, a in f.__dict__.items():
        if isinstance(a, np.ndarray):
            a[...] = rng.standard_normal(a.shape)
    for m in f.modes:
        for a in m.__dict__.values():
            a[...] = rng.standard_normal(a.shape)
    return f


@pytest.mark.parametrize("modes", [False, True])
def test_snapshot_round_trip_is_exact(tmp_path, modes):
    case = cavity_case(6, model="GiesekusLog", alpha=0.1)
    if modes:
        case = multimode_case(case)
    f = random_fields(case, np.random.default_rng(5))
    path = str(tmp_path / "snap.npz")
    checkpoint.save_fields(path, case, f, step=17, time=0.085)
    g, meta = checkpoint.load_fields(path, case)
    assert meta == {"step": 17, "time": 0.085}
    for name, a in f.__dict__.items():
        if isinstance(a, np.ndarray):
            assert np.array_equal(getattr(g, name), a), name
    assert len(g.modes) == len(f.modes)
    for gm, fm in zip(g.modes, f.modes):
        for name, a in fm.__dict__.items():
            assert np.array_equal(getattr(gm, name), a), name


def test_snapshot_of_another_case_is_refused(tmp_path):
    case = cavity_case(6, model="GiesekusLog", alpha=0.1)
    path = str(tmp_path / "snap.npz")
    checkpoint.save_fields(path, case, random_fields(case, np.random.default_rng(6)))
    with pytest.raises(ValueError, match="cells/faces"):
        checkpoint.load_fields(path, cavity_case(7))
    with pytest.raises(ValueError, match="models"):
        checkpoint.load_fields(path, cavity_case(6, model="PTTLog", epsilon=0.25))
    cn = cavity_case(6, model="GiesekusLog", alpha=0.1)
    cn.ddt = "CrankNicolson"
    with pytest.raises(ValueError, match="CrankNicolson"):
        checkpoint.load_fields(path, cn)
    with pytest.raises(ValueError, match="CrankNicolson"):
        checkpoint.save_fields(path, cn, random_fields(cn, np.random.default_rng(7)))
