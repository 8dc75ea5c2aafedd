"""bench.py's multi-rank bookkeeping on CPU (gloo, world size 2): the path
shards into independent replicas, one per GPU, with no data-path collective;
the only exchange is the max-over-ranks of the timed region, and the
whole-job value counts every rank's cells.  The reference arm prints on rank
0 only; the other ranks exit without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.rank_max(10.0 + 5.0 * rank, dist)
    v = bench.whole_job_value(1000, 4, world, ms)
    q.put((rank, ms, v))
    dist.destroy_process_group()


def test_rank_max_and_whole_job_value_gloo():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, v in got:
        assert ms == 15.0                        # the slowest rank's time on every rank
        assert v == pytest.approx(1000 * 4 * 2 / 15e-3)


def test_single_rank_is_identity():
    import bench
    assert bench.rank_max(3.5, None) == 3.5
    assert bench.whole_job_value(10, 2, 1, 1000.0) == pytest.approx(20.0)


def test_reference_arm_other_ranks_do_no_work(capsys):
    import argparse
    import bench
    args = argparse.Namespace(gpus=2, steps=1, warmup=0)
    assert bench.run_reference(args, 1) is None
    assert capsys.readouterr().out == ""


def test_reference_arm_line_on_the_sample(capsys):
    """The reference arm's JSON line: FP64, every host thread (the oracle's
    cell-local loops), the same config keys as the GPU arm (run here on the
    126,675-cell sample, one step)."""
    import argparse
    import json
    import bench
    args = argparse.Namespace(gpus=1, steps=1, warmup=0, small=True)
    bench.run_reference(args, 0)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["dtype"] == "f64" and line["cpu_baseline"]["cores"] == (os.cpu_count() or 1)
    assert line["config"]["cells"] == 126675 and line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
