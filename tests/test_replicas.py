"""The N > 1 path of bench.py on CPU: world-size-2 gloo process groups (127.0.0.1).

Replicas only: every rank renders its own frame with no data-path collective; the host takes the
maximum step time over the ranks (rank_max) and reports every rank's units over it (whole_job).
The reference arm runs on rank 0 alone.
"""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, e2e = bench.rank_max([100.0 + 10 * rank, 50.0 - rank], world)
        dist.barrier()
        out.put((rank, ms, e2e, bench.whole_job(world, 1_000_000, ms), bench.dist_info()))
    finally:
        dist.destroy_process_group()


def test_rank_max_and_whole_job_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, e2e, value, info in res:
        assert (ms, e2e) == (110.0, 50.0)          # the slowest rank's time, on every rank
        assert value == pytest.approx(2 * 1_000_000 / 0.110 / 1e6)
        assert info == (rank, rank, 2)


def test_single_rank_is_identity(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.rank_max([3.0, 4.0], 1) == [3.0, 4.0]
    assert bench.whole_job(1, 2_000_000, 1000.0) == pytest.approx(2.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    args = bench.parse()
    assert bench.run_reference(args) is None     # returns before any work
    assert capsys.readouterr().out == ""
