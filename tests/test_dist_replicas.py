"""Multi-process (N > 1) path of bench.py on CPU: two gloo ranks run the
replicas-only aggregation -- the job's step time is the slowest rank's, its
work the sum of every rank's -- and the reference arm does no work on a rank
other than 0.  No GPU is touched."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (10 + 5r) ms per step for 2e9 * (r + 1) flops
        ms, value = bench.job_time_and_value(10.0 + 5.0 * rank, 2e9 * (rank + 1), world, "cpu")
        q.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_replicas_job_time_is_max_and_work_is_summed():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, ms, value in res:
        assert ms == pytest.approx(15.0)                       # the slower rank's time
        assert value == pytest.approx((2e9 + 4e9) / 15e-3 / 1e9)  # all ranks' flops over it


def test_reference_arm_is_rank0_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        workload = "rmat20"  # would take minutes if rank 1 did any work
        warmup = 3
        steps = 3
        ref_step_s = 8.0

    assert bench.run_reference(Args()) is None
    assert capsys.readouterr().out == ""
