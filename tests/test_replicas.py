"""Multi-GPU = replicas: host-side logic of the N > 1 bench path, on CPU ranks (gloo, world size 2).

The path has no collective on its data: every rank solves its own seeded workload and the job
time is the slowest rank's.  These tests run the bench's rank aggregation and the reference arm's
rank handling in real torch.distributed processes without a GPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: device times 100+10r (median of three steps), walls 150+20r, 3 steps in 600+60r ms
        dev = [100.0 + 10 * rank, 90.0 + 10 * rank, 130.0 + 10 * rank]
        walls = [150.0 + 20 * rank] * 3
        job = bench.replica_job(dev, walls, 600.0 + 60 * rank, 3, world)
        launches = bench.rank_sum(1000 + rank, world)
        dist.barrier()
        (Path(out_dir) / f"rank{rank}.txt").write_text(
            f"{job['value']} {job['e2e']} {job['ms_per_step']} {job['slowest_rank_ms']} {launches}")
    finally:
        dist.destroy_process_group()


def test_replica_job_takes_the_slowest_rank(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    rows = [list(map(float, (tmp_path / f"rank{r}.txt").read_text().split())) for r in range(world)]
    assert rows[0] == rows[1]                       # every rank sees the same job figures
    value, e2e, step, slow, launches = rows[0]
    assert slow == 110.0                            # median of rank 1's device times
    assert value == pytest.approx(110.0 / world)    # slowest rank / solves per job step
    assert e2e == pytest.approx(170.0 / world)
    assert step == pytest.approx(660.0 / 3)         # slowest rank's wall per step
    assert launches == 2001                         # kernels of the whole job


def test_replica_job_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    job = bench.replica_job([3.0, 1.0, 2.0], [5.0, 4.0, 6.0], 30.0, 3, 1)
    assert job["value"] == 2.0 and job["e2e"] == 5.0 and job["ms_per_step"] == 10.0
    assert bench.rank_sum(7, 1) == 7


def test_reference_arm_prints_only_on_rank_zero(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        warmup, steps, workload = 3, 2, "ico8_sh8"

    bench.run_reference(A())          # rank 1 returns at once: no work, no line
    assert capsys.readouterr().out == ""
