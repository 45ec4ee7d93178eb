"""The N>1 path of bench.py on CPU ranks (gloo, world size 2).

The path shards by file: each rank runs a replica of the workload, the ranks
meet only to take the slowest rank's time (all-reduce MAX), and the whole-job
figure is all ranks' bytes over that time.  The reference arm runs on rank 0
alone; other ranks exit without work."""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took 100 * (r + 1) ms for its replica
    ms = bench.max_over_ranks(100.0 * (rank + 1), dist, "cpu")
    gbs = bench.whole_job_gbs(10**9, world, 2, ms)
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.txt").write_text(f"{ms} {gbs}")


def test_slowest_rank_sets_the_whole_job_figure(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        ms, gbs = map(float, (tmp_path / f"rank{r}.txt").read_text().split())
        assert ms == 200.0
        # 2 replicas x 1 GB x 2 steps in 0.2 s
        assert abs(gbs - 20.0) < 1e-9


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.dist_setup(1) == (0, 1, 0) or "RANK" in os.environ


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        workload = "short_reads_100k"
        steps = 1
        warmup = 0
        gpus = 2

    assert bench.run_reference(Args, 1, 2) is None
    assert capsys.readouterr().out == ""
