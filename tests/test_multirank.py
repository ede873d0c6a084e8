"""The N > 1 path of bench.py on the host: one process per rank as torchrun
launches them, two gloo ranks. Each rank times its own replica of the
workload (the voxels shard with no exchange); the job's time is the slowest
rank's, the value counts every rank's units, and the reference arm's other
ranks exit without work."""

from __future__ import annotations

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, seconds: list, out_dir: str) -> None:
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        job = bench.job_seconds(seconds[rank], dist, torch.device("cpu"))
        Path(out_dir, f"rank{rank}").write_text(repr(job))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_job_time_is_the_slowest_rank(tmp_path):
    import bench

    seconds = [0.75, 1.25]
    mp.spawn(_rank, args=(2, _free_port(), seconds, str(tmp_path)), nprocs=2, join=True)
    got = [float(Path(tmp_path, f"rank{r}").read_text()) for r in range(2)]
    assert got == [1.25, 1.25]
    # Every rank's units over the job's time: 2 ranks x 3 steps x 10 units / 1.25 s.
    assert bench.job_value(10.0, 3, 2, got[0]) == pytest.approx(48.0)
    assert bench.job_seconds(0.5, None, None) == 0.5


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2",
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    done = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
                           "--steps", "1", "--warmup", "3"], cwd=ROOT, env=env,
                          capture_output=True, timeout=300)
    assert done.returncode == 0, done.stderr.decode()[-2000:]
    assert done.stdout.strip() == b""
