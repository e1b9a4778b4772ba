"""The multi-rank logic of bench.py on CPU (gloo, two ranks): every rank
steps its own regions (distinct seeds, weak scaling) and the whole-job value
is all ranks' cells over the slowest rank's time."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out: str) -> None:
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 10.0 + 5.0 * rank            # rank 1 is the slow one
    ms = bench.max_over_ranks(local_ms, dist, device="cpu")
    value = bench.whole_job_rate(1000, world, ms * 1e-3)
    seed = bench.rank_seed(1002, rank)
    Path(out, f"r{rank}.txt").write_text(f"{ms} {value} {seed}")
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_max_time_and_distinct_regions(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r = [Path(tmp_path, f"r{i}.txt").read_text().split() for i in range(2)]
    for ms, value, _ in r:
        assert float(ms) == 15.0                      # the slowest rank
        assert float(value) == pytest.approx(2 * 1000 / 15e-3)
    assert r[0][2] != r[1][2]                         # each rank its own state
