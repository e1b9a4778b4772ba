"""The multi-rank logic of bench.py on CPU (gloo ranks): every rank steps its
own block of regions (weak scaling) and the whole-job value is all ranks'
cells over the slowest rank's time; the regions split over ranks give the
single-process result bit for bit."""
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
    from nicam_kokkos_microphysics_gb300.state import shard_regions
    block = shard_regions(10 * world, rank, world)
    Path(out, f"r{rank}.txt").write_text(f"{ms} {value} {block.start}")
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
    assert r[0][2] != r[1][2]                         # each rank its own block of regions


def _shard_worker(rank: int, world: int, port: int, out: str, lall: int) -> None:
    """One rank: generate and step its own block of regions (the C
    restatement of the reference step, per region), then gather the blocks."""
    import pickle

    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    from nicam_kokkos_microphysics_gb300.state import StateSpec, make_state, region_view, shard_regions
    from oracle import restatement
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = StateSpec(gall=64, kall=42, lall=lall, seed=4242, variant="convective")
    mine = shard_regions(lall, rank, world)
    st = make_state(spec, out_fill=0.0, regions=mine)
    results = {}
    for i, l in enumerate(mine):
        reg = region_view(st, i)
        rc, status = restatement.mp_driver(reg, st["_gz"], st["_gzh"], spec.dt)
        assert rc == 0, status
        results[l] = reg
    gathered = [None] * world
    dist.all_gather_object(gathered, results)
    if rank == 0:
        merged = {}
        for part in gathered:
            merged.update(part)
        Path(out, "sharded.pkl").write_bytes(pickle.dumps(merged))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,lall", [(2, 5), (3, 4)])
def test_region_sharding_equals_single_process(tmp_path, world, lall):
    """Regions split over gloo ranks (shard_regions: contiguous blocks, no data
    exchanged) and stepped there give, gathered, the single-process step over
    all regions bit for bit: the property the weak-scaling benchmark (one
    block of regions per GPU, no collective on the data path) relies on."""
    import pickle

    import numpy as np
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sys.path.insert(0, str(ROOT))
    from nicam_kokkos_microphysics_gb300.state import (OUTPUT_NAMES, StateSpec, make_state, region_view,
                                                       shard_regions)
    from oracle import restatement
    restatement.build("strict")
    mp.spawn(_shard_worker, args=(world, _free_port(), str(tmp_path), lall), nprocs=world, join=True)
    merged = pickle.loads(Path(tmp_path, "sharded.pkl").read_bytes())
    assert sorted(merged) == list(range(lall))
    assert sorted(l for r in range(world) for l in shard_regions(lall, r, world)) == list(range(lall))
    spec = StateSpec(gall=64, kall=42, lall=lall, seed=4242, variant="convective")
    st = make_state(spec, out_fill=0.0)
    for l in range(lall):
        reg = region_view(st, l)
        rc, status = restatement.mp_driver(reg, st["_gz"], st["_gzh"], spec.dt)
        assert rc == 0, status
        for n in OUTPUT_NAMES:
            assert np.array_equal(reg[n].view(np.int64), merged[l][n].view(np.int64)), (l, n)
