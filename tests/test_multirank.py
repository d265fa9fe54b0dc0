"""The multi-GPU split of the benchmarks, run as two gloo ranks on the CPU.

Boxes are independent, so N ranks share the work with no exchange on the
data path: each rank takes its own replicas of the 100k-monomer box
(disjoint seeds) or its own boxes of the ensemble (rank::world), and the
ranks only reduce the timing scalars (max of the wall times, sum of the
steps). Checked here with world_size 2: the shards are disjoint and cover
the work, and the reductions give the job totals.
"""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out_dir: str):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    n = 152
    seeds = [m.random_seed for m in bench.replica_models(n, rank)]
    inis = bench.ensemble_inis(64)[rank::world]
    # the timing reduction of run_ours: max wall time, summed steps
    t = torch.tensor([1.0 + rank, float(1000 * (rank + 1))], dtype=torch.float64)
    tmax, tsum = t.clone(), t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
    gathered = [None] * world
    dist.all_gather_object(gathered, (seeds, inis))
    if rank == 0:
        torch.save({"gathered": gathered, "wall": float(tmax[0]), "steps": float(tsum[1])},
                   os.path.join(out_dir, "result.pt"))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_split_boxes_without_overlap(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = torch.load(tmp_path / "result.pt", weights_only=False)
    (s0, e0), (s1, e1) = res["gathered"]
    assert len(s0) == len(s1) == 152
    assert not set(s0) & set(s1)
    assert 257 not in s0 + s1  # the degenerate seed is skipped on every rank
    sys.path.insert(0, str(ROOT))
    import bench
    all_inis = bench.ensemble_inis(64)
    assert sorted(e0 + e1) == sorted(all_inis) and not set(e0) & set(e1)
    assert res["wall"] == 2.0 and res["steps"] == 3000.0
