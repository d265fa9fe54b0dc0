"""The multi-GPU split of the benchmarks, run as two gloo ranks on the CPU.

Boxes are independent, so N ranks share the work with no exchange on the
data path: each rank takes its own replicas of the 100k-monomer box
(disjoint seeds) or its own boxes of the ensemble, assigned by monomer count
(the device-memory footprint), and the ranks only reduce the timing scalars
(max of the wall times, sum of the steps). Checked here with world_size 2:
the shards are disjoint, cover the work and hold near-equal monomers; each
rank runs the two benchmark windows on its own boxes (with the oracle, the
CPU stand-in for a rank's GPU) and the reduced totals equal those of one
process running every box. A rank that dies between steps is learned of by
the others at their next exchange, as an error of the collective within the
process group's timeout, not as a hang.
"""
import os
import socket
import sys
from pathlib import Path

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent

# a small ensemble and short windows keep the ranks' box work to seconds
N_BOXES = 12
WINDOW = dict(agg_limit_a=60, steps_a=3000, steps_b=200, final_limit=1)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _small_inis():
    import bench
    inis = bench.ensemble_inis(256)
    return [t for t in inis if bench.ini_monomers(t) <= 700][:N_BOXES]


def _worker(rank: int, world: int, port: int, out_dir: str):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle_py
    n = 152
    seeds = [m.random_seed for m in bench.replica_models(n, rank)]
    inis = _small_inis()
    mine = bench.assign_boxes([bench.ini_monomers(t) for t in inis], world)[rank]
    results = {b: oracle_py.run_windows(inis[b], **WINDOW) for b in mine}
    steps = sum(r["steps_a"] + r["steps_b"] for r in results.values())
    # the timing reduction of the benchmarks: max wall time, summed steps
    t = torch.tensor([1.0 + rank, float(steps)], dtype=torch.float64)
    tmax, tsum = t.clone(), t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
    gathered = [None] * world
    dist.all_gather_object(gathered, (seeds, mine, {b: (r["steps_a"], r["steps_b"], r["n_aggregates_b"])
                                                    for b, r in results.items()}))
    if rank == 0:
        torch.save({"gathered": gathered, "wall": float(tmax[0]), "steps": float(tsum[1])},
                   os.path.join(out_dir, "result.pt"))
    dist.barrier()
    dist.destroy_process_group()


def test_assign_boxes_balances_monomers():
    sys.path.insert(0, str(ROOT))
    import bench
    sizes = [bench.ini_monomers(t) for t in bench.ensemble_inis(512)]
    for world in (1, 2, 3, 8):
        parts = bench.assign_boxes(sizes, world)
        flat = sorted(b for p in parts for b in p)
        assert flat == list(range(512))
        loads = [sum(sizes[b] for b in p) for p in parts]
        # greedy largest-first: no rank exceeds another by more than the largest box
        assert max(loads) - min(loads) <= max(sizes)
        assert parts == bench.assign_boxes(sizes, world)  # deterministic


def test_two_ranks_split_boxes_without_overlap(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = torch.load(tmp_path / "result.pt", weights_only=False)
    (s0, m0, r0), (s1, m1, r1) = res["gathered"]
    assert len(s0) == len(s1) == 152
    assert not set(s0) & set(s1)
    assert 257 not in s0 + s1  # the degenerate seed is skipped on every rank
    sys.path.insert(0, str(ROOT))
    from oracle import oracle_py
    inis = _small_inis()
    assert sorted(m0 + m1) == list(range(len(inis))) and not set(m0) & set(m1)
    # every box's work on its rank is that of one process running all boxes
    alone = {b: oracle_py.run_windows(inis[b], **WINDOW) for b in range(len(inis))}
    merged = {**r0, **r1}
    for b, r in alone.items():
        assert merged[b] == (r["steps_a"], r["steps_b"], r["n_aggregates_b"])
    assert res["wall"] == 2.0
    assert res["steps"] == float(sum(r["steps_a"] + r["steps_b"] for r in alone.values()))


def _dying_worker(rank: int, world: int, port: int, out_dir: str):
    """Rank 1 leaves between steps (nothing in flight); rank 0 must learn of it
    at its next exchange, as an error, not hang."""
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      MCACG_PG_TIMEOUT_S="5")
    import bench
    bench.init_ranks("gloo")
    if rank == 1:
        os._exit(3)  # a worker that dies
    try:
        bench.reduce_max_sum(torch.tensor([1.0, 2.0], dtype=torch.float64))
        outcome = "no error"
    except Exception as e:  # the dead peer surfaces as an error of the collective
        outcome = "detected: " + type(e).__name__
    Path(out_dir, "rank0.txt").write_text(outcome)
    os._exit(0)


def test_a_rank_that_dies_is_detected_by_the_others(tmp_path):
    import time
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_dying_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    t0 = time.monotonic()
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    alive = [p for p in procs if p.is_alive()]
    for p in alive:
        p.kill()
    assert not alive, "a rank hung"
    assert procs[1].exitcode == 3
    assert procs[0].exitcode == 0
    assert (tmp_path / "rank0.txt").read_text().startswith("detected")
    assert time.monotonic() - t0 < 120
