"""Benchmark: MCAC aggregation steps per second on one GB300.

Workload (default): the 100 000-monomer box of the benchmark set --
LogNormal(30 nm, sigma_geo 1.25) diameters, 1000 ppm volume fraction,
T=1700 K, P=101300 Pa, rho=1800 kg/m3, kfe=1.4, dfe=1.8, no surface growth,
stop at 100 aggregates, seed 1. One "bench step" advances every replica of
that box by --mc-steps (default 2000) steps of the pick-move-collide-merge
loop; the metric is MC steps per second summed over replicas.

Arms:
  --impl ours       (default) R independent replicas of the box (seeds 1..,
                    skipping DEGENERATE_SEEDS; R = one per SM unless
                    --replicas) advanced by the
                    device-resident loop, one thread block per box; value is
                    timed with CUDA events on the launching stream; e2e goes
                    through the C-ABI from host buffers: upload of the R
                    states, the steps, download of the R states. The line
                    also reports the plain host-driven single-box path
                    (the bit-exact drop-in form) and a one-core CPU sample.
  --impl reference  the CPU restatement of the reference algorithm (oracle/)
                    on all host cores, one independent replica per core, on
                    a bounded sample of the same workload.

Under torchrun each rank runs its own replicas (boxes are independent; no
exchange): value = total steps of all ranks / max time.

--workload contact-search times the contact-search microbenchmark instead:
10,000 queries on a 1,000,000-sphere synthetic snapshot per bench step, all
in one batched launch (metric: contact queries/s; the reference arm is the
oracle on one core).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

C2_INI = """[monomers]
number = 100000
density = 1800
mean_diameter = 30
dispersion_diameter = 1.25
initialisation_mode = lognormal

[environment]
volume_fraction = 1e-3
temperature = 1700
pressure = 101300
fractal_prefactor = 1.4
fractal_dimension = 1.8

[limits]
number_of_aggregates = 100

[numerics]
random_seed = 1
with_domain_duplication = false
"""

METRIC = "MC aggregation steps/s"
UNIT = "MC steps/s"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def query_bytes(prof: dict) -> float:
    """Algorithmic bytes of the contact queries counted in 'prof'.

    Per query: the moving aggregate's spheres (FP32 x,y,z,r: 16 B each), the
    aggregate records read from the scanned Verlet cells (x,y,z,rmax FP64:
    32 B + the 4-byte slot), the cell headers (8 B each), the candidates'
    spheres (16 B each) and the FP64 x,y,z,r of both spheres of every pair
    refined in FP64 (64 B).
    """
    return (16.0 * prof["mov_spheres"] + 36.0 * prof["scanned"] + 8.0 * prof["cells"]
            + 16.0 * prof["cand_spheres"] + 64.0 * prof["refined"])


# Seeds whose reference initial state is degenerate: one monomer is drawn so
# far out in the log-normal tail that the volume-fraction rescaling shrinks
# every other sphere to about 1e-20 m and leaves that aggregate with a
# bounding radius far larger than the box, so every contact query scans the
# whole box. Found by scanning the initial states of seeds 1..2599.
DEGENERATE_SEEDS = frozenset({257})


def replica_seeds(n: int, first: int) -> list[int]:
    """n seeds from 'first' upwards, skipping the degenerate ones."""
    seeds, s = [], first
    while len(seeds) < n:
        if s not in DEGENERATE_SEEDS:
            seeds.append(s)
        s += 1
    return seeds


def replica_models(n: int, rank: int = 0):
    from mcac_gb300 import PhysicalModel
    # disjoint seed ranges per rank
    seeds = replica_seeds(n * (rank + 1), 1)[n * rank:]
    models = []
    for seed in seeds:
        pm = PhysicalModel(text=C2_INI)
        pm.set(random_seed=seed)
        models.append(pm)
    return models


def host_states(models):
    """The reference placement of every replica, on the host. Sequential: it
    draws from the C library's single random stream."""
    from mcac_gb300 import init_state
    return [init_state(m) for m in models]


def plain_single_box(args, stream) -> dict:
    """The host-driven loop on one box (the bit-exact drop-in form)."""
    import torch

    from mcac_gb300 import AggregatList, PhysicalModel
    pm = PhysicalModel(text=C2_INI)
    with AggregatList(pm, stream=stream.cuda_stream) as box:
        box.set_profiling(True)
        box.calcul(max_steps=args.plain_steps)
        box.take_profile()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st, _ = box.calcul(max_steps=args.plain_steps)
        e1.record(stream)
        e1.synchronize()
        prof = box.take_profile()
    ms = e0.elapsed_time(e1)
    return {"value": st.steps / (ms / 1000.0), "unit": UNIT, "steps": int(st.steps),
            "query_us_per_launch": 1000.0 * prof["query_ms"] / max(1, prof["queries"]),
            "note": "one box, one contact query / translation (/ merge) kernel launch per MC step, "
                    "pick CDF on the host exactly as the reference (std::sort after every merge)"}


def run_ours(args, rank: int, world: int) -> dict | None:
    import torch

    from mcac_gb300 import Batch

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    R = args.replicas or torch.cuda.get_device_properties(dev).multi_processor_count
    models = replica_models(R, rank)
    t0 = time.perf_counter()
    batch = Batch(models, stream=stream.cuda_stream)
    setup_s = time.perf_counter() - t0
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    M = args.mc_steps
    for _ in range(args.warmup):
        batch.run(max_steps=M, steps_per_launch=M)
    torch.cuda.synchronize()
    steps0 = int(batch.stats()["steps"].sum())
    work0 = batch.work()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(dev)
    sampler.start()
    total_ms, launches = 0.0, 0
    for _ in range(args.steps):
        flush.zero_()  # L2 flushed between timed iterations (outside the events)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run(max_steps=M, steps_per_launch=M)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        launches += batch.last_run()[1]
    torch.cuda.synchronize()
    clocks = sampler.stop()
    st = batch.stats()
    steps_done = int(st["steps"].sum()) - steps0
    work1 = batch.work()
    prof = {k: work1[k] - work0[k] for k in work1}
    n_alive = st["n_aggregates"].tolist()
    batch.close()
    del flush
    # end to end through the C-ABI from host buffers: upload R states, M steps
    # per box, download R states
    states = host_states(models)
    h2d = sum(int(b.spheres.nbytes + b.sphere_label.nbytes + b.aggregates.nbytes + b.n_spheres.nbytes
                  + b.members.nbytes) for b in states)
    e2e_steps, e2e_s, d2h = 0, 0.0, 0
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        with Batch(models, stream=stream.cuda_stream, states=states) as b2:
            b2.run(max_steps=M, steps_per_launch=M)
            outs = [b2.store(k) for k in range(R)]
            e2e_steps += int(b2.stats()["steps"].sum())
        e2e_s += time.perf_counter() - t
        d2h = sum(int(o.spheres.nbytes + o.sphere_label.nbytes + o.aggregates.nbytes + o.n_spheres.nbytes
                      + o.members.nbytes) for o in outs)
    times = torch.tensor([total_ms / 1000.0, float(steps_done), e2e_s, float(e2e_steps)], device="cuda",
                         dtype=torch.float64)
    if world > 1:
        import torch.distributed as dist
        tmax = times.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        tsum = times.clone()
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        wall, steps_all, e2e_wall, e2e_all = float(tmax[0]), float(tsum[1]), float(tmax[2]), float(tsum[3])
    else:
        wall, steps_all, e2e_wall, e2e_all = float(times[0]), float(times[1]), float(times[2]), float(times[3])
    if rank != 0:
        return None
    peak, peak_kind = peaks()
    qbytes = query_bytes(prof)
    achieved = qbytes / (total_ms / 1000.0) / 1e9 if total_ms > 0 else 0.0
    out = {
        "metric": METRIC, "value": steps_all / wall, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall * 1000.0 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "100k-monomer box: LogNormal(30 nm, 1.25), 1000 ppm, 1700 K, seed 1, "
                               "stop at 100 aggregates", "n_monomers": 100000, "replicas_per_gpu": R,
                   "replica_seeds": f"{models[0].random_seed}..{models[-1].random_seed} on rank 0, skipping "
                                    f"{sorted(DEGENERATE_SEEDS)} (degenerate initial state)",
                   "mc_steps_per_box_per_bench_step": M,
                   "path": "device-resident MC loop, one thread block per box, one launch per bench step",
                   "parallelism": f"{R} independent replicas per GPU x {world} GPU",
                   "l2": "flushed (256 MB write) between timed iterations", "setup_s": round(setup_s, 2),
                   "aggregates_left": [min(n_alive), max(n_alive)]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None, "kernel": "k_run (batched MC loop)",
                     "bytes_per_launch": qbytes / max(1, launches), "us_per_launch": 1000.0 * total_ms / max(1, launches),
                     "bytes_model": "per contact query: 16 B x moving spheres + 36 B x aggregates scanned + 8 B x cells "
                                    "+ 16 B x candidate spheres + 64 B x FP64-refined pairs"},
        "e2e": {"value": e2e_all / e2e_wall, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
        "work": prof,
    }
    if not args.no_plain:
        out["plain_single_box"] = plain_single_box(args, stream)
    out["cpu_baseline"] = cpu_baseline_sample(args) if not args.no_cpu_baseline else None
    return out


CS_WORKLOAD = ("contact-search microbenchmark: 1,000,000 spheres LogNormal(30 nm, 1.5) in 20,000 ballistic "
               "aggregates of 1-500 spheres, 5000 ppm, 10,000 queries (uniform label, random_direction, length lpm)")
CS_METRIC, CS_UNIT = "contact queries/s", "queries/s"


def oracle_queries(case, n: int) -> tuple[float, int]:
    """Seconds the oracle takes for the first n queries of 'case' (1 core)."""
    from oracle import oracle_py
    ob = oracle_py.OracleBox(case.model.to_ini(), case.state.to_snapshot())
    t = time.perf_counter()
    for k in range(n):
        ob.distance_to_next_contact(case.sources[k], case.directions[k], case.distances[k])
    dt = time.perf_counter() - t
    ob.close()
    return dt, n


def run_contact_search(args, rank: int, world: int) -> dict | None:
    import torch

    from mcac_gb300 import AggregatList
    from mcac_gb300.workloads import contact_search_case

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    case = contact_search_case(seed=1 + rank)
    gen_s = time.perf_counter() - t0
    nq = len(case.sources)
    box = AggregatList(case.model, case.state, stream=stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    for _ in range(args.warmup):
        box.distance_to_next_contacts(case.sources, case.directions, case.distances)
    box.set_profiling(True)
    box.take_profile()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(dev)
    sampler.start()
    total_ms = 0.0
    for _ in range(args.steps):
        flush.zero_()  # the snapshot (about 100 MB) would otherwise stay in L2
        torch.cuda.synchronize()
        _, ms = box.distance_to_next_contacts(case.sources, case.directions, case.distances)
        total_ms += ms
    clocks = sampler.stop()
    prof = box.take_profile()
    box.set_profiling(False)
    # end to end: queries from host memory, results back to host memory
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        out, _ = box.distance_to_next_contacts(case.sources, case.directions, case.distances)
        e2e_s += time.perf_counter() - t
    box.close()
    times = torch.tensor([total_ms / 1000.0, e2e_s], device="cuda", dtype=torch.float64)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(times, op=dist.ReduceOp.MAX)
    wall, e2e_wall = float(times[0]), float(times[1])
    if rank != 0:
        return None
    peak, peak_kind = peaks()
    qbytes = query_bytes(prof)
    achieved = qbytes / (total_ms / 1000.0) / 1e9 if total_ms > 0 else 0.0
    res = {
        "metric": CS_METRIC, "value": world * nq * args.steps / wall, "unit": CS_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1000.0 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 (FP32 screen)",
        "data": "synthetic",
        "config": {"workload": CS_WORKLOAD, "queries_per_step": nq, "snapshot_seed": "1 + rank",
                   "generation_s": round(gen_s, 2), "l2": "flushed (256 MB write) between timed iterations",
                   "path": "mcacg_distance_to_next_contacts: one thread block per query, all queries in one launch",
                   "hits": int((out["moving_sphere"] >= 0).sum())},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None, "kernel": "k_query_batch",
                     "bytes_per_launch": qbytes / max(1, args.steps),
                     "us_per_launch": 1000.0 * total_ms / max(1, args.steps),
                     "bytes_model": "per contact query: 16 B x moving spheres + 36 B x aggregates scanned + 8 B x cells "
                                    "+ 16 B x candidate spheres + 64 B x FP64-refined pairs"},
        "e2e": {"value": world * nq * args.steps / e2e_wall, "unit": CS_UNIT,
                "h2d_bytes_per_step": int(case.sources.nbytes + case.directions.nbytes + case.distances.nbytes),
                "d2h_bytes_per_step": int(out.nbytes)},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "work": prof,
    }
    if not args.no_cpu_baseline:
        n = min(nq, 4000)
        dt, n = oracle_queries(case, n)
        res["cpu_baseline"] = {"value": n / dt, "unit": CS_UNIT, "cores": 1, "kind": "port",
                               "sample": f"the first {n} queries of the same snapshot, oracle, 1 core"}
    else:
        res["cpu_baseline"] = None
    return res


def run_contact_search_reference(args) -> dict:
    from mcac_gb300.workloads import contact_search_case
    case = contact_search_case(seed=1)
    n = len(case.sources)
    total = 0.0
    for _ in range(args.warmup):
        oracle_queries(case, min(n, 500))
    for _ in range(args.steps):
        dt, _ = oracle_queries(case, n)
        total += dt
    v = n * args.steps / total
    return {
        "impl": "reference", "metric": CS_METRIC, "value": v, "unit": CS_UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "config": {"workload": CS_WORKLOAD, "queries_per_step": n},
        "cpu_baseline": {"value": v, "unit": CS_UNIT, "cores": 1, "kind": "port",
                         "sample": f"all {n} queries per step, oracle, 1 core"},
        "e2e": {"value": v, "unit": CS_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def cpu_baseline_sample(args) -> dict | None:
    try:
        from oracle import oracle_py
    except Exception as exc:  # the oracle library is built by build()
        return {"value": None, "unavailable": f"oracle not importable: {exc}"}
    return oracle_py.bench_sample(C2_INI, seconds=args.cpu_seconds, processes=1)


def run_reference(args) -> dict:
    try:
        from oracle import oracle_py
    except Exception as exc:
        return {"impl": "reference", "unavailable": f"oracle not importable: {exc}"}
    procs = os.cpu_count() or 1
    res = oracle_py.bench_sample(C2_INI, seconds=args.cpu_seconds, processes=procs, steps=args.steps,
                                 warmup=args.warmup)
    return {
        "impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "100k-monomer box: LogNormal(30 nm, 1.25), 1000 ppm, 1700 K, seed 1, "
                               "stop at 100 aggregates", "n_monomers": 100000},
        "cpu_baseline": res,
        "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mc-steps", type=int, default=2000, help="MC steps per box per bench step")
    ap.add_argument("--replicas", type=int, default=0, help="boxes per GPU (0: one per SM)")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--plain-steps", type=int, default=500)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "contact-search"],
                    help="c2: replicas of the 100k-monomer box (headline); contact-search: batched queries")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        ref = run_contact_search_reference if args.workload == "contact-search" else run_reference
        print(json.dumps(ref(args)))
        return 0
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    out = (run_contact_search if args.workload == "contact-search" else run_ours)(args, rank, world)
    if out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
