"""Benchmark: MCAC aggregation steps per second on one GB300.

Workload (default): the 100 000-monomer box of the benchmark set --
LogNormal(30 nm, sigma_geo 1.25) diameters, 1000 ppm volume fraction,
T=1700 K, P=101300 Pa, rho=1800 kg/m3, kfe=1.4, dfe=1.8, no surface growth,
stop at 100 aggregates, seed 1. One "bench step" advances every replica of
that box by --mc-steps (default 2000) steps of the pick-move-collide-merge
loop; the metric is MC steps per second summed over replicas.

Arms:
  --impl ours       (default) R independent replicas of the box (seeds 1..,
                    skipping DEGENERATE_SEEDS; R = the boxes the GPU keeps
                    resident at once unless --replicas) advanced by the
                    device-resident loop, one thread block per box; value is
                    timed with CUDA events on the launching stream; e2e goes
                    through the C-ABI from host buffers: upload of the R
                    states, --e2e-steps bench steps (statistics read back
                    after each), download of the R states. The line
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
oracle on one core). --workload ensemble runs the 512-box ensemble to
completion (or --cap-seconds) and reports boxes/hour, with the oracle's MC
steps/s on one box per host core beside it. --workload serve feeds a seeded
Poisson stream of runs to the continuous-batching server and reports p50/p99
run latency (arrival to completion).
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


# DRAM bytes per MC step of the batched loop on this machine, from one ncu
# capture of k_run (8 replicas x 200 steps, 32 threads per box): 10.76 MB
# read + 768 B written over 1,600 steps. The full-size launch (2432 boxes,
# ~185 GB) is too large to capture; its traffic grows with the steps done.
K_RUN_DRAM_BYTES_PER_STEP = 6.72e3
# DRAM bytes of one k_query_batch launch of the contact-search workload
# (10,000 queries on the 1,000,000-sphere snapshot), from one ncu capture.
K_QUERY_BATCH_DRAM_BYTES = 12.12e6
# DRAM bytes per MC step of k_run on the ensemble benchmark's window a, from
# one ncu capture of the full-size benchmark (1-pass metrics
# dram__bytes_read.sum + dram__bytes_write.sum, window a's launch: 72.1 GB
# read + 13.1 GB written over 18.15 M steps in 2.94 s). A small case of the
# same kernel that stays in L2 moves 1.28 kB per step.
K_RUN_ENS_DRAM_BYTES_PER_STEP = 4.69e3
K_RUN_ENS_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum (1 pass) of window a's k_run launch of "
                            "this benchmark at full size: 85.2 GB over 18.15 M MC steps, 4.69 kB per step, scaled "
                            "by the MC steps of one launch (window b's launch moves less per step)")


# Seeds whose reference initial state is degenerate: one monomer is drawn so
# far out in the log-normal tail that the volume-fraction rescaling shrinks
# every other sphere to about 1e-20 m and leaves that aggregate with a
# bounding radius far larger than the box, so every contact query scans the
# whole box. Found by scanning the initial states of seeds 1..2599.
DEGENERATE_SEEDS = frozenset({257})


def phase_share(prof: dict) -> dict:
    """Share of the device loop's SM cycles per phase of the MC step."""
    keys = ("cycles_pick", "cycles_query", "cycles_move", "cycles_merge")
    tot = sum(prof.get(k, 0) for k in keys)
    out = {k[7:]: (prof.get(k, 0) / tot if tot else None) for k in keys}
    # the query's own split: neighbourhood + filter, pairs + walk
    for k in ("cycles_query_scan", "cycles_query_pairs"):
        out[k[7:]] = prof.get(k, 0) / tot if tot else None
    return out


def replica_seeds(n: int, first: int) -> list[int]:
    """n seeds from 'first' upwards, skipping the degenerate ones."""
    seeds, s = [], first
    while len(seeds) < n:
        if s not in DEGENERATE_SEEDS:
            seeds.append(s)
        s += 1
    return seeds


def replica_models(n: int, rank: int = 0, monomers: int = 100000):
    from mcac_gb300 import PhysicalModel
    # disjoint seed ranges per rank
    seeds = replica_seeds(n * (rank + 1), 1)[n * rank:]
    text = C2_INI.replace("number = 100000", f"number = {int(monomers)}")
    models = []
    for seed in seeds:
        pm = PhysicalModel(text=text)
        pm.set(random_seed=seed)
        models.append(pm)
    return models


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

    from mcac_gb300 import Batch, resident_boxes

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    R = args.replicas or resident_boxes(32)  # the most boxes one wave holds
    models = replica_models(R, rank, args.monomers)
    # page-locked host arrays for the end-to-end leg, in one block made
    # before the host memory fragments (such blocks copy fastest)
    from mcac_gb300 import StateBuffers
    n_mono = int(models[0].params.n_monomeres)
    states = StateBuffers.many([(n_mono, n_mono)] * R, pinned=True)
    t0 = time.perf_counter()
    batch = Batch(models, stream=stream.cuda_stream)
    batch.threads = args.threads
    setup_s = time.perf_counter() - t0
    # the reference placements of the replicas, kept as host arrays
    states = batch.store_all(raw=True, out=states)
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
    threads_used = batch.threads
    steps_done = int(st["steps"].sum()) - steps0
    work1 = batch.work()
    prof = {k: work1[k] - work0[k] for k in work1}
    n_alive = st["n_aggregates"].tolist()
    batch.close()
    del flush
    # end to end through the C-ABI from host buffers: the R host states are
    # uploaded, advanced by K bench steps of M MC steps each (the per-box
    # statistics read back after every bench step), and downloaded
    state_bytes = sum(int(b.spheres.nbytes + b.sphere_label.nbytes + b.aggregates.nbytes + b.n_spheres.nbytes
                          + b.members.nbytes) for b in states)
    K = max(1, args.e2e_steps)
    # the results come back into the input arrays (already resident in host
    # memory; the upload has finished when the batch exists)
    outs = states
    torch.cuda.synchronize()
    t = time.perf_counter()
    stats_bytes = 0
    with Batch(models, stream=stream.cuda_stream, states=states) as b2:
        t_up = time.perf_counter() - t
        b2.threads = threads_used
        for _ in range(K):
            b2.run(max_steps=M, steps_per_launch=M)
            st2 = b2.stats()
            stats_bytes += int(st2.nbytes)
        e2e_steps = int(st2["steps"].sum())
        t_run = time.perf_counter() - t - t_up
        outs = b2.store_all(raw=True, out=outs)  # the final states in host arrays
        t_down = time.perf_counter() - t - t_up - t_run
    e2e_s = time.perf_counter() - t
    out_bytes = sum(int(o.spheres.nbytes + o.sphere_label.nbytes + o.aggregates.nbytes + o.n_spheres.nbytes
                        + o.members.nbytes) for o in outs)
    h2d = state_bytes // K
    d2h = (out_bytes + stats_bytes) // K
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
        "config": {"workload": f"{args.monomers // 1000}k-monomer box: LogNormal(30 nm, 1.25), 1000 ppm, 1700 K, "
                               "seed 1, stop at 100 aggregates", "n_monomers": args.monomers, "replicas_per_gpu": R,
                   "replica_seeds": f"{models[0].random_seed}..{models[-1].random_seed} on rank 0, skipping "
                                    f"{sorted(DEGENERATE_SEEDS)} (degenerate initial state)",
                   "mc_steps_per_box_per_bench_step": M,
                   "path": "device-resident MC loop, one thread block per box, one launch per bench step",
                   "parallelism": f"{R} independent replicas per GPU x {world} GPU",
                   "l2": "flushed (256 MB write) between timed iterations", "setup_s": round(setup_s, 2),
                   "threads_per_box": threads_used,
                   "aggregates_left": [min(n_alive), max(n_alive)]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": K_RUN_DRAM_BYTES_PER_STEP * steps_all / max(1, launches),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_run launch on "
                                       "8 replicas x 200 steps (32 threads per box), 6.7 kB per MC step, scaled "
                                       "by the MC steps of one launch",
                     "kernel": "k_run (batched MC loop)",
                     "bytes_per_launch": qbytes / max(1, launches), "us_per_launch": 1000.0 * total_ms / max(1, launches),
                     "bytes_model": "per contact query: 16 B x moving spheres + 36 B x aggregates scanned + 8 B x cells "
                                    "+ 16 B x candidate spheres + 64 B x FP64-refined pairs"},
        "e2e": {"value": e2e_all / e2e_wall, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "bench_steps": K, "note": "host states uploaded, K bench steps with per-box statistics read back "
                                          "after each, final states downloaded; bytes are per bench step",
                "upload_s": round(t_up, 3), "steps_s": round(t_run, 3), "download_s": round(t_down, 3)},
        "gpu_launches": launches,
        "clocks": clocks,
        "work": prof,
        "phase_share": phase_share(prof),
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
                     "peak_kind": peak_kind, "traffic": K_QUERY_BATCH_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_query_batch "
                                       "launch of this workload (9.90 MB + 0.71 MB)",
                     "kernel": "k_query_batch",
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


ENS_WORKLOAD = ("batched ensemble: 512 independent boxes, seed 1000+b, N ~ round(exp(U[ln 256, ln 16384])), "
                "50/50 monodisperse 30 nm or LogNormal(30 nm, 1.25), volume fraction ~ U[100, 5000] ppm, "
                "T ~ U[1500, 1900] K, stop at 1 aggregate or 10000 steps without an event")
# The two step windows of the ensemble benchmark. Window a runs every box
# from its initial placement until at most ENS_A_AGGREGATES aggregates are
# left (or ENS_A_STEPS steps, or a stop criterion); window b continues each
# box for ENS_B_STEPS more steps under its own criteria. A box's first
# ~10^5 steps are cheap on a CPU core; below ~100 aggregates one step costs
# the reference 1-100 ms, so a whole run to one aggregate takes a core hours
# for the largest boxes: window b samples that stage at a fixed step count.
ENS_A_AGGREGATES = 100
ENS_A_STEPS = 100_000
ENS_B_STEPS = 500
ENS_WINDOWS = (f"every box from its reference initial placement through window a (until at most "
               f"{ENS_A_AGGREGATES} aggregates are left, {ENS_A_STEPS} MC steps are done or a stop criterion "
               f"is met), then window b (the next {ENS_B_STEPS} MC steps under the box's own stop criteria)")


def init_ranks(backend: str) -> None:
    """Joins the ranks (RANK, WORLD_SIZE, MASTER_ADDR/PORT from the
    environment). A rank that dies or never arrives ends the others' next
    collective with an error after MCACG_PG_TIMEOUT_S seconds (default 600)
    instead of holding their GPUs: the ranks exchange only timing scalars,
    between steps, with no kernel in flight."""
    import datetime

    import torch.distributed as dist
    timeout = datetime.timedelta(seconds=float(os.environ.get("MCACG_PG_TIMEOUT_S", "600")))
    dist.init_process_group(backend, timeout=timeout)


def reduce_max_sum(t):
    """The benchmarks' only exchange: the max (wall and kernel times) and the
    sum (steps) of each rank's timing scalars."""
    import torch.distributed as dist
    tmax, tsum = t.clone(), t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
    return tmax, tsum


def ensemble_inis(n_boxes: int = 512, first_seed: int = 1000) -> list[str]:
    """Parameter files of the ensemble (seeded with numpy's PCG64 per box)."""
    import numpy as np
    inis = []
    for b in range(n_boxes):
        rng = np.random.Generator(np.random.PCG64(first_seed + b))
        n = int(round(np.exp(rng.uniform(np.log(256), np.log(16384)))))
        disp = 1.0 if rng.random() < 0.5 else 1.25
        fv = rng.uniform(100e-6, 5000e-6)
        temp = rng.uniform(1500, 1900)
        inis.append(f"[monomers]\nnumber = {n}\nmean_diameter = 30\ndispersion_diameter = {disp}\n"
                    f"initialisation_mode = lognormal\ndensity = 1800\n[environment]\nvolume_fraction = {fv!r}\n"
                    f"temperature = {temp!r}\npressure = 101300\nfractal_prefactor = 1.4\nfractal_dimension = 1.8\n"
                    f"[limits]\nnumber_of_aggregates = 1\nn_iter_without_event = 10000\n"
                    f"[numerics]\nrandom_seed = {first_seed + b}\nwith_domain_duplication = false\n")
    return inis


def ini_monomers(ini: str) -> int:
    for line in ini.splitlines():
        k, _, v = line.partition("=")
        if k.strip() == "number":
            return int(v)
    raise ValueError("no [monomers] number")


def assign_boxes(sizes: list[int], world: int) -> list[list[int]]:
    """Box indices per rank: largest box first to the rank holding the
    fewest monomers so far (device-memory footprint grows with the monomer
    count), so that ranks hold near-equal memory and work. Deterministic;
    every box goes to exactly one rank; each rank's list is in box order."""
    loads = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for b in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(world), key=lambda q: (loads[q], q))
        out[r].append(b)
        loads[r] += sizes[b]
    return [sorted(x) for x in out]


def ens_config(n_boxes: int) -> dict:
    """The workload description both arms print (identical by construction)."""
    return {"workload": ENS_WORKLOAD + "; " + ENS_WINDOWS, "boxes": n_boxes,
            "window_a": {"until_aggregates": ENS_A_AGGREGATES, "max_steps": ENS_A_STEPS},
            "window_b": {"steps": ENS_B_STEPS}, "seeds": f"1000..{999 + n_boxes}"}


def merge_bytes(prof: dict) -> float:
    """Algorithmic bytes of the merges counted in 'prof': the merged
    aggregate's FP64 sphere rows (72 B each), its 168-byte record and its
    intra-aggregate contact pairs (16 B each). The removed spheres' 32-byte
    rewrite is not counted (no per-merge count of removed spheres is kept;
    it is at most 32 B x merged spheres)."""
    return 72.0 * prof["merged_spheres"] + 168.0 * prof["merges"] + 16.0 * prof["merge_pairs"]


def _ens_models(inis, boxes, limit_a):
    from mcac_gb300 import PhysicalModel
    models = []
    for b in boxes:
        pm = PhysicalModel(text=inis[b])
        pm.set(number_of_aggregates_limit=limit_a)
        models.append(pm)
    return models


def _windows_once(models, states, outs, stream, flush, threads=0, a_steps=ENS_A_STEPS):
    """One bench step: upload the initial states, run window a then window b
    on the GPU, download the final states. Returns (kernel ms, wall s,
    steps, k_run launches, work counters, per-box stats, threads used)."""
    import torch

    from mcac_gb300 import Batch
    flush.zero_()  # L2 flushed between timed iterations
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = Batch(models, stream=stream.cuda_stream, states=states)  # host -> device
    b.threads = threads
    e0, em, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(stream)
    b.run(max_steps=a_steps, steps_per_launch=a_steps)
    la = b.last_run()[1]
    threads_a = (b.threads, b.speculation)
    steps_a = int(b.stats()["steps"].sum())
    em.record(stream)
    b.set_aggregate_limit(1)
    b.threads = threads  # chosen again for the later stage
    b.speculation = 0
    b.run(max_steps=ENS_B_STEPS, steps_per_launch=ENS_B_STEPS)
    lb = b.last_run()[1]
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    windows = {"a_ms": e0.elapsed_time(em), "b_ms": em.elapsed_time(e1), "a_steps": steps_a}
    st = b.stats()
    if outs is not None:
        b.store_all(raw=True, out=outs)  # device -> host
    wall = time.perf_counter() - t0
    work = b.work()
    threads_b = (b.threads, b.speculation)
    b.close()
    windows["b_steps"] = int(st["steps"].sum()) - steps_a
    return ms, wall, int(st["steps"].sum()), la + lb, work, st, (threads_a, threads_b), windows


def plain_single_box_windows(models, states, stream, flush, picks) -> dict:
    """The plain single-box GPU path: the same device loop with one box per
    launch (what mcacg_run_device runs), the same two windows, box by box."""
    tot_ms, tot_steps = 0.0, 0
    for k in picks:
        ms, _, steps, _, _, _, _, _ = _windows_once([models[k]], [states[k]], None, stream, flush)
        tot_ms += ms
        tot_steps += steps
    return {"value": tot_steps / (tot_ms / 1000.0), "unit": UNIT, "boxes": len(picks), "steps": tot_steps,
            "note": "one box per launch through the device-resident loop (mcacg_run_device's path), same windows, "
                    "boxes run one after another; a sample of the ensemble's boxes (every "
                    f"{max(1, len(models) // max(1, len(picks)))}th of this rank's)"}


def run_ensemble_windows(args, rank: int, world: int) -> dict | None:
    """The ensemble benchmark (default): MC steps/s over windows a and b."""
    import numpy as np
    import torch

    from mcac_gb300 import Batch, StateBuffers

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    inis = ensemble_inis(args.boxes)
    sizes = [ini_monomers(t) for t in inis]
    mine = assign_boxes(sizes, world)[rank]
    cpu_pool = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle_py  # the CPU sample's processes start before any GPU work
        cpu_pool = oracle_py.window_pool(os.cpu_count() or 1)
    t0 = time.perf_counter()
    models = _ens_models(inis, mine, ENS_A_AGGREGATES)
    # the reference placements (host, bit-identical with the reference),
    # kept in page-locked arrays; a second set receives the final states
    n = [int(m.params.n_monomeres) for m in models]
    states = StateBuffers.many([(k, k) for k in n], pinned=True)
    outs = StateBuffers.many([(k, k) for k in n], pinned=True)
    with Batch(models, stream=stream.cuda_stream) as b0:
        b0.store_all(raw=True, out=states)
    setup_s = time.perf_counter() - t0
    state_bytes = sum(int(s.spheres.nbytes + s.sphere_label.nbytes + s.aggregates.nbytes + s.n_spheres.nbytes
                          + s.members.nbytes) for s in states)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    for _ in range(args.warmup):
        _windows_once(models, states, outs, stream, flush, args.threads, args.a_steps or ENS_A_STEPS)  # untimed
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev)
    sampler.start()
    tot_ms = tot_wall = 0.0
    tot_steps = launches = 0
    work_sum: dict = {}
    threads_seen = set()
    out_bytes = 0
    win = {"a_ms": 0.0, "b_ms": 0.0, "a_steps": 0, "b_steps": 0}
    for _ in range(args.steps):
        ms, wall, steps, nl, work, st, th, w = _windows_once(models, states, outs, stream, flush, args.threads,
                                                             args.a_steps or ENS_A_STEPS)
        for k in win:
            win[k] += w[k]
        tot_ms += ms
        tot_wall += wall
        tot_steps += steps
        launches += nl + 1  # k_run launches + the window switch
        threads_seen.add(th)
        for k, v in work.items():
            work_sum[k] = work_sum.get(k, 0) + v
        out_bytes = sum(int(o.spheres.nbytes + o.sphere_label.nbytes + o.aggregates.nbytes + o.n_spheres.nbytes
                            + o.members.nbytes) for o in outs) + int(st.nbytes)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    last_stats = st
    times = torch.tensor([tot_ms / 1000.0, float(tot_steps), tot_wall], device="cuda", dtype=torch.float64)
    if world > 1:
        tmax, tsum = reduce_max_sum(times)
        kern_s, steps_all, wall_s = float(tmax[0]), float(tsum[1]), float(tmax[2])
    else:
        kern_s, steps_all, wall_s = float(times[0]), float(times[1]), float(times[2])
    completion = None
    if not args.no_completion:
        completion = ensemble_to_completion(args, inis, mine, states, stream, world)
    if rank != 0:
        return None
    peak, peak_kind = peaks()
    qb, mb = query_bytes(work_sum), merge_bytes(work_sum)
    achieved = (qb + mb) / kern_s / 1e9 if kern_s > 0 else 0.0
    out = {
        "metric": METRIC, "value": steps_all / kern_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": kern_s * 1000.0 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": ens_config(args.boxes) if not args.a_steps else dict(ens_config(args.boxes), profiling_case=
                  f"window a capped at {args.a_steps} steps"),
        "run": {"path": "device-resident MC loop, one thread block per box, all boxes of a window in one launch",
                "parallelism": f"{len(mine)} boxes on rank 0 of {world} (assigned by monomer count)",
                "l2": "flushed (256 MB write) before each bench step; states > L2",
                "setup_s": round(setup_s, 2),
                "threads_and_ctas_per_box": sorted(threads_seen),
                "windows": {"a": {"mc_steps_per_s": win["a_steps"] / (win["a_ms"] / 1e3) if win["a_ms"] else None,
                                  "ms_per_bench_step": win["a_ms"] / args.steps},
                            "b": {"mc_steps_per_s": win["b_steps"] / (win["b_ms"] / 1e3) if win["b_ms"] else None,
                                  "ms_per_bench_step": win["b_ms"] / args.steps}},
                "steps_per_bench_step": tot_steps // max(1, args.steps),
                "aggregates_after": {"min": int(last_stats["n_aggregates"].min()),
                                     "median": float(np.median(last_stats["n_aggregates"])),
                                     "max": int(last_stats["n_aggregates"].max())},
                "boxes_finished": int((last_stats["finished"] == 1).sum()),
                "boxes_failed": int((last_stats["status"] != 0).sum())},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None,
                     "kernel": "k_run (batched MC loop)",
                     "bytes_per_launch": (qb + mb) / max(1, launches - args.steps),
                     "us_per_launch": 1e6 * kern_s / max(1, launches - args.steps),
                     "bytes_model": "per contact query: 16 B x moving spheres + 36 B x aggregates scanned + 8 B x "
                                    "cells + 16 B x candidate spheres + 64 B x FP64-refined pairs; per merge: 72 B x "
                                    "merged spheres + 168 B + 16 B x contact pairs"},
        "e2e": {"value": steps_all / wall_s, "unit": UNIT, "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": out_bytes,
                "note": "per bench step: the initial states uploaded from page-locked host arrays, windows a and b "
                        "run, the final states and per-box statistics downloaded (wall clock)"},
        "gpu_launches": launches,
        "clocks": clocks,
        "work": work_sum,
        "phase_share": phase_share(work_sum),
    }
    k_traffic = K_RUN_ENS_DRAM_BYTES_PER_STEP
    if k_traffic:
        out["roofline"]["traffic"] = k_traffic * (steps_all / max(1, launches - args.steps))
        out["roofline"]["traffic_source"] = K_RUN_ENS_TRAFFIC_SOURCE
    if completion is not None:
        out["to_completion"] = completion
    if not args.no_plain:
        picks = list(range(0, len(models), max(1, len(models) // args.plain_boxes)))[:args.plain_boxes]
        out["plain_single_box"] = plain_single_box_windows(models, states, stream, flush, picks)
    if cpu_pool is not None:
        out["cpu_baseline"] = ens_cpu_sample(inis, cpu_pool, args.cpu_boxes)
        cpu_pool.close()
    else:
        out["cpu_baseline"] = None
    return out


def ensemble_to_completion(args, inis, mine, states, stream, world) -> dict:
    """Every box from its initial placement to its own stop criteria
    (1 aggregate or 10000 steps without an event): boxes/hour, with each
    box's finish time. Launches of at most 200 ms in which each box does as
    many steps as fit."""
    import numpy as np
    import torch

    from mcac_gb300 import Batch
    models = _ens_models(inis, mine, 1)
    with Batch(models, stream=stream.cuda_stream, states=states) as batch:
        done_at = np.full(len(models), np.nan)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kernel_ms, launches = 0.0, 0
        while True:
            batch.run_timed(1000.0)
            ms, nl = batch.last_run()
            kernel_ms += ms
            launches += nl
            st = batch.stats()
            now = time.perf_counter() - t0
            fin = (st["finished"] == 1) | (st["status"] != 0)
            done_at[fin & np.isnan(done_at)] = now
            if fin.all() or now > args.cap_seconds:
                break
        wall = time.perf_counter() - t0
        st = batch.stats()
        steps = int(st["steps"].sum())
        n_done = int(np.isfinite(done_at).sum())
        failed = int((st["status"] != 0).sum())
        box_work = [batch.box_work(k) for k in range(len(models))]
    vals = torch.tensor([wall, float(steps), float(n_done)], device="cuda", dtype=torch.float64)
    if world > 1:
        import torch.distributed as dist
        tmax, tsum = vals.clone(), vals.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        wall, steps, n_done = float(tmax[0]), int(tsum[1]), int(tsum[2])
    cyc = np.array([sum(bw[c] for c in ("cycles_pick", "cycles_query", "cycles_move", "cycles_merge"))
                    for bw in box_work], dtype=np.float64)
    slow = int(np.argmax(cyc))
    fin_times = np.sort(done_at[np.isfinite(done_at)])
    return {"boxes_per_hour": n_done / wall * 3600.0, "wall_s": wall, "finished": n_done, "failed": failed,
            "cap_s": args.cap_seconds, "mc_steps": steps, "mc_steps_per_s": steps / wall,
            "kernel_s": kernel_ms / 1000.0, "launches": launches,
            "time_to_finish_s": {q: float(np.quantile(fin_times, p)) for q, p in
                                 (("p50", 0.5), ("p90", 0.9), ("max", 1.0))} if len(fin_times) else None,
            "slowest_box": {"box": int(mine[slow]), "n_monomers": int(models[slow].params.n_monomeres),
                            "steps": int(st["steps"][slow]), "device_s": float(cyc[slow] / 2.07e9),
                            "done_s": float(done_at[slow]) if np.isfinite(done_at[slow]) else None,
                            "phase_share": phase_share(box_work[slow])},
            "note": "every box to its own stop criteria; launches of at most 200 ms, each box doing as many steps "
                    "as fit; the CPU reference is not run this far (one large box takes it hours)"}


def _ens_jobs(inis, boxes):
    sizes = [ini_monomers(inis[b]) for b in boxes]
    order = sorted(range(len(boxes)), key=lambda k: (-sizes[k], boxes[k]))  # largest first
    return [(boxes[k], inis[boxes[k]], ENS_A_AGGREGATES, ENS_A_STEPS, ENS_B_STEPS, 1) for k in order]


def _farm_summary(res, wall, procs) -> dict:
    steps = sum(r["steps_a"] + r["steps_b"] for _, r in res)
    return {"steps": steps, "wall_s": wall, "value": steps / wall,
            "steps_a": sum(r["steps_a"] for _, r in res), "steps_b": sum(r["steps_b"] for _, r in res),
            "cpu_s_a": sum(r["s_a"] for _, r in res), "cpu_s_b": sum(r["s_b"] for _, r in res),
            "procs": procs}


def ens_cpu_sample(inis, pool, n_boxes: int) -> dict:
    """The oracle on all host cores over a sample of the ensemble's boxes
    (every k-th box), the same two windows."""
    procs = os.cpu_count() or 1
    from oracle import oracle_py
    boxes = list(range(0, len(inis), max(1, len(inis) // n_boxes)))[:n_boxes]
    t = time.perf_counter()
    res = oracle_py.farm_windows(_ens_jobs(inis, boxes), procs, pool=pool)
    s = _farm_summary(res, time.perf_counter() - t, procs)
    return {"value": s["value"], "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{len(boxes)} of the {len(inis)} boxes (every {len(inis) // len(boxes)}th), both windows, "
                      f"farmed over {procs} processes, largest first ({s['steps']} MC steps in {s['wall_s']:.1f} s)"}


def run_ensemble_reference(args) -> dict:
    """The reference arm of the ensemble benchmark: the oracle (the C
    restatement of the reference, pinned to it) on every host core, over all
    boxes and both windows. The K timed bench steps each take 1/K of the
    boxes (box b in step b mod K); all are farmed at once, largest box first,
    so the cores stay busy, and the value is steps / wall time."""
    from oracle import oracle_py
    procs = os.cpu_count() or 1
    inis = ensemble_inis(args.boxes)
    pool = oracle_py.window_pool(procs)
    small = min(range(len(inis)), key=lambda b: ini_monomers(inis[b]))
    for _ in range(args.warmup):  # untimed: every worker once on a short run
        oracle_py.farm_windows([(small, inis[small], ENS_A_AGGREGATES, 2000, 0, 1)] * procs, procs, pool=pool)
    t = time.perf_counter()
    res = oracle_py.farm_windows(_ens_jobs(inis, list(range(len(inis)))), procs, pool=pool)
    wall = time.perf_counter() - t
    pool.close()
    s = _farm_summary(res, wall, procs)
    sample = (f"all {len(inis)} boxes, both windows, farmed over {procs} processes largest first "
              f"({s['steps']} MC steps: {s['steps_a']} in window a, {s['steps_b']} in window b; "
              f"{s['cpu_s_a']:.0f} + {s['cpu_s_b']:.0f} core-seconds); each box placed by the oracle's own "
              f"restatement of the reference placement")
    return {
        "impl": "reference", "metric": METRIC, "value": s["value"], "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": ens_config(args.boxes),
        "cpu_baseline": {"value": s["value"], "unit": UNIT, "cores": procs, "kind": "port", "sample": sample,
                         "host_cpus": os.cpu_count()},
        "e2e": {"value": s["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "windows": {"a_steps_per_s": s["steps_a"] / wall if wall else None,
                    "core_seconds": {"a": s["cpu_s_a"], "b": s["cpu_s_b"]}},
    }


SERVE_WORKLOAD = ("serving stream: seeded Poisson arrivals at --rate runs/s for --serve-seconds, "
                  "N ~ round(exp(U[ln 500, ln --serve-nmax])), LogNormal(30 nm, sigma_geo ~ U[1.1, 1.6]), "
                  "volume fraction ~ U[100, 5000] ppm, 1700 K, 30% with surface growth (flux 1e-3), "
                  "stop at 1 aggregate or 60 s of physical time")


def serve_requests(seconds: float, rate: float, nmax: int, seed: int = 5000) -> list[tuple[float, str, bool]]:
    """(arrival time, parameter file, surface-growth flag) of each request."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    out, t, k = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            return out
        n = int(round(np.exp(rng.uniform(np.log(500), np.log(nmax)))))
        fv = rng.uniform(100e-6, 5000e-6)
        sg = rng.uniform(1.1, 1.6)
        growth = bool(rng.random() < 0.3)
        growth_section = ("[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = 1e-3\n"
                          if growth else "")
        ini = (f"[monomers]\nnumber = {n}\nmean_diameter = 30\ndispersion_diameter = {sg!r}\n"
               f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = {fv!r}\ntemperature = 1700\n"
               f"{growth_section}[limits]\nnumber_of_aggregates = 1\nphysical_time = 60\n"
               f"[numerics]\nrandom_seed = {seed + 1 + k}\nwith_domain_duplication = false\n")
        out.append((t, ini, growth))
        k += 1


def run_serve(args, rank: int, world: int) -> dict | None:
    """Continuous batching of a seeded request stream: p50/p99 latency."""
    import numpy as np
    import torch

    from mcac_gb300 import PhysicalModel, Server, resident_boxes

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    reqs = serve_requests(args.serve_seconds, args.rate, args.serve_nmax, seed=5000 + rank)
    models = [PhysicalModel(text=ini) for _, ini, _ in reqs]
    threads = args.threads  # 0: each epoch at the largest size keeping every active run resident
    capacity = resident_boxes(threads or 32)
    budget = int(0.5 * torch.cuda.get_device_properties(dev).total_memory)
    lat, steps_done, finished = [], 0, 0
    sampler = ClockSampler(dev)
    with Server(capacity=capacity, memory_budget=budget, stream=stream.cuda_stream) as srv:
        srv.set_threads(threads)
        srv.set_epoch_ms(args.epoch_ms)
        sampler.start()
        t0 = time.perf_counter()
        nxt = 0
        while True:
            now = time.perf_counter() - t0
            while nxt < len(reqs) and reqs[nxt][0] <= now:
                srv.submit(models[nxt])
                nxt += 1
            active, pending = srv.step(args.epoch_steps)
            for c in srv.poll():
                lat.append(float(c["finish_s"] - c["submit_s"]))
                steps_done += int(c["steps"])
                finished += int(c["finished"] == 1 and c["status"] == 0)
            if nxt == len(reqs) and active == 0 and pending == 0:
                break
            if now > args.serve_seconds + args.cap_seconds:
                break
            if active == 0 and pending == 0 and nxt < len(reqs):
                time.sleep(max(0.0, min(0.01, reqs[nxt][0] - (time.perf_counter() - t0))))
        wall = time.perf_counter() - t0
        kernel_ms, launches = srv.kernel_time()
        clocks = sampler.stop()
    if rank != 0:
        return None
    lat = np.array(lat)
    q = (lambda p: float(np.quantile(lat, p)) if len(lat) else None)
    return {
        "metric": "run latency p50/p99", "value": q(0.5), "unit": "s", "n_gpus": world, "steps": launches,
        "warmup": 0, "ms_per_step": kernel_ms / max(1, launches), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "latency_s": {"p50": q(0.5), "p90": q(0.9), "p99": q(0.99), "max": q(1.0)},
        "config": {"workload": SERVE_WORKLOAD, "rate_per_s": args.rate, "arrival_seconds": args.serve_seconds,
                   "n_max": args.serve_nmax, "requests": len(reqs), "completed": int(len(lat)),
                   "finished_to_criterion": finished, "capacity_slots": capacity,
                   "threads_per_box": threads or "largest keeping every active run resident, per epoch",
                   "memory_budget_bytes": budget, "epoch_steps": args.epoch_steps, "epoch_ms": args.epoch_ms,
                   "wall_s": wall,
                   "surface_growth_requests": int(sum(g for _, _, g in reqs)),
                   "surface_growth": "flux_surfgrowth = 1e-3 kg/m^2/s on those requests (xsurfgrowth has no "
                                     "counterpart in the reference's parameters)"},
        "throughput": {"runs_per_s": len(lat) / wall, "mc_steps_per_s": steps_done / wall},
        "gpu_launches": launches,
        "clocks": clocks,
    }


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
    ap.add_argument("--replicas", type=int, default=0, help="boxes per GPU (0: as many as stay resident)")
    ap.add_argument("--monomers", type=int, default=100000,
                    help="monomers per box (the benchmark's box has 100000; smaller boxes for profiling)")
    ap.add_argument("--threads", type=int, default=0, help="threads per box (64/128/256; 0: timed at the first run)")
    ap.add_argument("--e2e-steps", type=int, default=5, help="bench steps between upload and download (e2e)")
    ap.add_argument("--plain-steps", type=int, default=500)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="ensemble", choices=["ensemble", "c2", "contact-search", "serve"],
                    help="ensemble (default): the 512-box ensemble through two step windows, MC steps/s, plus "
                         "its run to completion (boxes/hour); c2: replicas of the 100k-monomer box; "
                         "contact-search: batched queries; serve: the serving stream (p50/p99)")
    ap.add_argument("--no-completion", action="store_true", help="ensemble: skip the run to completion")
    ap.add_argument("--plain-boxes", type=int, default=8, help="ensemble: boxes of the plain single-box sample")
    ap.add_argument("--cpu-boxes", type=int, default=16, help="ensemble: boxes of the rank-0 CPU sample")
    ap.add_argument("--a-steps", type=int, default=0,
                    help="ensemble: cap of window a's steps (0: the benchmark's 100000); a smaller cap makes a small "
                         "profiling case of the same kernels")
    ap.add_argument("--boxes", type=int, default=512, help="ensemble boxes")
    ap.add_argument("--cap-seconds", type=float, default=240.0, help="ensemble / serving wall-time cap")
    ap.add_argument("--rate", type=float, default=50.0, help="serving arrivals per second")
    ap.add_argument("--serve-seconds", type=float, default=30.0, help="serving arrival window")
    ap.add_argument("--serve-nmax", type=int, default=5000, help="serving: largest request (monomers)")
    ap.add_argument("--epoch-steps", type=int, default=100000, help="serving: most MC steps per box per epoch")
    ap.add_argument("--epoch-ms", type=float, default=100.0, help="serving: wall-time cap of an epoch")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        ref = {"ensemble": run_ensemble_reference, "contact-search": run_contact_search_reference,
               "c2": run_reference}.get(args.workload)
        if ref is None:
            print(json.dumps({"impl": "reference", "unavailable": f"no CPU reference for --workload {args.workload}"}))
            return 0
        print(json.dumps(ref(args)))
        return 0
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        init_ranks("nccl")
    runner = {"c2": run_ours, "contact-search": run_contact_search, "ensemble": run_ensemble_windows,
              "serve": run_serve}[args.workload]
    out = runner(args, rank, world)
    if out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
