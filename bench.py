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


def run_ensemble(args, rank: int, world: int) -> dict | None:
    """The 512-box ensemble to completion (or --cap-seconds): boxes/hour."""
    import numpy as np
    import torch

    from mcac_gb300 import Batch, PhysicalModel

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    inis = ensemble_inis(args.boxes)[rank::world]  # boxes are sharded across ranks
    models = [PhysicalModel(text=t) for t in inis]
    t0 = time.perf_counter()
    batch = Batch(models, stream=stream.cuda_stream)
    batch.threads = args.threads
    setup_s = time.perf_counter() - t0
    done_at = np.full(len(models), np.nan)
    sampler = ClockSampler(dev)
    sampler.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    kernel_ms, launches = 0.0, 0
    while True:
        # each box as fast as it goes; finish times read every second
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
    clocks = sampler.stop()
    st = batch.stats()
    steps = int(st["steps"].sum())
    n_done = int(np.isfinite(done_at).sum())
    failed = int((st["status"] != 0).sum())
    work = batch.work()
    threads_used = batch.threads
    # where the boxes with the most device time spend it
    box_work = [batch.box_work(k) for k in range(len(models))]
    box_cycles = np.array([sum(bw[c] for c in ("cycles_pick", "cycles_query", "cycles_move", "cycles_merge"))
                           for bw in box_work], dtype=np.float64)
    order = np.argsort(box_cycles)[::-1][:8]
    slowest = []
    for k in order:
        bw = box_work[int(k)]
        q = max(1, bw["queries"])
        cyc = sum(bw[c] for c in ("cycles_pick", "cycles_query", "cycles_move", "cycles_merge"))
        slowest.append({"box": int(k), "n_monomers": int(models[k].params.n_monomeres),
                        "aggregates_left": int(st["n_aggregates"][k]), "steps": int(st["steps"][k]),
                        "done_s": None if not np.isfinite(done_at[k]) else float(done_at[k]),
                        "cycles_per_step": cyc / q, "device_s": cyc / 2.07e9, "phase_share": phase_share(bw),
                        "per_query": {f: bw[f] / q for f in ("mov_spheres", "scanned", "cells", "candidates",
                                                             "cand_spheres", "refined")},
                        "per_merge": {f: bw[f] / max(1, bw["merges"]) for f in ("merged_spheres", "merge_pairs")}})
    batch.close()
    vals = torch.tensor([wall, float(steps), float(n_done), kernel_ms / 1000.0], device="cuda",
                        dtype=torch.float64)
    if world > 1:
        import torch.distributed as dist
        tmax, tsum = vals.clone(), vals.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        wall, steps, n_done = float(tmax[0]), int(tsum[1]), int(tsum[2])
    if rank != 0:
        return None
    fin_times = np.sort(done_at[np.isfinite(done_at)])
    res = {
        "metric": "boxes/hour", "value": n_done / wall * 3600.0, "unit": "boxes/h", "n_gpus": world,
        "steps": launches, "warmup": 0, "ms_per_step": 1000.0 * wall / max(1, launches),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": ENS_WORKLOAD, "boxes": args.boxes, "finished": n_done, "failed": failed,
                   "wall_s": wall, "cap_s": args.cap_seconds, "setup_s": round(setup_s, 2),
                   "launches": "at most 200 ms each, every box doing as many steps as fit",
                   "threads_per_box": threads_used,
                   "time_to_finish_s": {q: float(np.quantile(fin_times, p)) for q, p in
                                        (("p50", 0.5), ("p90", 0.9), ("max", 1.0))} if len(fin_times) else None},
        "mc_steps_per_s": steps / wall,
        "kernel_s": kernel_ms / 1000.0,
        "clocks": clocks,
        "gpu_launches": launches,
        "work": work,
        "phase_share": phase_share(work),
        "slowest_boxes": slowest,
    }
    if not args.no_cpu_baseline:
        res["cpu_baseline"] = ensemble_cpu_sample(inis, args.cpu_seconds)
    return res


def _ens_worker(job):
    ini, seconds = job
    from oracle import oracle_py
    box = oracle_py.OracleBox(ini)
    steps, t0 = 0, time.perf_counter()
    finished = False
    while time.perf_counter() - t0 < seconds:
        st, _ = box.calcul(max_steps=500)
        steps += int(st.steps)
        if st.finished:
            finished = True
            break
    dt = time.perf_counter() - t0
    box.close()
    return steps, dt, finished


def ensemble_cpu_sample(inis, seconds: float) -> dict:
    """The oracle on all host cores: one box per core from the start of the
    ensemble, each advanced for at most 'seconds'; MC steps/s summed."""
    import multiprocessing as mp
    procs = os.cpu_count() or 1
    jobs = [(ini, seconds) for ini in inis[:procs]]
    with mp.get_context("spawn").Pool(procs) as pool:
        res = pool.map(_ens_worker, jobs)
    return {"value": sum(r[0] / r[1] for r in res), "unit": "MC steps/s", "cores": procs, "kind": "port",
            "sample": f"the first {len(jobs)} boxes of the ensemble, one per core, up to {seconds:.0f} s each "
                      f"({sum(r[2] for r in res)} finished in that time)"}


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
    threads = args.threads or 32
    capacity = resident_boxes(threads)
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
                   "finished_to_criterion": finished, "capacity_slots": capacity, "threads_per_box": threads,
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
    ap.add_argument("--workload", default="c2", choices=["c2", "contact-search", "ensemble", "serve"],
                    help="c2: replicas of the 100k-monomer box (headline); contact-search: batched queries; "
                         "ensemble: the 512-box ensemble to completion (boxes/hour)")
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
        ref = run_contact_search_reference if args.workload == "contact-search" else run_reference
        print(json.dumps(ref(args)))
        return 0
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    runner = {"c2": run_ours, "contact-search": run_contact_search, "ensemble": run_ensemble,
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
