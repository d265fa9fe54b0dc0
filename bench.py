"""Benchmark: MCAC aggregation steps per second on one GB300.

Workload (default): the 100 000-monomer box of the benchmark set --
LogNormal(30 nm, sigma_geo 1.25) diameters, 1000 ppm volume fraction,
T=1700 K, P=101300 Pa, rho=1800 kg/m3, kfe=1.4, dfe=1.8, no surface growth,
stop at 100 aggregates, seed 1. One "bench step" advances every replica of
that box by --mc-steps (default 2000) steps of the pick-move-collide-merge
loop; the metric is MC steps per second summed over replicas.

Arms:
  --impl ours       (default) R independent replicas of the box (seeds 1..R,
                    R = one per SM unless --replicas) advanced by the
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


def replica_models(n: int, base_seed: int):
    from mcac_gb300 import PhysicalModel
    models = []
    for i in range(n):
        pm = PhysicalModel(text=C2_INI)
        pm.set(random_seed=base_seed + i)
        models.append(pm)
    return models


def host_states(models):
    """The reference placement of every replica, on the host (parallel)."""
    from concurrent.futures import ThreadPoolExecutor

    from mcac_gb300 import init_state
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(init_state, models))


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
    models = replica_models(R, 1 + rank * R)
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
                   "replica_seeds": f"{1 + rank * R}..{R + rank * R}", "mc_steps_per_box_per_bench_step": M,
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
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)))
        return 0
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
