"""Benchmark: MCAC aggregation steps per second on one GB300.

Workload (default): the 100 000-monomer box of the benchmark set --
LogNormal(30 nm, sigma_geo 1.25) diameters, 1000 ppm volume fraction,
T=1700 K, P=101300 Pa, rho=1800 kg/m3, kfe=1.4, dfe=1.8, no surface growth,
stop at 100 aggregates, seed 1. One "bench step" is a batch of MC steps
(--mc-steps, default 2000) of the pick-move-collide-merge loop; the metric is
MC steps per second.

Arms:
  --impl ours       (default) the host-driven loop of the C-ABI with the
                    contact search, translation and merge on the GPU; value
                    is timed with CUDA events on the box's stream, e2e adds
                    the upload of the state from host buffers and the
                    download of the final state through the C-ABI.
  --impl reference  the CPU restatement of the reference algorithm (oracle/)
                    on the host cores, one independent box per core, on a
                    bounded sample of the same workload.

Under torchrun each rank runs an independent replica (the single-box loop
has no data-parallel exchange): value = total steps of all ranks / max time.
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


def run_ours(args, rank: int, world: int) -> dict | None:
    import torch
    import numpy as np

    from mcac_gb300 import AggregatList, PhysicalModel, init_state
    from mcac_gb300._lib import StateBuffers

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    pm = PhysicalModel(text=C2_INI)
    if world > 1:
        pm.set(random_seed=int(pm.params.random_seed) + rank)
    t0 = time.perf_counter()
    sb = init_state(pm)
    init_s = time.perf_counter() - t0
    box = AggregatList(pm, sb, stream=stream.cuda_stream)
    box.set_profiling(True)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    M = args.mc_steps
    for _ in range(args.warmup):
        box.calcul(max_steps=M)
    box.take_profile()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(dev)
    sampler.start()
    total_ms = 0.0
    steps_done = 0
    for _ in range(args.steps):
        flush.zero_()  # L2 flushed between timed iterations (outside the events)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stats, _ = box.calcul(max_steps=M)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        steps_done += int(stats.steps)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    prof = box.take_profile()
    # end to end through the C-ABI with host buffers: upload, M steps, download
    snap = box.store()
    e2e_steps, e2e_s = 0, 0.0
    h2d = d2h = 0
    for _ in range(max(1, args.steps // 2)):
        sbuf = StateBuffers.from_snapshot(snap)
        h2d = int(sbuf.spheres.nbytes + sbuf.sphere_label.nbytes + sbuf.aggregates.nbytes + sbuf.n_spheres.nbytes
                  + sbuf.members.nbytes)
        torch.cuda.synchronize()
        t = time.perf_counter()
        with AggregatList(pm, sbuf, stream=stream.cuda_stream) as b2:
            st, _ = b2.calcul(max_steps=M)
            out = b2.store()
        e2e_s += time.perf_counter() - t
        e2e_steps += int(st.steps)
        d2h = int(out.spheres.nbytes + out.sphere_label.nbytes + out.aggregates.nbytes + out.n_spheres.nbytes
                  + out.members.nbytes)
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
    q_s = prof["query_ms"] / 1000.0
    achieved = qbytes / q_s / 1e9 if q_s > 0 else 0.0
    launches = int(prof["queries"] + prof["translates"] + 2 * prof["merges"])
    return {
        "metric": METRIC, "value": steps_all / wall, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall * 1000.0 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "100k-monomer box: LogNormal(30 nm, 1.25), 1000 ppm, 1700 K, seed 1, "
                               "stop at 100 aggregates", "n_monomers": 100000, "mc_steps_per_bench_step": M,
                   "path": "host-driven MC loop, contact search/translate/merge kernels on the GPU",
                   "parallelism": f"replicas x{world}", "l2": "flushed (256 MB write) between timed iterations",
                   "init_s": round(init_s, 3)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                     "kernel": "k_query", "bytes_per_launch": qbytes / max(1, prof["queries"]),
                     "us_per_launch": 1000.0 * prof["query_ms"] / max(1, prof["queries"])},
        "e2e": {"value": e2e_all / e2e_wall, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
        "profile": prof,
        "cpu_baseline": cpu_baseline_sample(args) if not args.no_cpu_baseline else None,
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
    ap.add_argument("--mc-steps", type=int, default=2000)
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
