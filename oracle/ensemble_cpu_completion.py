"""Runs a sample of the 512-box benchmark ensemble to completion on the CPU.

The benchmark's CPU arm cannot run the ensemble to completion (a large box
takes a core hours), so the boxes/hour of the GPU's run to completion has no
CPU number measured in the same run. This script measures one: every 16th
box (32 boxes, the same seeded placements and stop criteria as bench.py's
ensemble) run to its stop criteria by the oracle's C restatement, one box
per process, largest first, printing per box: box, monomers, MC steps,
aggregates left and wall seconds (one JSON list per line). Scaled by 16, the
sum estimates the core-seconds of the whole ensemble.

Run from the repository root (hours on 8 cores):

    python oracle/ensemble_cpu_completion.py [processes]
"""
from __future__ import annotations

import json
import multiprocessing as mp
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def run_box(b: int):
    import bench
    from oracle import oracle_py
    ini = bench.ensemble_inis(512)[b]
    t = time.perf_counter()
    box = oracle_py.OracleBox(ini)
    st, _ = box.calcul()
    dt = time.perf_counter() - t
    box.close()
    return b, bench.ini_monomers(ini), int(st.steps), int(st.n_aggregates), dt


def main() -> int:
    import bench
    procs = int(sys.argv[1]) if len(sys.argv) > 1 else (mp.cpu_count() or 1)
    inis = bench.ensemble_inis(512)
    boxes = sorted(range(0, 512, 16), key=lambda b: -bench.ini_monomers(inis[b]))
    with mp.get_context("spawn").Pool(procs) as pool:
        for r in pool.imap_unordered(run_box, boxes):
            print(json.dumps(r), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
