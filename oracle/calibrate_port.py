"""Times the reference and the oracle's C restatement on the same runs.

The CPU baseline of bench.py is the restatement (oracle/mcac_oracle.c),
because the reference sources are not present where the benchmark runs.
This script measures how fast the restatement is against the reference
itself (oracle/_ref/mcac_ref_harness, mode ``calcul``: the reference's own
``mcac::calcul`` built from its sources by oracle/ref.mk), one core each, on
runs that are identical step for step on both sides (seeded boxes of the
benchmark configurations run to a stop criterion). It checks that both end
in the same state (aggregate count and physical time, bit for bit) and
prints one JSON line per run with both wall times (placement included on
both sides) and their ratio.

Needs the reference build (python -c "import __graft_entry__ as g; g.build()"
where the reference sources are mounted); run from the repository root:

    python oracle/calibrate_port.py
"""
from __future__ import annotations

import json
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
from oracle import oracle_py  # noqa: E402

HARNESS = ROOT / "oracle" / "_ref" / "mcac_ref_harness"


def c2_ini(n_agg: int) -> str:
    return ("[monomers]\nnumber = 100000\ndensity = 1800\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 1e-3\ntemperature = 1700\n"
            "pressure = 101300\nfractal_prefactor = 1.4\nfractal_dimension = 1.8\n"
            f"[limits]\nnumber_of_aggregates = {n_agg}\n[numerics]\nrandom_seed = 1\n"
            "with_domain_duplication = false\n")


def runs() -> list[tuple[str, str]]:
    import bench
    inis = bench.ensemble_inis(512)
    sizes = [bench.ini_monomers(t) for t in inis]
    out = []
    for target in (1000, 4000, 8000, 16000):
        b = min(range(len(inis)), key=lambda k: abs(sizes[k] - target))
        out.append((f"ensemble box {b} ({sizes[b]} monomers) to 100 aggregates (window a)",
                    inis[b].replace("number_of_aggregates = 1", "number_of_aggregates = 100")))
    for target in (1000, 4000):
        b = min(range(len(inis)), key=lambda k: abs(sizes[k] - target))
        out.append((f"ensemble box {b} ({sizes[b]} monomers) to 20 aggregates",
                    inis[b].replace("number_of_aggregates = 1", "number_of_aggregates = 20")))
    out.append(("C2 100k-monomer box to 99000 aggregates (placement dominates)", c2_ini(99000)))
    return out


def main() -> int:
    if not HARNESS.exists():
        print("reference build not found (oracle/_ref); nothing measured", file=sys.stderr)
        return 1
    for name, ini in runs():
        with tempfile.TemporaryDirectory() as tmp:
            work = Path(tmp)
            (work / "box.ini").write_text(ini + "[output]\noutput_dir = out\n")
            t0 = time.perf_counter()
            proc = subprocess.run([str(HARNESS), "calcul", "box.ini", "ref"], cwd=work, check=True,
                                  capture_output=True, text=True)
            t_ref = time.perf_counter() - t0
            words = next(line for line in proc.stdout.splitlines() if line.startswith("n_agg ")).split()
            ref_agg, ref_time = int(words[1]), float(words[3])
            t0 = time.perf_counter()
            box = oracle_py.OracleBox(ini)
            t_place = time.perf_counter() - t0
            st, _ = box.calcul()
            t_port = time.perf_counter() - t0
            same = ref_agg == int(st.n_aggregates) and np.float64(ref_time) == np.float64(st.time)
            box.close()
        print(json.dumps({"run": name, "reference_s": round(t_ref, 3), "port_s": round(t_port, 3),
                          "port_placement_s": round(t_place, 3), "steps": int(st.steps),
                          "reference_steps_per_s": round(st.steps / t_ref, 1),
                          "port_steps_per_s": round(st.steps / t_port, 1),
                          "port_over_reference": round(t_ref / t_port, 3), "same_final_state": bool(same)}),
              flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
