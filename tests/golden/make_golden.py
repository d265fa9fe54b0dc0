"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs the reference MCAC built from its own sources (oracle/ref.mk ->
oracle/_ref/mcac_ref_harness) on seeded configurations and stores, as
compressed .npz files:

* c1_trace.npz   -- configuration 1 of the benchmark set (N=1000,
                    Normal(30, 1.25) nm, 1000 ppm, seed 0, stop at 10
                    aggregates): initial state, one row per MC step (picked
                    label, contact, merge, contact spheres/aggregate,
                    distance, time) and every merged aggregate record.
* c1_q5000.npz   -- the state before step 5000 of that run, 2000 seeded
                    distance_to_next_contact queries with the reference's
                    answers, and the merged records of the contacts.
* ln_late.npz    -- a LogNormal(30 nm, 1.5) box of 3000 monomers at
                    5000 ppm (seed 11) run down to 30 aggregates: the state
                    when 60 aggregates are left, 2000 queries, merges, and
                    the final-state digest of the whole run.
* meta.npz       -- PhysicalModel-derived values (box length, gas
                    properties) for the reference's validation parameter
                    files and for the configurations above.

Needs the reference sources (MCAC_REFERENCE names their directory) and
a C++ compiler; run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from mcac_gb300 import build  # noqa: E402
from mcac_gb300.snapshot import QUERY_DTYPE, STEP_DTYPE, Snapshot, read_merge_records  # noqa: E402

OUT = Path(__file__).resolve().parent
HARNESS = ROOT / "oracle" / "_ref" / "mcac_ref_harness"

C1_INI = """[monomers]
number = 1000
density = 1800
mean_diameter = 30
dispersion_diameter = 1.25
initialisation_mode = normal

[environment]
volume_fraction = 1e-3
temperature = 1700
pressure = 101300
fractal_prefactor = 1.4
fractal_dimension = 1.8

[limits]
number_of_aggregates = 10

[numerics]
random_seed = 0
with_domain_duplication = false

[output]
output_dir = out
"""

LN_INI = """[monomers]
number = 3000
density = 1800
mean_diameter = 30
dispersion_diameter = 1.5
initialisation_mode = lognormal

[environment]
volume_fraction = 5e-3
temperature = 1600
pressure = 101300
fractal_prefactor = 1.4
fractal_dimension = 1.8

[limits]
number_of_aggregates = 30

[numerics]
random_seed = 11
with_domain_duplication = false

[output]
output_dir = out
"""


def run(args, cwd):
    subprocess.run([str(HARNESS)] + [str(a) for a in args], cwd=cwd, check=True, stdin=subprocess.DEVNULL,
                   stdout=subprocess.PIPE, timeout=3600)


def state_digest(snap: Snapshot) -> str:
    h = hashlib.sha256()
    for arr in (snap.spheres, snap.sphere_label, snap.aggregates, snap.n_spheres, snap.members):
        h.update(np.ascontiguousarray(arr).tobytes())
    h.update(np.array([snap.maxradius, snap.box_length], dtype=np.float64).tobytes())
    return h.hexdigest()


def compact_trace(tr: np.ndarray) -> dict:
    return {
        "t_picked": tr["picked"].astype(np.int32),
        "t_contact": tr["contact"].astype(np.int8),
        "t_merged": tr["merged"].astype(np.int8),
        "t_moving_sphere": tr["moving_sphere"].astype(np.int32),
        "t_other_sphere": tr["other_sphere"].astype(np.int32),
        "t_other_agg": tr["other_agg"].astype(np.int32),
        "t_contact_distance": tr["contact_distance"],
        "t_time_after": tr["time_after"],
    }


def merges_dict(path: Path, prefix: str, with_spheres: bool) -> dict:
    recs = read_merge_records(path, with_spheres)
    out = {
        prefix + "index": np.array([r["index"] for r in recs], dtype=np.int64),
        prefix + "merged": np.array([r["merged"] for r in recs], dtype=np.int8),
        prefix + "keep": np.array([r["keep"] for r in recs], dtype=np.int64),
        prefix + "n": np.array([r["n"] for r in recs], dtype=np.int64),
        prefix + "record": np.array([r["record"] for r in recs]).reshape(-1, 21),
        prefix + "maxradius": np.array([r["maxradius"] for r in recs]),
    }
    if with_spheres:
        out[prefix + "sphere_ids"] = np.concatenate([r["sphere_ids"] for r in recs]) if recs else np.zeros(0, np.int64)
        out[prefix + "sphere_rows"] = (np.concatenate([r["sphere_rows"] for r in recs])
                                       if recs else np.zeros((0, 9)))
    return out


def queries_dict(path: Path) -> dict:
    q = np.fromfile(path, dtype=QUERY_DTYPE)
    return {"q_label": q["label"], "q_dir": q["dir"], "q_distance": q["distance"],
            "q_contact_distance": q["contact_distance"], "q_contact": q["contact"].astype(np.int8),
            "q_moving_sphere": q["moving_sphere"], "q_other_sphere": q["other_sphere"],
            "q_other_agg": q["other_agg"]}


def parse_meta(text: str) -> dict:
    out = {}
    for line in text.splitlines():
        k, v = line.split()
        out[k] = float(v)
    return out


def main() -> int:
    ref = build.build_reference(build.reference_dir(), verbose=True)
    if ref is None or not HARNESS.exists():
        print("reference sources not found; nothing generated", file=sys.stderr)
        return 1
    work = Path(tempfile.mkdtemp(prefix="mcac_golden_"))
    try:
        # ---- configuration 1: full trace
        (work / "c1.ini").write_text(C1_INI)
        run(["trace", "c1.ini", "c1", 5000], work)
        tr = np.fromfile(work / "c1_trace.bin", dtype=STEP_DTYPE)
        init = Snapshot.load(work / "c1_init.snap")
        final = Snapshot.load(work / "c1_final.snap")
        data = {}
        data.update(init.to_npz_dict("init_"))
        data.update(compact_trace(tr))
        data.update(merges_dict(work / "c1_merges.bin", "m_", False))
        data["final_digest"] = np.array(state_digest(final))
        data["final_time"] = np.array(final.time)
        data["final_n_agg"] = np.array(final.na)
        data["ini"] = np.array(C1_INI)
        np.savez_compressed(OUT / "c1_trace.npz", **data)
        # ---- queries and merges on the state before step 5000
        run(["queries", "c1.ini", "c1_step5000.snap", 2000, 7, "c1_q.bin"], work)
        run(["merges", "c1.ini", "c1_step5000.snap", "c1_q.bin", "c1_m.bin"], work)
        snap = Snapshot.load(work / "c1_step5000.snap")
        data = snap.to_npz_dict("s_")
        data.update(queries_dict(work / "c1_q.bin"))
        data.update(merges_dict(work / "c1_m.bin", "m_", True))
        data["ini"] = np.array(C1_INI)
        np.savez_compressed(OUT / "c1_q5000.npz", **data)

        # ---- lognormal box down to 30 aggregates; state at 60 aggregates
        (work / "ln.ini").write_text(LN_INI)
        run(["trace", "ln.ini", "ln0"], work)
        tr = np.fromfile(work / "ln0_trace.bin", dtype=STEP_DTYPE)
        final = Snapshot.load(work / "ln0_final.snap")
        step60 = int(np.argmax(tr["n_agg_after"] <= 60)) + 1
        run(["trace", "ln.ini", "ln", step60], work)
        run(["queries", "ln.ini", f"ln_step{step60}.snap", 2000, 13, "ln_q.bin"], work)
        run(["merges", "ln.ini", f"ln_step{step60}.snap", "ln_q.bin", "ln_m.bin"], work)
        snap = Snapshot.load(work / f"ln_step{step60}.snap")
        data = snap.to_npz_dict("s_")
        data.update(queries_dict(work / "ln_q.bin"))
        data.update(merges_dict(work / "ln_m.bin", "m_", True))
        data["ini"] = np.array(LN_INI)
        data["snap_step"] = np.array(step60)
        data["run_steps"] = np.array(len(tr))
        data["run_events"] = np.array(int(tr["merged"].sum()))
        data["final_digest"] = np.array(state_digest(final))
        data["final_time"] = np.array(final.time)
        data["merge_steps"] = np.flatnonzero(tr["merged"]).astype(np.int64)
        np.savez_compressed(OUT / "ln_late.npz", **data)

        # ---- PhysicalModel-derived values
        meta = {}
        refdir = build.reference_dir()
        inis = {p.stem: p.read_text() for p in sorted((refdir / "validation").glob("params_*.ini"))}
        # examples/classic.ini is left out: it enables interaction potentials
        # with an external table, a path this library does not cover.
        inis["c1"] = C1_INI
        inis["ln"] = LN_INI
        for name, text in inis.items():
            d = work / f"meta_{name}"
            d.mkdir()
            # the reference creates its output directory; keep it inside the scratch dir
            run_text = "\n".join("output_dir = out" if line.strip().startswith("output_dir") else line
                                  for line in text.splitlines()) + "\n"
            (d / "p.ini").write_text(run_text)
            out = subprocess.run([str(HARNESS), "meta", "p.ini"], cwd=d, check=True, stdin=subprocess.DEVNULL,
                                 capture_output=True, text=True, timeout=600).stdout
            vals = parse_meta("\n".join(line for line in out.splitlines() if line and line[0].isalpha()
                                        and len(line.split()) == 2))
            meta[f"{name}__keys"] = np.array(sorted(vals))
            meta[f"{name}__values"] = np.array([vals[k] for k in sorted(vals)])
            meta[f"{name}__ini"] = np.array(text)
        np.savez_compressed(OUT / "meta.npz", **meta)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    for p in sorted(OUT.glob("*.npz")):
        print(f"{p.name}: {p.stat().st_size} bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
