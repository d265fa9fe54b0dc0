"""Generates tests/golden/ensemble64.npz from the reference itself.

Runs the reference's own ``mcac::calcul`` (built from the reference sources
by oracle/ref.mk into oracle/_ref/mcac_ref_harness, mode ``calcul``) on 64
boxes of the 512-box benchmark ensemble (boxes 0, 8, 16, ..., 504: sizes
from a few hundred to ~16 000 monomers, monodisperse and LogNormal(1.25),
100-5000 ppm, 1500-1900 K) from their seeded placements until at most 20
aggregates are left (or 10 000 steps pass without an event), and stores per
box the physical time reached and the aggregate count, and per aggregate its
monomer count, Rg/dp and box. tests/test_ensemble_gpu.py runs the same boxes
with the device loop and compares the distributions.

Needs the reference sources (MCAC_REFERENCE names their directory) and a C++
compiler; run from the repository root (about half an hour on 8 cores):

    python tests/golden/make_ensemble_golden.py
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402
from mcac_gb300 import build  # noqa: E402
from mcac_gb300.snapshot import A, Snapshot  # noqa: E402

OUT = Path(__file__).resolve().parent
HARNESS = ROOT / "oracle" / "_ref" / "mcac_ref_harness"
BOXES = list(range(0, 512, 8))
STOP_AGGREGATES = 20


def box_ini(b: int) -> str:
    ini = bench.ensemble_inis(512)[b]
    return ini.replace("number_of_aggregates = 1\n", f"number_of_aggregates = {STOP_AGGREGATES}\n")


def run_box(b: int, work: Path):
    d = work / f"b{b}"
    d.mkdir()
    (d / "box.ini").write_text(box_ini(b) + "[output]\noutput_dir = out\n")
    t0 = time.perf_counter()
    subprocess.run([str(HARNESS), "calcul", "box.ini", "ref"], cwd=d, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    snap = Snapshot.load(d / "ref_final.snap")
    return b, snap.time, snap.na, snap.n_spheres.copy(), snap.aggregates[A["dg_over_dp"]].copy(), \
        time.perf_counter() - t0


def main() -> int:
    build.build_reference(build.reference_dir())
    res = {}
    with tempfile.TemporaryDirectory(dir=ROOT) as tmp:
        work = Path(tmp)
        sizes = {b: bench.ini_monomers(bench.ensemble_inis(512)[b]) for b in BOXES}
        order = sorted(BOXES, key=lambda b: -sizes[b])  # largest first
        with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
            for b, t, na, npp, dgdp, wall in ex.map(lambda k: run_box(k, work), order):
                res[b] = (t, na, npp, dgdp)
                print(f"box {b} ({sizes[b]} monomers): {na} aggregates at t = {t:.4g} s, {wall:.0f} s", flush=True)
    boxes = np.array(BOXES, dtype=np.int64)
    npp = np.concatenate([res[b][2] for b in BOXES]).astype(np.int64)
    dgdp = np.concatenate([res[b][3] for b in BOXES])
    box_of = np.concatenate([np.full(len(res[b][2]), b) for b in BOXES]).astype(np.int64)
    np.savez_compressed(OUT / "ensemble64.npz", boxes=boxes, stop_aggregates=np.array(STOP_AGGREGATES),
                        time=np.array([res[b][0] for b in BOXES]),
                        n_aggregates=np.array([res[b][1] for b in BOXES], dtype=np.int64),
                        npp=npp, dg_over_dp=dgdp, box=box_of)
    print(f"ensemble64.npz: {len(BOXES)} boxes, {len(npp)} aggregates")
    return 0


if __name__ == "__main__":
    sys.exit(main())
