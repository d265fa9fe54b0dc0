"""Generates tests/golden/volsurf_{alphas,caps}.npz from the reference itself.

With surface growth the spheres of an aggregate overlap, and the aggregate's
volume and surface follow ``volsurf_method`` (src/aggregats/aggregat.cpp:
321-430): "alphas" corrects the sums by the coordination and overlap
statistics, "caps" takes the spherical caps of every contact off each
sphere. This script runs the reference's own ``mcac::calcul`` (built from
its sources by oracle/ref.mk into oracle/_ref/mcac_ref_harness) on the
reference's surface-growth validation case (validation/params_surface_growth.ini:
800 LogNormal(10 nm, 1.2) monomers at 10 ppm, flux 1e-4, full update every
100 steps, stop at 40 monomers per aggregate) with 32 seeds per method and
stores, per box, the final physical time and mean sphere radius, and per
final aggregate its monomer count, Rg/dp, and its volume and surface over
the plain sums of its spheres' (the corrections' effect). The device loop is
compared with these distributions (tests/test_volsurf_gpu.py).

Needs the reference sources (MCAC_REFERENCE names their directory) and a C++
compiler; run from the repository root:

    python tests/golden/make_volsurf_golden.py
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from mcac_gb300 import build  # noqa: E402
from mcac_gb300.snapshot import A, S, Snapshot  # noqa: E402

OUT = Path(__file__).resolve().parent
HARNESS = ROOT / "oracle" / "_ref" / "mcac_ref_harness"
N_BOXES = 32
SEED0 = 700


def volsurf_ini(method: str, seed: int) -> str:
    return (f"[environment]\ninitial_time = 0\nfractal_dimension = 1.78\nfractal_prefactor = 1.30\n"
            f"pressure = 101300\ntemperature = 1700\nvolume_fraction = 10e-6\n"
            f"[limits]\nmean_monomere_per_aggregate = 40\n"
            f"[monomers]\ndensity = 1800\ndispersion_diameter = 1.20\ninitialisation_mode = lognormal\n"
            f"mean_diameter = 10\nnumber = 800\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = 1e-04\n"
            f"volsurf_method = {method}\nfull_aggregate_update_frequency = 100\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n[output]\noutput_dir = out\n")


def box_stats(snap: Snapshot):
    off = snap.member_offsets()
    vol_ratio, surf_ratio = [], []
    for a in range(snap.na):
        mem = snap.members[off[a]:off[a + 1]]
        vol_ratio.append(snap.aggregates[A["volume"], a] / snap.spheres[S["volume"], mem].sum())
        surf_ratio.append(snap.aggregates[A["surface"], a] / snap.spheres[S["surface"], mem].sum())
    return vol_ratio, surf_ratio


def main() -> int:
    build.build_reference(build.reference_dir())
    for method in ("alphas", "caps"):
        with tempfile.TemporaryDirectory(dir=ROOT) as tmp:
            work = Path(tmp)

            def one(b):
                d = work / f"b{b}"
                d.mkdir()
                (d / "run.ini").write_text(volsurf_ini(method, SEED0 + b))
                subprocess.run([str(HARNESS), "calcul", "run.ini", "g"], cwd=d, check=True,
                               stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
                return Snapshot.load(d / "g_final.snap")

            with ThreadPoolExecutor(max_workers=8) as ex:
                snaps = list(ex.map(one, range(N_BOXES)))
        times, mean_r, npp, dgdp, vr, sr, box_of = [], [], [], [], [], [], []
        for b, snap in enumerate(snaps):
            times.append(snap.time)
            mean_r.append(float(snap.spheres[S["r"]].mean()))
            npp.extend(snap.n_spheres.tolist())
            dgdp.extend(snap.aggregates[A["dg_over_dp"]].tolist())
            v, s = box_stats(snap)
            vr.extend(v)
            sr.extend(s)
            box_of.extend([b] * snap.na)
        np.savez_compressed(OUT / f"volsurf_{method}.npz", ini=np.array(volsurf_ini(method, 0)),
                            seeds=np.arange(SEED0, SEED0 + N_BOXES), time=np.array(times), mean_r=np.array(mean_r),
                            npp=np.array(npp, dtype=np.int64), dg_over_dp=np.array(dgdp),
                            vol_ratio=np.array(vr), surf_ratio=np.array(sr), box=np.array(box_of, dtype=np.int64))
        print(f"{method}: mean time {np.mean(times):.4g} s, mean radius {np.mean(mean_r):.4g} m, "
              f"volume ratio {np.mean(vr):.4f}, surface ratio {np.mean(sr):.4f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
