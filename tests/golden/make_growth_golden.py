"""Generates tests/golden/growth_{ensemble,individual}.npz from the reference itself.

Surface growth (``[surface_growth] with_surface_reactions``) runs in the
reference's own ``mcac::calcul`` (src/calcul.cpp:157-206: every sphere grows
by u_sg dt each step, every aggregate is updated). This script runs that
code, built from the reference sources by oracle/ref.mk
(oracle/_ref/mcac_ref_harness, mode ``calcul``), on 32 seeded boxes of 300
LogNormal(30 nm, 1.25) monomers at 5000 ppm with flux_surfgrowth = 0.5
kg/m^2/s (spheres grow by about 2 nm before 15 aggregates are left) and
stores, per box, the final physical time, the mean sphere radius and the
(monomers, Rg/dp) pairs of the final aggregates. The device loop is compared
with these distributions (tests/test_growth_gpu.py).

Needs the reference sources (MCAC_REFERENCE names their directory) and a C++
compiler; run from the repository root:

    python tests/golden/make_growth_golden.py [growth_ensemble.npz] [growth_individual.npz]
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from mcac_gb300 import build  # noqa: E402
from mcac_gb300.snapshot import A, S, Snapshot  # noqa: E402

OUT = Path(__file__).resolve().parent
HARNESS = ROOT / "oracle" / "_ref" / "mcac_ref_harness"
N_BOXES = 32


def growth_ini(seed: int, individual: bool = False) -> str:
    return (f"[monomers]\nnumber = 300\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 5e-3\ntemperature = 1700\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = 0.5\n"
            f"[limits]\nnumber_of_aggregates = 15\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n"
            + ("individual_surf_reactions = true\n" if individual else "")
            + "[output]\noutput_dir = out\n")


def run_set(individual: bool, name: str) -> None:
    times, mean_r, npp, dgdp, box_of = [], [], [], [], []
    with tempfile.TemporaryDirectory(dir=ROOT) as tmp:
        work = Path(tmp)
        for b in range(N_BOXES):
            ini = work / f"g{b}.ini"
            ini.write_text(growth_ini(600 + b, individual))
            subprocess.run([str(HARNESS), "calcul", ini.name, f"g{b}"], cwd=work, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            snap = Snapshot.load(work / f"g{b}_final.snap")
            times.append(snap.time)
            mean_r.append(float(snap.spheres[S["r"]].mean()))
            npp.extend(snap.n_spheres.tolist())
            dgdp.extend(snap.aggregates[A["dg_over_dp"]].tolist())
            box_of.extend([b] * snap.na)
    np.savez_compressed(OUT / name, ini=np.array(growth_ini(0, individual)), seeds=np.arange(600, 600 + N_BOXES),
                        time=np.array(times), mean_r=np.array(mean_r), npp=np.array(npp, dtype=np.int64),
                        dg_over_dp=np.array(dgdp), box=np.array(box_of, dtype=np.int64))
    print(f"{name}: {N_BOXES} boxes: mean time {np.mean(times):.4g} s, mean radius {np.mean(mean_r):.4g} m")


def main() -> int:
    build.build_reference(build.reference_dir())
    sets = {"growth_ensemble.npz": False, "growth_individual.npz": True}
    for name, individual in sets.items():
        if len(sys.argv) > 1 and name not in sys.argv[1:]:
            continue
        run_set(individual, name)
    return 0


if __name__ == "__main__":
    sys.exit(main())
