"""Generates tests/golden/oxidation.npz from the reference itself.

Oxidation (``[surface_growth] flux_surfgrowth < 0``) runs in the reference's
own ``mcac::calcul``: every sphere shrinks by |u_sg| dt a step, spheres at or
below ``[oxidation] rp_min`` leave their aggregate, aggregates left empty
disappear and aggregates whose spheres no longer touch split
(src/calcul.cpp:157-170, src/aggregats/aggregat.cpp:230-243, 545-655).

This script runs that code, built from the reference sources by
oracle/ref.mk (oracle/_ref/mcac_ref_harness):

1. four seeded boxes of 300 LogNormal(30 nm, 1.25) monomers at 5000 ppm grow
   (flux_surfgrowth = 0.5 kg/m^2/s, mode ``calcul``) until 15 aggregates of
   overlapping spheres are left; these states are stored (start_<k>_*);
2. from each, mode ``calcul_from`` runs oxidation at flux -0.5 kg/m^2/s
   until a physical time 3 us later (default rp_min), and 6 us later with
   rp_min = 13 nm (spheres removed as well), both with the shrink applied to
   every aggregate at every step: the number of spheres left and the sizes of
   the aggregates they form are stored (coll_<case>_<k>_*);
3. the same 6 us / 13 nm case with the shrink of the moved aggregate only
   (individual_surf_reactions), 8 seeds from each start: the numbers of
   aggregates and spheres left are stored (ind_*);
4. for the step-exact check of the oracle, from each start the 6 us / 13 nm
   case both ways with the seed 900 + k: the final state's digest, the
   numbers of aggregates and spheres and the physical time (exact_*). The
   harness places one monomer before it loads the state, which draws four
   values from the seeded stream first.

The device loop is compared with these runs in tests/test_oxidation_gpu.py.

Needs the reference sources (MCAC_REFERENCE names their directory) and a C++
compiler; run from the repository root:

    python tests/golden/make_oxidation_golden.py
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
from mcac_gb300.snapshot import Snapshot  # noqa: E402

OUT = Path(__file__).resolve().parent
HARNESS = ROOT / "oracle" / "_ref" / "mcac_ref_harness"
START_SEEDS = (700, 701, 702, 703)
FLUX = -0.5
# (name, physical time after the start, rp_min)
COLLECTIVE = (("a", 3e-6, 1.66e-10), ("b", 6e-6, 1.3e-8))
INDIVIDUAL = (6e-6, 1.3e-8)
IND_SEEDS = 8


def grow_ini(seed: int) -> str:
    return (f"[monomers]\nnumber = 300\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 5e-3\ntemperature = 1700\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = 0.5\n"
            f"[limits]\nnumber_of_aggregates = 15\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n[output]\noutput_dir = out\n")


def oxidation_ini(seed: int, time_limit: float, rp_min: float, individual: bool) -> str:
    """The oxidation phase's parameters (the box length comes from the state)."""
    return (f"[monomers]\nnumber = 300\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 5e-3\ntemperature = 1700\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = {FLUX!r}\n"
            f"[oxidation]\nrp_min = {rp_min!r}\n"
            f"[limits]\nnumber_of_aggregates = 0\nphysical_time = {time_limit!r}\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n"
            + ("individual_surf_reactions = true\n" if individual else "") + "[output]\noutput_dir = out\n")


def digest(snap) -> str:
    import hashlib
    h = hashlib.sha256()
    for arr in (snap.spheres, snap.sphere_label, snap.aggregates, snap.n_spheres, snap.members):
        h.update(np.ascontiguousarray(arr).tobytes())
    h.update(np.array([snap.maxradius, snap.box_length], dtype=np.float64).tobytes())
    return h.hexdigest()


def run(args: list[str], cwd: Path) -> None:
    subprocess.run([str(HARNESS)] + args, cwd=cwd, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)


def main() -> int:
    build.build_reference(build.reference_dir())
    out: dict[str, np.ndarray] = {"start_seeds": np.array(START_SEEDS), "flux": np.array(FLUX),
                                  "coll_cases": np.array([c[0] for c in COLLECTIVE]),
                                  "coll_dt": np.array([c[1] for c in COLLECTIVE]),
                                  "coll_rp_min": np.array([c[2] for c in COLLECTIVE]),
                                  "ind_dt": np.array(INDIVIDUAL[0]), "ind_rp_min": np.array(INDIVIDUAL[1]),
                                  "ind_seeds": np.array(IND_SEEDS)}
    ind_na, ind_ns = [], []
    with tempfile.TemporaryDirectory(dir=ROOT) as tmp:
        work = Path(tmp)
        for k, seed in enumerate(START_SEEDS):
            (work / "g.ini").write_text(grow_ini(seed))
            run(["calcul", "g.ini", "g"], work)
            start = Snapshot.load(work / "g_final.snap")
            out.update(start.to_npz_dict(f"start_{k}_"))
            for name, dt, rp_min in COLLECTIVE:
                (work / "o.ini").write_text(oxidation_ini(seed + 100, start.time + dt, rp_min, False))
                run(["calcul_from", "o.ini", "g_final.snap", "o"], work)
                end = Snapshot.load(work / "o_final.snap")
                out[f"coll_{name}_{k}_sizes"] = np.sort(end.n_spheres)[::-1].copy()
                out[f"coll_{name}_{k}_ns"] = np.array(end.ns)
                out[f"coll_{name}_{k}_time"] = np.array(end.time)
            for mode, individual in (("coll", False), ("ind", True)):
                (work / "x.ini").write_text(oxidation_ini(900 + k, start.time + INDIVIDUAL[0], INDIVIDUAL[1],
                                                          individual))
                run(["calcul_from", "x.ini", "g_final.snap", "x"], work)
                end = Snapshot.load(work / "x_final.snap")
                out[f"exact_{mode}_{k}_digest"] = np.array(digest(end))
                out[f"exact_{mode}_{k}_na"] = np.array(end.na)
                out[f"exact_{mode}_{k}_ns"] = np.array(end.ns)
                out[f"exact_{mode}_{k}_time"] = np.array(end.time)
            for j in range(IND_SEEDS):
                (work / "i.ini").write_text(oxidation_ini(seed + 200 + j, start.time + INDIVIDUAL[0], INDIVIDUAL[1],
                                                          True))
                run(["calcul_from", "i.ini", "g_final.snap", "i"], work)
                end = Snapshot.load(work / "i_final.snap")
                ind_na.append(end.na)
                ind_ns.append(end.ns)
    out["ind_na"] = np.array(ind_na)
    out["ind_ns"] = np.array(ind_ns)
    np.savez_compressed(OUT / "oxidation.npz", **out)
    for name, _, _ in COLLECTIVE:
        print(name, [len(out[f"coll_{name}_{k}_sizes"]) for k in range(len(START_SEEDS))],
              [int(out[f"coll_{name}_{k}_ns"]) for k in range(len(START_SEEDS))])
    print("individual: aggregates", np.mean(ind_na), "spheres", np.mean(ind_ns))
    return 0


if __name__ == "__main__":
    sys.exit(main())
