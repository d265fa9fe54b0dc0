"""Generates tests/golden/growth_exact.npz from the reference itself.

Three seeded runs of the reference's own ``mcac::calcul`` with surface growth
(src/calcul.cpp:157-206), built from its sources by oracle/ref.mk
(oracle/_ref/mcac_ref_harness, mode ``calcul``): 200 LogNormal(30 nm, 1.25)
monomers at 5000 ppm, flux_surfgrowth = 0.5 kg/m^2/s, to 20 aggregates,
with the growth of every aggregate at every step ("collective"), of the moved
aggregate only ("individual"), and with update_partial on two steps out of
three ("partial", full_aggregate_update_frequency = 3). For each: the INI,
the final physical time, the number of aggregates and the digest of the
final state. tests/test_oracle.py checks the oracle against them; the
host-driven loop is checked against the oracle (tests/test_growth_exact_gpu.py).

Needs the reference sources (MCAC_REFERENCE names their directory) and a C++
compiler; run from the repository root:

    python tests/golden/make_growth_exact_golden.py
"""
from __future__ import annotations

import hashlib
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
CASES = {"collective": dict(seed=650), "individual": dict(seed=651, individual=True),
         "partial": dict(seed=652, every=3)}


def growth_ini(seed: int, individual: bool = False, every: int = 1) -> str:
    return (f"[monomers]\nnumber = 200\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 5e-3\ntemperature = 1700\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = 0.5\n"
            f"full_aggregate_update_frequency = {every}\n[limits]\nnumber_of_aggregates = 20\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n"
            + ("individual_surf_reactions = true\n" if individual else "") + "[output]\noutput_dir = out\n")


def digest(snap) -> str:
    h = hashlib.sha256()
    for arr in (snap.spheres, snap.sphere_label, snap.aggregates, snap.n_spheres, snap.members):
        h.update(np.ascontiguousarray(arr).tobytes())
    h.update(np.array([snap.maxradius, snap.box_length], dtype=np.float64).tobytes())
    return h.hexdigest()


def main() -> int:
    build.build_reference(build.reference_dir())
    out: dict[str, np.ndarray] = {"cases": np.array(list(CASES))}
    with tempfile.TemporaryDirectory(dir=ROOT) as tmp:
        work = Path(tmp)
        for name, kw in CASES.items():
            text = growth_ini(**kw)
            (work / "g.ini").write_text(text)
            subprocess.run([str(HARNESS), "calcul", "g.ini", "g"], cwd=work, check=True, stdout=subprocess.DEVNULL,
                           stderr=subprocess.DEVNULL)
            snap = Snapshot.load(work / "g_final.snap")
            out[f"{name}_ini"] = np.array(text)
            out[f"{name}_time"] = np.array(snap.time)
            out[f"{name}_na"] = np.array(snap.na)
            out[f"{name}_digest"] = np.array(digest(snap))
            print(name, snap.na, snap.time)
    np.savez_compressed(OUT / "growth_exact.npz", **out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
