"""Generates tests/golden/advancement_*.dat: the reference's own advancement.dat.

The reference's ``mcac::calcul`` appends one line of the physical model's
time-resolved values to ``<output_dir>/advancement.dat`` whenever
``PhysicalModel::time_to_write`` says so and once at the end
(src/calcul.cpp:29-43, 67-70, 282; src/physical_model/physical_model.cpp:338-356).
This script runs the reference binary built from its sources by oracle/ref.mk
(oracle/_ref/MCAC) on three seeded configurations — configuration 1 with the
default write rule, and two others with non-default write_events_frequency,
write_between_event_frequency and write_Delta_t — and stores those files with
the parameter files that made them (advancement_<case>.ini).
tests/test_advancement_gpu.py compares the host-driven loop's file with them
byte for byte.

Needs the reference sources (MCAC_REFERENCE names their directory) and a C++
compiler; run from the repository root:

    python tests/golden/make_advancement_golden.py
"""
from __future__ import annotations

import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from mcac_gb300 import build  # noqa: E402

OUT = Path(__file__).resolve().parent
MCAC = ROOT / "oracle" / "_ref" / "MCAC"

BASE = """[monomers]
number = {n}
density = 1800
mean_diameter = 30
dispersion_diameter = {disp}
initialisation_mode = {mode}

[environment]
volume_fraction = {fv}
temperature = 1700
pressure = 101300
fractal_prefactor = 1.4
fractal_dimension = 1.8

[limits]
number_of_aggregates = {nagg}

[numerics]
random_seed = {seed}
with_domain_duplication = false

[output]
output_dir = out
{extra}"""

CASES = {
    "c1": dict(n=1000, disp=1.25, mode="normal", fv=1e-3, nagg=10, seed=0, extra=""),
    "freq": dict(n=600, disp=1.3, mode="lognormal", fv=3e-3, nagg=20, seed=5,
                 extra="write_events_frequency = 3\nwrite_between_event_frequency = 37\n"),
    "dt": dict(n=500, disp=1.25, mode="normal", fv=2e-3, nagg=15, seed=9,
               extra="write_events_frequency = 1000000\nwrite_between_event_frequency = 1000000\n"
                     "write_Delta_t = 2e-6\n"),
}


def ini_text(name: str) -> str:
    return BASE.format(**CASES[name])


def main() -> int:
    build.build_reference(build.reference_dir())
    with tempfile.TemporaryDirectory(dir=ROOT) as tmp:
        for name in CASES:
            work = Path(tmp) / name
            work.mkdir()
            (work / "run.ini").write_text(ini_text(name))
            subprocess.run([str(MCAC), "run.ini"], cwd=work, check=True, stdin=subprocess.DEVNULL,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            shutil.copyfile(work / "out" / "advancement.dat", OUT / f"advancement_{name}.dat")
            (OUT / f"advancement_{name}.ini").write_text(ini_text(name))
            lines = (OUT / f"advancement_{name}.dat").read_text().count("\n")
            print(f"{name}: {lines} lines")
    return 0


if __name__ == "__main__":
    sys.exit(main())
