"""advancement.dat: the reference's time-resolved output, byte for byte.

The reference's calcul appends the physical model's values (time,
aggregate and monomer concentrations, volume fraction, mean monomers per
aggregate, temperature, box volume, u_sg, nucleation flux) whenever
PhysicalModel::time_to_write says so, and once at the end
(src/calcul.cpp:29-43, 67-70, 282; physical_model.cpp:338-356). The host-driven
loop writes the same lines: compared with the files the reference binary
itself wrote on three seeded configurations (tests/golden/advancement_*,
made by tests/golden/make_advancement_golden.py), including non-default
write_events_frequency, write_between_event_frequency and write_Delta_t.
"""
from pathlib import Path

import pytest

from mcac_gb300 import AggregatList, PhysicalModel

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c1", "freq", "dt"])
def test_advancement_file_matches_reference(case, tmp_path):
    model = PhysicalModel(text=(GOLDEN / f"advancement_{case}.ini").read_text())
    out = tmp_path / "advancement.dat"
    with AggregatList(model) as box:
        # in pieces: the write rule carries across calls
        stats, _ = box.calcul(max_steps=5000, advancement=out)
        while not stats.finished:
            stats, _ = box.calcul(max_steps=5000, advancement=out)
        box.calcul(max_steps=10, advancement=out)  # a finished run adds nothing
    ref = (GOLDEN / f"advancement_{case}.dat").read_bytes()
    got = out.read_bytes()
    assert got.count(b"\n") == ref.count(b"\n")
    assert got == ref
