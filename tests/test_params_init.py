"""Parameter-file semantics and the initial placement, against the reference.

The golden values come from the reference compiled from its own sources
(tests/golden/make_golden.py); these tests need no GPU.
"""
import math

import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import PhysicalModel, init_state
from mcac_gb300.snapshot import Snapshot

META = load_golden("meta.npz")
NAMES = sorted({k.split("__")[0] for k in META.files})
FIELDS = {"box_length", "gaz_mean_free_path", "viscosity", "mean_massic_radius", "friction_exponnant", "u_sg",
          "fractal_dimension", "fractal_prefactor", "temperature", "pressure", "density", "volume_fraction",
          "mean_diameter", "dispersion_diameter", "volsurf_method", "random_seed", "n_verlet_divisions"}


@pytest.mark.parametrize("name", NAMES)
def test_physical_model_matches_reference(name):
    keys = [str(k) for k in META[f"{name}__keys"]]
    vals = dict(zip(keys, META[f"{name}__values"]))
    pm = PhysicalModel(text=str(META[f"{name}__ini"]))
    for k in FIELDS & set(keys):
        got = getattr(pm.params, k)
        assert got == vals[k], (name, k, got, vals[k])   # bit-identical
    assert pm.params.n_monomeres == vals["n_monomeres"]


def test_read_metadata_known_answers():
    # pymcac/tests/test_read.py:31-48 pins these PhysicalModel values of
    # validation/params_pytest.ini at 6 significant digits.
    pm = PhysicalModel(text=str(META["params_pytest__ini"]))
    p = pm.params
    six = lambda x: float(f"{x:.6g}")  # noqa: E731
    assert six(p.box_length) == 1.06741e-06
    assert six(p.gaz_mean_free_path) == 4.98113e-07
    assert six(p.viscosity) == 5.662e-05
    assert six(p.friction_exponnant) == 1.378
    assert six(p.mean_massic_radius) == 5.25563e-09
    assert six(p.u_sg) == 5.55556e-08
    assert (p.fractal_dimension, p.fractal_prefactor) == (1.78, 1.3)


def test_invalid_enumeration_is_input_error():
    from mcac_gb300._lib import InputError
    with pytest.raises(InputError):
        PhysicalModel(text="[monomers]\ninitialisation_mode = gaussian\n")
    with pytest.raises(InputError):
        PhysicalModel(text="[surface_growth]\nvolsurf_method = exact\n")


def test_reused_string_quirk():
    # the reference reuses one string for three enumeration keys and relies on
    # missing keys reading as "": a set mode must not leak into the others
    pm = PhysicalModel(text="[monomers]\ninitialisation_mode = normal\n")
    assert pm.params.initialisation_mode == 1
    assert pm.params.volsurf_method == 4 and pm.params.pick_method == 0


def test_initial_placement_is_bit_identical():
    g = load_golden("c1_trace.npz")
    ref = Snapshot.from_npz(g, "init_")
    pm = PhysicalModel(text=str(g["ini"]))
    snap = init_state(pm).to_snapshot()
    assert snap.box_length == ref.box_length
    assert snap.maxradius == ref.maxradius
    np.testing.assert_array_equal(snap.spheres, ref.spheres)
    np.testing.assert_array_equal(snap.aggregates, ref.aggregates)
    np.testing.assert_array_equal(snap.sphere_label, ref.sphere_label)
    np.testing.assert_array_equal(snap.members, ref.members)


def test_too_dense_is_reported():
    from mcac_gb300._lib import TooDenseError
    pm = PhysicalModel(text="[monomers]\nnumber = 200\n[environment]\nvolume_fraction = 0.9\n"
                            "[numerics]\nrandom_seed = 1\n")
    with pytest.raises(TooDenseError):
        init_state(pm)


def test_output_write_rule_parameters():
    # [output] write_* keys (physical_model.cpp:76-78, 185-187): defaults,
    # values, and the reference's extract semantics (an invalid value leaves
    # the default)
    p = PhysicalModel(text="[monomers]\nnumber = 10\n").params
    assert (p.write_events_frequency, p.write_between_event_frequency, p.write_delta_t) == (1, 100, -1.0)
    p = PhysicalModel(text="[output]\nwrite_events_frequency = 3\nwrite_between_event_frequency = 37\n"
                           "write_Delta_t = 2e-6\n").params
    assert (p.write_events_frequency, p.write_between_event_frequency, p.write_delta_t) == (3, 37, 2e-6)
    p = PhysicalModel(text="[output]\nwrite_between_event_frequency = often\n").params
    assert p.write_between_event_frequency == 100


@pytest.mark.parametrize("method", ["caps", "alphas"])
def test_placement_with_corrected_volume_methods(method):
    # a monomer has no contact: "caps" and "alphas" leave its volume and
    # surface as "none" does, so the placement is the same bit for bit
    base = "[monomers]\nnumber = 300\ndispersion_diameter = 1.3\n[numerics]\nrandom_seed = 5\n"
    ref = init_state(PhysicalModel(text=base)).to_snapshot()
    got = init_state(PhysicalModel(text=base + f"[surface_growth]\nvolsurf_method = {method}\n")).to_snapshot()
    np.testing.assert_array_equal(got.spheres, ref.spheres)
    np.testing.assert_array_equal(got.aggregates, ref.aggregates)


def test_exact_volume_back_ends_are_reported():
    # the SBL and ARVO back-ends are optional libraries of the reference,
    # which stops with their error codes when they are absent
    from mcac_gb300._lib import ARVOError, SBLError
    base = "[monomers]\nnumber = 20\n[numerics]\nrandom_seed = 5\n[surface_growth]\nvolsurf_method = "
    with pytest.raises(SBLError):
        init_state(PhysicalModel(text=base + "sbl\n"))
    with pytest.raises(ARVOError):
        init_state(PhysicalModel(text=base + "arvo\n"))
