"""Whole seeded runs through the host-driven MC loop, against the oracle.

The loop of src/calcul.cpp runs on the host, the contact search, translation
and merge geometry on the GPU. Directions and aggregate physics come from the
C library's libm (acos/sin/cos, erf/exp/pow), which is not bit-identical
across CPU architectures, so a run is compared with the oracle (the C
restatement, itself pinned to the reference by tests/test_oracle.py) run on
the same machine: every MC step must pick the same aggregate, find the same
contact at the same FP64 distance and merge the same pair, and the final
state must be identical byte for byte.
"""
import hashlib

import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import AggregatList, PhysicalModel
from oracle import oracle_py as O

FIELDS = ["picked", "contact", "merged", "moving_sphere", "other_sphere", "moving_agg", "other_agg", "n_agg_after"]
DFIELDS = ["deltatemps", "full_distance", "dir", "contact_distance", "move_distance", "time_after"]


def digest(snap):
    h = hashlib.sha256()
    for arr in (snap.spheres, snap.sphere_label, snap.aggregates, snap.n_spheres, snap.members):
        h.update(np.ascontiguousarray(arr).tobytes())
    h.update(np.array([snap.maxradius, snap.box_length], dtype=np.float64).tobytes())
    return h.hexdigest()


def compare_runs(ini_text, max_steps=0):
    pm = PhysicalModel(text=ini_text)
    ob = O.OracleBox(ini_text)
    ost, otr = ob.calcul(max_steps=max_steps, trace=True, trace_capacity=max_steps or 2_000_000)
    with AggregatList(pm) as box:
        st, tr = box.calcul(max_steps=max_steps, trace=True, trace_capacity=max_steps or 2_000_000)
        assert (st.steps, st.events, st.n_aggregates) == (ost.steps, ost.events, ost.n_aggregates)
        for f in FIELDS:
            np.testing.assert_array_equal(tr[f], otr[f], err_msg=f)
        for f in DFIELDS:
            np.testing.assert_array_equal(tr[f].view(np.int64), otr[f].view(np.int64), err_msg=f)
        assert st.time == ost.time
        assert digest(box.store()) == digest(ob.store())
    return st


@pytest.mark.gpu
def test_config1_run_matches_oracle_step_by_step():
    g = load_golden("c1_trace.npz")
    st = compare_runs(str(g["ini"]))
    assert st.steps == len(g["t_picked"])  # same length as the reference's own run


@pytest.mark.gpu
def test_lognormal_run_matches_oracle_step_by_step():
    g = load_golden("ln_late.npz")
    st = compare_runs(str(g["ini"]))
    assert st.events == int(g["run_events"])


@pytest.mark.gpu
def test_monodisperse_run_matches_oracle():
    # identical monomers: every pick goes through the tie order of std::sort
    ini = ("[monomers]\nnumber = 800\nmean_diameter = 30\ndispersion_diameter = 1.0\n"
           "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 3e-3\ntemperature = 1800\n"
           "[limits]\nnumber_of_aggregates = 20\n[numerics]\nrandom_seed = 1005\nwith_domain_duplication = false\n")
    compare_runs(ini)
