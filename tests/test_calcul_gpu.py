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
from mcac_gb300 import AggregatList, PhysicalModel, set_merge_grid_min
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
@pytest.mark.parametrize("fixture", ["c1_trace.npz", "ln_late.npz"])
def test_run_with_cell_grid_pair_search_matches_oracle(fixture):
    """Every merge finds its intra-aggregate contact pairs on the hashed cell
    grid (used from 2048 merged spheres by default, here from 2): same steps,
    same merges, same final state byte for byte."""
    g = load_golden(fixture)
    prev = set_merge_grid_min(2)
    try:
        compare_runs(str(g["ini"]))
    finally:
        set_merge_grid_min(prev)


@pytest.mark.gpu
def test_monodisperse_run_matches_oracle():
    # identical monomers: every pick goes through the tie order of std::sort
    ini = ("[monomers]\nnumber = 800\nmean_diameter = 30\ndispersion_diameter = 1.0\n"
           "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 3e-3\ntemperature = 1800\n"
           "[limits]\nnumber_of_aggregates = 20\n[numerics]\nrandom_seed = 1005\nwith_domain_duplication = false\n")
    compare_runs(ini)


@pytest.mark.gpu
def test_partly_tied_weights_run_matches_oracle():
    """Distinct weights with a few runs of equal ones: the pick order comes
    from the kept time-step order, and from std::sort's order of equal keys
    only when a pick lands inside a run. Forty monomers are given the radius
    (and so every aggregate field but the position) of monomer 0."""
    import ctypes

    from mcac_gb300 import init_state
    from mcac_gb300.snapshot import A, S
    ini = ("[monomers]\nnumber = 1500\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
           "initialisation_mode = normal\n[environment]\nvolume_fraction = 2e-3\ntemperature = 1700\n"
           "[limits]\nnumber_of_aggregates = 200\n[numerics]\nrandom_seed = 77\nwith_domain_duplication = false\n")
    pm = PhysicalModel(text=ini)
    snap = init_state(pm).to_snapshot()
    L = snap.box_length
    pos = snap.spheres[[S["x"], S["y"], S["z"]]].T
    r = snap.spheres[S["r"]]
    keep_pos = [A["x"], A["y"], A["z"], A["rx"], A["ry"], A["rz"], A["time"]]
    chosen = []
    for m in range(1, len(r)):
        d = pos - pos[m]
        d -= L * np.floor(d / L + 0.5)
        dist = np.sqrt((d ** 2).sum(1))
        dist[m] = np.inf
        if np.all(dist - (r + r[0]) > 1e-8):  # room for the new radius
            chosen.append(m)
        if len(chosen) == 40:
            break
    for m in chosen:
        s = snap.members[snap.member_offsets()[m]]
        for f in ("r", "volume", "surface"):
            snap.spheres[S[f], s] = snap.spheres[S[f], 0]
        for f in range(21):
            if f not in keep_pos:
                snap.aggregates[f, m] = snap.aggregates[f, 0]
    libc = ctypes.CDLL(None)
    libc.srand(77)
    ob = O.OracleBox(ini, snap)
    ost, otr = ob.calcul(max_steps=30000, trace=True, trace_capacity=30000)
    libc.srand(77)
    with AggregatList(pm, snap) as box:
        st, tr = box.calcul(max_steps=30000, trace=True, trace_capacity=30000)
        assert (st.steps, st.events) == (ost.steps, ost.events)
        for f in FIELDS:
            np.testing.assert_array_equal(tr[f], otr[f], err_msg=f)
        for f in DFIELDS:
            np.testing.assert_array_equal(tr[f].view(np.int64), otr[f].view(np.int64), err_msg=f)
        assert digest(box.store()) == digest(ob.store())
    assert len(chosen) == 40
    assert st.events > 100


@pytest.mark.gpu
def test_dense_box_run_matches_oracle_step_by_step():
    """100,000 monomers: the fine neighbour grid is used and kept up to date
    through translations and merges; 4,000 steps stay the oracle's."""
    ini = ("[monomers]\nnumber = 100000\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
           "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 1e-3\ntemperature = 1700\n"
           "[limits]\nnumber_of_aggregates = 100\n[numerics]\nrandom_seed = 1\nwith_domain_duplication = false\n")
    st = compare_runs(ini, max_steps=4000)
    assert st.events > 100


@pytest.mark.gpu
def test_cpu_time_limits_stop_the_run():
    """[limits] cpu and cpu_event (physical_model.cpp:311-326): processor
    seconds since the box was made, and since the last event, stop calcul."""
    import time

    base = ("[monomers]\nnumber = 3000\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            "initialisation_mode = lognormal\n[environment]\nvolume_fraction = {fv}\ntemperature = 1700\n"
            "[limits]\nnumber_of_aggregates = 1\n{limit}\n"
            "[numerics]\nrandom_seed = 31\nwith_domain_duplication = false\n")
    # (events are rare in the dilute box: 0.05 s pass between two of them)
    for limit, fv in (("cpu = 0.3", "1e-3"), ("cpu_event = 0.05", "1e-6")):
        pm = PhysicalModel(text=base.format(limit=limit, fv=fv))
        with AggregatList(pm) as box:
            c0 = time.process_time()
            st, _ = box.calcul(max_steps=2_000_000)
            used = time.process_time() - c0
        assert st.finished == 1 and st.n_aggregates > 1, limit
        assert st.steps < 2_000_000
        if limit.startswith("cpu ="):
            assert used >= 0.3 * 0.9
