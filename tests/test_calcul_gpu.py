"""Whole seeded runs through the host-driven MC loop, against the reference.

The loop of src/calcul.cpp runs on the host, the contact search, translation
and merge geometry on the GPU. With identical seeds every MC step must pick
the same aggregate, find the same contact at the same FP64 distance, merge
the same pair, and the final state must be identical byte for byte.
"""
import hashlib

import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import AggregatList, PhysicalModel


def digest(snap):
    h = hashlib.sha256()
    for arr in (snap.spheres, snap.sphere_label, snap.aggregates, snap.n_spheres, snap.members):
        h.update(np.ascontiguousarray(arr).tobytes())
    h.update(np.array([snap.maxradius, snap.box_length], dtype=np.float64).tobytes())
    return h.hexdigest()


@pytest.mark.gpu
def test_config1_run_reproduces_reference_step_by_step():
    g = load_golden("c1_trace.npz")
    pm = PhysicalModel(text=str(g["ini"]))
    with AggregatList(pm) as box:
        stats, tr = box.calcul(trace=True, trace_capacity=len(g["t_picked"]) + 10)
        n = len(g["t_picked"])
        assert stats.steps == n and stats.n_aggregates == int(g["final_n_agg"])
        np.testing.assert_array_equal(tr["picked"], g["t_picked"])
        np.testing.assert_array_equal(tr["contact"], g["t_contact"])
        np.testing.assert_array_equal(tr["merged"], g["t_merged"])
        np.testing.assert_array_equal(tr["moving_sphere"], g["t_moving_sphere"])
        np.testing.assert_array_equal(tr["other_sphere"], g["t_other_sphere"])
        np.testing.assert_array_equal(tr["other_agg"], g["t_other_agg"])
        np.testing.assert_array_equal(tr["contact_distance"].view(np.int64), g["t_contact_distance"].view(np.int64))
        np.testing.assert_array_equal(tr["time_after"].view(np.int64), g["t_time_after"].view(np.int64))
        assert digest(box.store()) == str(g["final_digest"])


@pytest.mark.gpu
def test_lognormal_run_reproduces_reference_final_state():
    g = load_golden("ln_late.npz")
    pm = PhysicalModel(text=str(g["ini"]))
    with AggregatList(pm) as box:
        stats, tr = box.calcul(trace=True, trace_capacity=int(g["run_steps"]) + 10)
        assert stats.steps == int(g["run_steps"])
        assert stats.events == int(g["run_events"])
        np.testing.assert_array_equal(np.flatnonzero(tr["merged"]), g["merge_steps"])
        assert stats.time == float(g["final_time"])
        assert digest(box.store()) == str(g["final_digest"])
