"""The seeded synthetic snapshot of the contact-search benchmark (host only).

Checked: it is deterministic in the seed, has the requested sphere and
aggregate counts with sizes in [1, max_size], fills the requested volume
fraction, keeps every aggregate field equal to its definition, touches
within each aggregate (ballistic sticking) and never across aggregates, and
loads into the oracle, whose queries find contacts on it.
"""
import numpy as np
import pytest

from mcac_gb300 import PhysicalModel, synthetic_state
from mcac_gb300._lib import MCACError
from mcac_gb300.snapshot import A, S
from mcac_gb300.workloads import contact_search_case, contact_search_ini
from oracle import oracle_py as O
from test_device_loop_gpu import check_state


def test_synthetic_state_is_deterministic_and_sized():
    a = contact_search_case(n_spheres=8000, n_aggregates=160, n_queries=50, seed=4)
    b = contact_search_case(n_spheres=8000, n_aggregates=160, n_queries=50, seed=4)
    c = contact_search_case(n_spheres=8000, n_aggregates=160, n_queries=50, seed=5)
    assert np.array_equal(a.state.spheres.view(np.int64), b.state.spheres.view(np.int64))
    assert np.array_equal(a.sources, b.sources) and np.array_equal(a.directions, b.directions)
    assert not np.array_equal(a.state.spheres, c.state.spheres)
    st = a.state.state
    assert st.n_spheres == 8000 and st.n_aggregates == 160
    n = a.state.n_spheres
    assert n.sum() == 8000 and n.min() >= 1 and n.max() <= 500
    vol = a.state.spheres[S["volume"]].sum()
    assert abs(vol / st.box_length ** 3 - 5e-3) < 1e-9
    np.testing.assert_allclose(np.linalg.norm(a.directions, axis=1), 1.0, rtol=1e-15)
    assert np.array_equal(a.distances, a.state.aggregates[A["lpm"], a.sources])


def test_synthetic_state_is_a_valid_box():
    case = contact_search_case(n_spheres=3000, n_aggregates=60, n_queries=10, seed=9)
    snap = case.state.to_snapshot()
    check_state(snap)
    # every sphere of an aggregate touches another one of it (coordination)
    multi = snap.n_spheres > 1
    assert np.all(snap.aggregates[A["coordination_number"], multi] >= 1.0)
    assert snap.maxradius == snap.aggregates[A["rmax"]].max()


def test_oracle_answers_queries_on_synthetic_state():
    case = contact_search_case(n_spheres=20_000, n_aggregates=400, n_queries=400, seed=3)
    ob = O.OracleBox(case.model.to_ini(), case.state.to_snapshot())
    hits = 0
    for k in range(len(case.sources)):
        c = ob.distance_to_next_contact(case.sources[k], case.directions[k], 5 * case.distances[k])
        if c.moving_sphere >= 0:
            hits += 1
            assert 0 <= c.distance <= 5 * case.distances[k]
            assert c.other_aggregate != case.sources[k]
    assert hits > 10


def test_synthetic_state_rejects_bad_sizes():
    pm = PhysicalModel(text=contact_search_ini(1000))
    with pytest.raises(MCACError):
        synthetic_state(pm, 1, 500)      # 1000 spheres cannot fit one aggregate of <= 500
    with pytest.raises(MCACError):
        synthetic_state(pm, 2000, 500)   # more aggregates than spheres
