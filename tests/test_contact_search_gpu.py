"""Many contact queries at once (mcacg_distance_to_next_contacts).

The batched entry point runs the same block-level search as the per-step
query, one thread block per query, with each block's candidate scratch kept
apart. Checked: its answers on the reference's golden states equal the
reference's bit for bit; on synthetic ballistic snapshots (the
contact-search benchmark's shape: log-normal diameters, aggregates of 1-500
spheres, 5000 ppm) they equal the oracle's bit for bit, distance bits and
sphere and aggregate indices, up to the full 1,000,000-sphere,
10,000-query case; and they equal the one-at-a-time entry point.
"""
import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import AggregatList, PhysicalModel
from mcac_gb300._lib import MCACError
from mcac_gb300.snapshot import A, Snapshot
from mcac_gb300.workloads import contact_search_case
from oracle import oracle_py as O


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


@pytest.mark.gpu
@pytest.mark.parametrize("fixture", ["c1_q5000.npz", "ln_late.npz"])
def test_batched_queries_match_reference_bitwise(fixture):
    g = load_golden(fixture)
    snap = Snapshot.from_npz(g, "s_")
    with AggregatList(PhysicalModel(text=str(g["ini"])), snap) as box:
        out, ms = box.distance_to_next_contacts(g["q_label"], g["q_dir"], g["q_distance"])
    assert ms > 0
    assert np.array_equal(bits(out["distance"]), bits(g["q_contact_distance"]))
    assert np.array_equal(out["moving_sphere"], g["q_moving_sphere"])
    assert np.array_equal(out["other_sphere"], g["q_other_sphere"])
    assert np.array_equal(out["other_aggregate"], g["q_other_agg"])
    hit = out["moving_sphere"] >= 0
    assert np.array_equal(out["moving_aggregate"][hit], g["q_label"][hit])
    assert np.all(out["moving_aggregate"][~hit] == -1)


def oracle_answers(case):
    ob = O.OracleBox(case.model.to_ini(), case.state.to_snapshot())
    res = np.zeros(len(case.sources), dtype=[("d", np.float64), ("ms", np.int64), ("os", np.int64),
                                              ("oa", np.int64)])
    for k in range(len(case.sources)):
        c = ob.distance_to_next_contact(case.sources[k], case.directions[k], case.distances[k])
        res[k] = (c.distance, c.moving_sphere, c.other_sphere, c.other_aggregate)
    ob.close()
    return res


def check_against_oracle(case, out):
    ref = oracle_answers(case)
    bad = np.flatnonzero((bits(out["distance"]) != bits(ref["d"])) | (out["moving_sphere"] != ref["ms"])
                         | (out["other_sphere"] != ref["os"]) | (out["other_aggregate"] != ref["oa"]))
    assert bad.size == 0, [(int(k), out[k], ref[k]) for k in bad[:5]]
    return ref


@pytest.mark.gpu
@pytest.mark.parametrize("n, na, nq, seed", [(20_000, 400, 3000, 3), (60_000, 1200, 4000, 11)])
def test_batched_queries_match_oracle(n, na, nq, seed):
    case = contact_search_case(n_spheres=n, n_aggregates=na, n_queries=nq, seed=seed)
    with AggregatList(case.model, case.state) as box:
        out, _ = box.distance_to_next_contacts(case.sources, case.directions, case.distances)
        # the same queries, five times as long: more candidates and contacts
        out5, _ = box.distance_to_next_contacts(case.sources, case.directions, 5 * case.distances)
    ref = check_against_oracle(case, out)
    case.distances = 5 * case.distances
    ref5 = check_against_oracle(case, out5)
    assert (ref["ms"] >= 0).sum() > 20 and (ref5["ms"] >= 0).sum() > (ref["ms"] >= 0).sum()


@pytest.mark.gpu
def test_batched_equals_single_queries():
    case = contact_search_case(n_spheres=30_000, n_aggregates=600, n_queries=500, seed=5)
    with AggregatList(case.model, case.state) as box:
        out, _ = box.distance_to_next_contacts(case.sources, case.directions, 4 * case.distances)
        for k in range(len(case.sources)):
            one = box.distance_to_next_contact(int(case.sources[k]), case.directions[k], 4 * case.distances[k])
            assert bits(one.distance) == bits(out["distance"][k])
            assert (one.moving_sphere, one.other_sphere, one.moving_aggregate, one.other_aggregate) == tuple(
                int(out[f][k]) for f in ("moving_sphere", "other_sphere", "moving_aggregate", "other_aggregate"))
        # a state that only reads: a second batch gives the same answers
        again, _ = box.distance_to_next_contacts(case.sources, case.directions, 4 * case.distances)
        assert np.array_equal(again.view(np.uint8), out.view(np.uint8))


@pytest.mark.gpu
def test_batched_queries_edge_cases():
    case = contact_search_case(n_spheres=5_000, n_aggregates=100, n_queries=10, seed=2)
    with AggregatList(case.model, case.state) as box:
        out, ms = box.distance_to_next_contacts(np.zeros(0, np.int64), np.zeros((0, 3)), np.zeros(0))
        assert len(out) == 0 and ms == 0.0
        with pytest.raises(MCACError):
            box.distance_to_next_contacts([len(box)], [[1.0, 0.0, 0.0]], [1e-7])
        with pytest.raises(MCACError):
            box.distance_to_next_contacts([-1], [[1.0, 0.0, 0.0]], [1e-7])
        # zero length: no contact anywhere; one query repeated many times
        out, _ = box.distance_to_next_contacts(case.sources, case.directions, np.zeros(10))
        assert np.all(out["moving_sphere"] == -1)
        rep = np.full(2000, case.sources[0])
        out, _ = box.distance_to_next_contacts(rep, np.repeat(case.directions[:1], 2000, 0),
                                               np.full(2000, 20 * case.distances[0]))
        assert np.all(bits(out["distance"]) == bits(out["distance"][0]))


@pytest.mark.gpu
def test_contact_search_full_size_matches_oracle():
    """1,000,000 spheres in 20,000 aggregates, 10,000 queries."""
    case = contact_search_case()
    with AggregatList(case.model, case.state) as box:
        out, ms = box.distance_to_next_contacts(case.sources, case.directions, case.distances)
    ref = check_against_oracle(case, out)
    assert (ref["ms"] >= 0).sum() > 100


DENSE_INI = ("[monomers]\nnumber = 100000\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
             "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 1e-3\ntemperature = 1700\n"
             "[limits]\nnumber_of_aggregates = 100\n[numerics]\nrandom_seed = 1\nwith_domain_duplication = false\n")


@pytest.mark.gpu
def test_fine_grid_queries_match_oracle_on_dense_box():
    """100,000 monomers, 100 per Verlet cell: neighbours are found through
    the fine grid (few aggregates visited per query), and the answers are
    still the oracle's, bit for bit. Queries four times as long mix both
    ways of finding neighbours."""
    from mcac_gb300 import init_state
    from mcac_gb300.workloads import random_directions
    pm = PhysicalModel(text=DENSE_INI)
    snap = init_state(pm).to_snapshot()
    rng = np.random.Generator(np.random.PCG64(7))
    src = rng.integers(0, snap.na, 3000).astype(np.int64)
    dirs = random_directions(rng, 3000)
    lpm = snap.aggregates[A["lpm"], src]
    ob = O.OracleBox(DENSE_INI, snap)
    with AggregatList(pm, snap) as box:
        for scale in (1.0, 4.0):
            dist = scale * lpm
            box.set_profiling(True)
            out, _ = box.distance_to_next_contacts(src, dirs, dist)
            prof = box.take_profile()
            box.set_profiling(False)
            if scale == 1.0:
                # the Verlet cells alone hold ~1,000 aggregates per query
                assert prof["scanned"] / prof["queries"] < 200
            for k in range(200):
                one = box.distance_to_next_contact(int(src[k]), dirs[k], float(dist[k]))
                assert bits(one.distance) == bits(out["distance"][k])
            for k in range(len(src)):
                c = ob.distance_to_next_contact(src[k], dirs[k], dist[k])
                assert bits(c.distance) == bits(out["distance"][k]), (scale, k)
                assert (c.moving_sphere, c.other_sphere, c.other_aggregate) == (
                    out["moving_sphere"][k], out["other_sphere"][k], out["other_aggregate"][k]), (scale, k)
            assert (out["moving_sphere"] >= 0).sum() > (20 if scale == 1.0 else 50)


@pytest.mark.gpu
def test_large_aggregate_queries_match_oracle():
    """A box taken to four aggregates of ~750 spheres, each about as wide as
    half the box: the sphere-pair search meets the cross-motion grid and
    several periodic images. Queries of 5 to 200 mean free paths, bit for
    bit against the oracle."""
    from mcac_gb300 import Batch
    from mcac_gb300.workloads import random_directions
    ini = ("[monomers]\nnumber = 3000\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
           "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 4e-3\ntemperature = 1700\n"
           "[limits]\nnumber_of_aggregates = 4\n[numerics]\nrandom_seed = 31\nwith_domain_duplication = false\n")
    pm = PhysicalModel(text=ini)
    with Batch([pm]) as b:
        b.run(max_steps=0, steps_per_launch=20000)
        assert b.stats()["finished"][0] == 1
        snap = b.store(0)
    assert snap.na <= 4 and snap.aggregates[A["rmax"]].max() > 0.2 * snap.box_length
    rng = np.random.Generator(np.random.PCG64(99))
    n = 300
    src = rng.integers(0, snap.na, n).astype(np.int64)
    dirs = random_directions(rng, n)
    # late in a run a mean free path is a few nm against gaps of ~100 nm
    dist = snap.aggregates[A["lpm"], src] * np.exp(rng.uniform(np.log(5.0), np.log(200.0), n))
    ob = O.OracleBox(ini, snap)
    with AggregatList(pm, snap) as box:
        box.set_profiling(True)
        out, _ = box.distance_to_next_contacts(src, dirs, dist)
        prof = box.take_profile()
    assert prof["cand_spheres"] > 100 * n  # large candidates: the pair search is exercised
    hits = 0
    for k in range(n):
        c = ob.distance_to_next_contact(src[k], dirs[k], dist[k])
        assert bits(c.distance) == bits(out["distance"][k]), k
        assert (c.moving_sphere, c.other_sphere, c.other_aggregate) == (
            out["moving_sphere"][k], out["other_sphere"][k], out["other_aggregate"][k]), k
        hits += c.moving_sphere >= 0
    assert hits > 20
