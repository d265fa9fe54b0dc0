"""Oxidation in the device loop, against the reference's own runs.

With a negative surface-growth flux every sphere shrinks by |u_sg| dt at
every step; spheres at or below rp_min leave their aggregate, aggregates left
empty disappear, and aggregates whose spheres no longer touch split into one
aggregate per connected part (src/calcul.cpp:157-170,
src/aggregats/aggregat.cpp:230-243, 545-655). tests/golden/oxidation.npz
(tests/golden/make_oxidation_golden.py) holds four states grown by the
reference until 15 aggregates of overlapping spheres were left, and the
reference's oxidation runs from them.

When every aggregate shrinks at every step (the default), the shrink after a
physical time t is |u_sg| t for every sphere, and no two aggregates merge
(the merge re-checks the contact after the shrink, aggregat_list.cpp:375);
so which spheres are left and how they group depends on the state and t
alone, not on the moves: the device loop must give the reference's numbers
of spheres and aggregate sizes (up to contacts that break within the last
step, whose end time differs). With the shrink of the moved aggregate only
the outcome is random: 32 runs a side are compared by their means.

The host-driven loop runs oxidation step-exactly: from two of those states,
both ways, it must match the oracle (itself pinned byte for byte to the
reference's runs, tests/test_oracle.py) step by step and byte for byte.
"""
import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import Batch, PhysicalModel
from mcac_gb300.snapshot import A, S, Snapshot

CONTACT_EPSILON = 1e-28


def oxidation_ini(seed: int, time_limit: float, rp_min: float, individual: bool, flux: float) -> str:
    return (f"[monomers]\nnumber = 300\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 5e-3\ntemperature = 1700\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = {flux!r}\n"
            f"[oxidation]\nrp_min = {rp_min!r}\n"
            f"[limits]\nnumber_of_aggregates = 0\nphysical_time = {time_limit!r}\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n"
            + ("individual_surf_reactions = true\n" if individual else ""))


def starts(g):
    return [Snapshot.from_npz(g, f"start_{k}_") for k in range(len(g["start_seeds"]))]


def run_batch(models, states, threads=0):
    with Batch(models, states=states) as b:
        if threads:
            b.threads = threads
        b.run(max_steps=0, steps_per_launch=20000)
        st = b.stats()
        out = b.store_all()
    assert np.all(st["status"] == 0), st["status"]
    assert np.all(st["finished"] == 1)
    return st, out


def periodic_d2(p, q, L):
    d = p - q
    d -= L * np.round(d / L)
    return float(np.sum(d * d))


def check_state(snap: Snapshot, rp_min: float):
    """Every sphere above rp_min, member lists covering the spheres once,
    each aggregate one network of touching spheres, volumes the sums."""
    assert snap.spheres[S["r"]].min() > rp_min
    off = snap.member_offsets()
    assert np.array_equal(np.sort(snap.members), np.arange(snap.ns))
    L = snap.box_length
    pos = snap.spheres[[S["x"], S["y"], S["z"]]].T
    for a in range(snap.na):
        mem = snap.members[off[a]:off[a + 1]]
        assert np.all(snap.sphere_label[mem] == a)
        n = len(mem)
        parent = list(range(n))

        def find(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x
        r = snap.spheres[S["r"], mem]
        for i in range(n):
            for j in range(i + 1, n):
                if periodic_d2(pos[mem[i]], pos[mem[j]], L) - (r[i] + r[j]) ** 2 <= CONTACT_EPSILON:
                    parent[find(j)] = find(i)
        assert len({find(i) for i in range(n)}) == 1, f"aggregate {a} is not connected"
        v = 0.0
        for s in mem:
            v += snap.spheres[S["volume"], s]
        assert snap.aggregates[A["volume"], a] == v


@pytest.mark.gpu
@pytest.mark.parametrize("case", [0, 1])
def test_collective_oxidation_gives_the_reference_structure(case):
    g = load_golden("oxidation.npz")
    name = str(g["coll_cases"][case])
    dt, rp_min, flux = float(g["coll_dt"][case]), float(g["coll_rp_min"][case]), float(g["flux"])
    snaps = starts(g)
    models = [PhysicalModel(text=oxidation_ini(int(g["start_seeds"][k]) + 100, s.time + dt, rp_min, False, flux))
              for k, s in enumerate(snaps)]
    st, out = run_batch(models, snaps)
    for k, snap in enumerate(out):
        ref_sizes = g[f"coll_{name}_{k}_sizes"]
        ref_ns = int(g[f"coll_{name}_{k}_ns"])
        check_state(snap, rp_min)
        # the same shrink: the same spheres left
        assert abs(snap.ns - ref_ns) <= 1, (k, snap.ns, ref_ns)
        sizes = np.sort(snap.n_spheres)[::-1]
        assert abs(len(sizes) - len(ref_sizes)) <= max(2, len(ref_sizes) // 30), (k, len(sizes), len(ref_sizes))
        m = max(len(sizes), len(ref_sizes))
        a = np.zeros(m, dtype=np.int64)
        b = np.zeros(m, dtype=np.int64)
        a[:len(sizes)] = sizes
        b[:len(ref_sizes)] = ref_sizes
        assert np.abs(a - b).sum() <= max(4, ref_ns // 25), (k, sizes[:10], ref_sizes[:10])
        # every sphere shrank by |u_sg| times the elapsed time
        assert snap.time >= snaps[k].time + dt


@pytest.mark.gpu
def test_individual_oxidation_matches_reference_means():
    g = load_golden("oxidation.npz")
    dt, rp_min, flux = float(g["ind_dt"]), float(g["ind_rp_min"]), float(g["flux"])
    snaps = starts(g)
    n_seeds = int(g["ind_seeds"])
    models, states = [], []
    for k, s in enumerate(snaps):
        for j in range(n_seeds):
            models.append(PhysicalModel(text=oxidation_ini(int(g["start_seeds"][k]) + 300 + j, s.time + dt, rp_min,
                                                           True, flux)))
            states.append(s)
    st, out = run_batch(models, states)
    na = np.array([o.na for o in out], dtype=float)
    ns = np.array([o.ns for o in out], dtype=float)
    for o in out[::n_seeds]:
        check_state(o, rp_min)
    ref_na, ref_ns = g["ind_na"].astype(float), g["ind_ns"].astype(float)
    # the same design on both sides (start k, n_seeds runs each): the pooled
    # means within 4 standard errors of their difference, the spread taken
    # from the reference's runs about their own start's mean
    def se(x):
        resid = (x.reshape(len(snaps), n_seeds) - x.reshape(len(snaps), n_seeds).mean(axis=1, keepdims=True))
        return np.sqrt(2.0) * resid.std(ddof=1) / np.sqrt(len(x))
    assert abs(na.mean() - ref_na.mean()) < 4 * se(ref_na) + 1.0, (na.mean(), ref_na.mean(), se(ref_na))
    assert abs(ns.mean() - ref_ns.mean()) < 4 * se(ref_ns) + 1.0, (ns.mean(), ref_ns.mean(), se(ref_ns))


@pytest.mark.gpu
def test_oxidation_is_the_same_at_every_block_size():
    g = load_golden("oxidation.npz")
    snaps = starts(g)[:2]
    outs = []
    for threads in (32, 128):
        models = [PhysicalModel(text=oxidation_ini(900 + k, s.time + 6e-6, 1.3e-8, k == 1, -0.5))
                  for k, s in enumerate(snaps)]
        outs.append(run_batch(models, snaps, threads=threads)[1])
    for x, y in zip(*outs):
        assert x.ns == y.ns and x.na == y.na
        assert np.array_equal(x.spheres, y.spheres)
        assert np.array_equal(x.aggregates, y.aggregates)
        assert np.array_equal(x.members, y.members)


@pytest.mark.gpu
def test_every_sphere_oxidised_leaves_an_empty_box():
    # monodisperse monomers shrink together: all reach rp_min at one step
    ini = ("[monomers]\nnumber = 200\nmean_diameter = 30\ndispersion_diameter = 1.0\n"
           "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 1e-3\ntemperature = 1700\n"
           "[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = -0.5\n"
           "[oxidation]\nrp_min = 1e-8\n[limits]\nnumber_of_aggregates = 0\n"
           "[numerics]\nrandom_seed = 5\nwith_domain_duplication = false\n")
    with Batch([PhysicalModel(text=ini)]) as b:
        b.run(max_steps=0, steps_per_launch=20000)
        st = b.stats()
        snap = b.store_all()[0]
    assert st["status"][0] == 0 and st["finished"][0] == 1
    assert st["n_aggregates"][0] == 0
    assert snap.ns == 0 and snap.na == 0
    # the radius reached rp_min after (15 nm - 10 nm) / |u_sg|
    u = 0.5 / 1800.0
    assert st["time"][0] >= (15e-9 - 1e-8) / u * (1 - 1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["coll", "ind"])
def test_host_loop_oxidation_matches_oracle_step_by_step(mode):
    """The host-driven loop with oxidation, from two of the reference-grown
    states: every step picks, moves, removes, splits and merges as the oracle
    (pinned byte for byte to the reference's own runs, tests/test_oracle.py),
    and the final state is identical byte for byte."""
    import ctypes

    from mcac_gb300 import AggregatList
    from oracle import oracle_py as O
    from test_calcul_gpu import DFIELDS, FIELDS, digest
    g = load_golden("oxidation.npz")
    libc = ctypes.CDLL(None)
    for k in (0, 1):
        start = starts(g)[k]
        text = oxidation_ini(900 + k, start.time + float(g["ind_dt"]), float(g["ind_rp_min"]), mode == "ind",
                             float(g["flux"]))
        libc.srand(900 + k)
        ob = O.OracleBox(text, start)
        ost, otr = ob.calcul(trace=True, trace_capacity=200000)
        libc.srand(900 + k)
        with AggregatList(PhysicalModel(text=text), start) as box:
            st, tr = box.calcul(trace=True, trace_capacity=200000)
            assert (st.steps, st.events, st.n_aggregates) == (ost.steps, ost.events, ost.n_aggregates)
            for f in FIELDS:
                np.testing.assert_array_equal(tr[f], otr[f], err_msg=f)
            for f in DFIELDS:
                np.testing.assert_array_equal(tr[f].view(np.int64), otr[f].view(np.int64), err_msg=f)
            assert st.time == ost.time
            out = box.store()
            assert digest(out) == digest(ob.store())
        assert out.ns < start.ns and out.na > start.na  # spheres removed, aggregates split
