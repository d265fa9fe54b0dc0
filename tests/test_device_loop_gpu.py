"""The device-resident MC loop (batched form).

Its contact search, translation and merge geometry are the kernels checked
bit for bit in test_contact_gpu.py; its pick walks a sum tree and its
directions and aggregate physics use CUDA's libm, so it follows the reference
statistically. Checked here: the state stays a valid MCAC state (partition of
the spheres, aggregate fields equal to their definitions, no two aggregates
interpenetrating), runs are deterministic, and ensemble statistics agree with
the oracle (the C restatement of the reference) within sampling error.
"""
import numpy as np
import pytest

from mcac_gb300 import AggregatList, Batch, PhysicalModel, run_device
from mcac_gb300.snapshot import A, S
from oracle import oracle_py as O


def small_ini(n, seed, mode="normal", disp=1.25, fv=1e-3, nagg=1, T=1700, wait=-1):
    return (f"[monomers]\nnumber = {n}\nmean_diameter = 30\ndispersion_diameter = {disp}\n"
            f"initialisation_mode = {mode}\n[environment]\nvolume_fraction = {fv}\ntemperature = {T}\n"
            f"[limits]\nnumber_of_aggregates = {nagg}\nn_iter_without_event = {wait}\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n")


def seq_sum(x):
    return float(np.cumsum(np.asarray(x, dtype=np.float64))[-1]) if len(x) else 0.0


def periodic(d, L):
    return d - L * np.floor(d / L + 0.5)


def check_state(snap, tol=1e-12):
    L = snap.box_length
    ns, na = snap.ns, snap.na
    # the member lists partition the spheres and agree with the sphere labels
    assert snap.n_spheres.sum() == ns
    assert np.array_equal(np.sort(snap.members), np.arange(ns))
    off = snap.member_offsets()
    for a in range(na):
        mem = snap.members[off[a]:off[a + 1]]
        assert np.all(snap.sphere_label[mem] == a)
        vol = snap.spheres[S["volume"], mem]
        V = seq_sum(vol)
        assert snap.aggregates[A["volume"], a] == V
        rel = snap.spheres[[S["rx"], S["ry"], S["rz"]]][:, mem]
        r = np.array([seq_sum(rel[k] * vol) for k in range(3)]) / V
        np.testing.assert_allclose(snap.aggregates[[A["rx"], A["ry"], A["rz"]], a], r, rtol=tol, atol=1e-30)
        dc = np.sqrt(((rel - r[:, None]) ** 2).sum(0))
        rmax = np.max(snap.spheres[S["r"], mem] + dc)
        if len(mem) > 1:
            # a monomer keeps the r_max of its radius before the reference's
            # volume-fraction rescaling (aggregat_list_storage.cpp:75-87)
            np.testing.assert_allclose(snap.aggregates[A["rmax"], a], rmax, rtol=tol)
        # sphere positions = aggregate reference point + relative positions
        pos = snap.spheres[[S["x"], S["y"], S["z"]]][:, mem]
        ref = pos - rel
        assert np.all(np.abs(periodic(ref - ref[:, :1], L)) < 1e-12 * L)
    # no two aggregates interpenetrate, except by what the reference's own
    # bounding-sphere filter can miss: a monomer that was never merged keeps
    # the r_max of its radius before the volume-fraction rescaling, so its
    # sphere may reach r - r_max beyond its bounding sphere
    p = snap.spheres[[S["x"], S["y"], S["z"]]].T
    rad = snap.spheres[S["r"]]
    lab = snap.sphere_label
    agg_slack = np.where(snap.n_spheres == 1,
                         np.maximum(0.0, rad[snap.members[snap.member_offsets()[:-1]]]
                                    - snap.aggregates[A["rmax"]]), 0.0)
    slack = agg_slack[lab]
    for i in range(ns):
        d = periodic(p[i + 1:] - p[i], L)
        dist = np.sqrt((d ** 2).sum(1))
        other = lab[i + 1:] != lab[i]
        gap = dist - (rad[i + 1:] + rad[i])
        allowed = -(slack[i + 1:] + slack[i]) - 1e-9 * rad[i]
        assert np.all(gap[other] > allowed[other]), (i, (gap - allowed)[other].min())


@pytest.mark.gpu
def test_batch_keeps_valid_states():
    models = [PhysicalModel(text=small_ini(n, 40 + k, mode=("normal" if k % 2 else "lognormal"),
                                           disp=(1.25 if k % 2 else 1.4), fv=(1e-3 if k % 3 else 5e-3)))
              for k, n in enumerate([200, 350, 500, 800, 300, 650, 420, 900])]
    with Batch(models) as b:
        b.run(max_steps=4000, steps_per_launch=1000)
        st = b.stats()
        assert np.all(st["status"] == 0)
        assert np.all(st["steps"] > 0)
        every = b.store_all()
        # into buffers sized for the initial state (more room than needed)
        from mcac_gb300._lib import StateBuffers
        bufs = [StateBuffers(m.params.n_monomeres, m.params.n_monomeres) for m in models]
        again = [x.to_snapshot() for x in b.store_all(raw=True, out=bufs)]
        for s1, s2 in zip(again, every):
            assert np.array_equal(s1.aggregates.view(np.int64), s2.aggregates.view(np.int64))
            assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64))
            assert np.array_equal(s1.members, s2.members) and np.array_equal(s1.n_spheres, s2.n_spheres)
        for k in range(len(models)):
            snap = b.store(k)
            assert snap.na == models[k].params.n_monomeres - st["events"][k]
            check_state(snap)
            assert np.array_equal(every[k].spheres.view(np.int64), snap.spheres.view(np.int64))
            assert np.array_equal(every[k].members, snap.members) and every[k].time == snap.time


@pytest.mark.gpu
def test_batch_is_deterministic():
    models = [PhysicalModel(text=small_ini(400, 7 + k, mode="lognormal", disp=1.3, fv=3e-3)) for k in range(4)]
    snaps = []
    for _ in range(2):
        with Batch(models) as b:
            b.run(max_steps=3000, steps_per_launch=700)
            snaps.append([b.store(k) for k in range(len(models))])
    for s1, s2 in zip(*snaps):
        assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64))
        assert np.array_equal(s1.aggregates.view(np.int64), s2.aggregates.view(np.int64))
        assert np.array_equal(s1.members, s2.members)


@pytest.mark.gpu
def test_device_and_host_steps_interleave():
    pm = PhysicalModel(text=small_ini(600, 3, fv=3e-3))
    with AggregatList(pm) as box:
        box.calcul(max_steps=500)
        s = run_device(box, max_steps=1500)
        assert s.steps == 1500
        box.calcul(max_steps=500)
        s2 = run_device(box, max_steps=500)
        assert s2.steps == 500
        check_state(box.store())


@pytest.mark.gpu
def test_batch_runs_to_stop_criterion():
    models = [PhysicalModel(text=small_ini(150 + 50 * k, 100 + k, fv=5e-3, nagg=5)) for k in range(6)]
    with Batch(models) as b:
        b.run(max_steps=0, steps_per_launch=5000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        assert np.all(st["n_aggregates"] <= 5)


def ensemble_summary(snaps):
    """Fractal law fit over all aggregates (as in the reference's validation
    notebooks: log Np against log(2 Rg / dp)) and the mean aggregate size."""
    npp, rg_dp = [], []
    for s in snaps:
        for a in range(s.na):
            n = s.n_spheres[a]
            if n >= 3:
                npp.append(n)
                rg_dp.append(s.aggregates[A["dg_over_dp"], a])
    npp, rg_dp = np.array(npp, float), np.array(rg_dp)
    slope, icpt = np.polyfit(np.log(rg_dp), np.log(npp), 1)
    return slope, np.exp(icpt), npp.mean()


@pytest.mark.gpu
def test_ensemble_statistics_match_oracle():
    n_boxes, n, stop = 32, 300, 15
    inis = [small_ini(n, 500 + k, mode="lognormal", disp=1.25, fv=5e-3, nagg=stop) for k in range(n_boxes)]
    with Batch([PhysicalModel(text=t) for t in inis]) as b:
        b.run(max_steps=0, steps_per_launch=10000)
        st = b.stats()
        assert np.all(st["finished"] == 1)
        gpu_snaps = [b.store(k) for k in range(n_boxes)]
        gpu_steps = st["steps"].astype(float)
        gpu_time = st["time"]
    cpu_snaps, cpu_steps, cpu_time = [], [], []
    for t in inis:
        ob = O.OracleBox(t)
        s, _ = ob.calcul()
        cpu_snaps.append(ob.store())
        cpu_steps.append(s.steps)
        cpu_time.append(s.time)
    cpu_steps, cpu_time = np.array(cpu_steps, float), np.array(cpu_time)

    def close(a, b_, k=4.0):
        se = np.sqrt(a.var(ddof=1) / len(a) + b_.var(ddof=1) / len(b_))
        return abs(a.mean() - b_.mean()) <= k * se

    assert close(np.log(gpu_steps), np.log(cpu_steps)), (gpu_steps.mean(), cpu_steps.mean())
    assert close(np.log(gpu_time), np.log(cpu_time)), (gpu_time.mean(), cpu_time.mean())
    dg, kg, mg = ensemble_summary(gpu_snaps)
    dc, kc, mc = ensemble_summary(cpu_snaps)
    assert abs(dg - dc) < 0.15, (dg, dc)     # fractal dimension
    assert abs(np.log(kg / kc)) < 0.3, (kg, kc)  # prefactor
    assert abs(mg / mc - 1) < 0.1, (mg, mc)


@pytest.mark.gpu
def test_results_do_not_depend_on_threads_per_box():
    models = [PhysicalModel(text=small_ini(n, 70 + k, mode="lognormal", disp=1.3, fv=4e-3, nagg=20))
              for k, n in enumerate([300, 650, 1200])]
    snaps = {}
    for nt in (32, 64, 128, 256, 512):
        with Batch(models) as b:
            b.threads = nt
            b.run(max_steps=0, steps_per_launch=5000)  # to 20 aggregates: large tiles and merges
            assert b.threads == nt
            assert np.all(b.stats()["status"] == 0)
            snaps[nt] = [b.store(k) for k in range(len(models))]
    for nt in (32, 64, 128, 512):  # 32: the small shared-memory plan
        for s1, s2 in zip(snaps[nt], snaps[256]):
            assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64))
            assert np.array_equal(s1.aggregates.view(np.int64), s2.aggregates.view(np.int64))
            assert np.array_equal(s1.members, s2.members)
    with Batch(models[:1]) as b:
        with pytest.raises(Exception):
            b.threads = 96


@pytest.mark.gpu
def test_timed_runs_give_the_same_boxes():
    """Launches cut by wall time (each box as many steps as fit) leave every
    trajectory as it is."""
    models = [PhysicalModel(text=small_ini(n, 80 + k, fv=5e-3, nagg=4)) for k, n in enumerate([180, 420, 260])]
    with Batch(models) as b:
        b.run(max_steps=0, steps_per_launch=4000)
        ref = b.store_all()
        ref_steps = b.stats()["steps"].copy()
    with Batch(models) as b:
        for _ in range(1000):
            b.run_timed(3.0)
            st = b.stats()
            if np.all(st["finished"] == 1):
                break
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        assert np.array_equal(st["steps"], ref_steps)
        for s1, s2 in zip(b.store_all(), ref):
            assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64))
            assert np.array_equal(s1.members, s2.members)


@pytest.mark.gpu
def test_batch_loads_host_states_in_place():
    """A batch made from host states (page-locked or not) holds them bit for
    bit, continues them identically, and rejects inconsistent ones with the
    reference's InputError-style status instead of reading out of bounds."""
    from mcac_gb300._lib import MCACError, StateBuffers
    models = [PhysicalModel(text=small_ini(n, 90 + k, mode="lognormal", disp=1.3, fv=4e-3))
              for k, n in enumerate([240, 510, 330])]
    with Batch(models) as b:
        b.run(max_steps=1500, steps_per_launch=1500)
        mid = b.store_all()
        pinned = b.store_all(raw=True, pinned=True)
    plain = [StateBuffers.from_snapshot(s) for s in mid]
    finals = []
    for states in (pinned, plain):
        with Batch(models, states=states) as b:
            for s1, s2 in zip(b.store_all(), mid):  # held exactly
                assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64))
                assert np.array_equal(s1.aggregates.view(np.int64), s2.aggregates.view(np.int64))
                assert np.array_equal(s1.members, s2.members) and np.array_equal(s1.sphere_label, s2.sphere_label)
                assert s1.time == s2.time
            b.run(max_steps=1000, steps_per_launch=1000)
            assert np.all(b.stats()["status"] == 0)
            finals.append(b.store_all())
    for s1, s2 in zip(*finals):
        assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64))
        assert np.array_equal(s1.members, s2.members)
    check_state(finals[0][0])

    def broken(edit):
        sb = StateBuffers.from_snapshot(mid[0])
        edit(sb)
        return sb

    na = mid[0].na
    first = int(mid[0].members[0])
    other = int(mid[0].members[mid[0].n_spheres[0]])  # first member of aggregate 1
    cases = [
        (lambda sb: sb.sphere_label.__setitem__(3, na), "sphere label out of range"),
        (lambda sb: sb.n_spheres.__setitem__(0, 0), "bad sphere count"),
        (lambda sb: sb.n_spheres.__setitem__(1, sb.n_spheres[1] + 1), "cover every sphere"),
        (lambda sb: sb.members.__setitem__(0, -7), "inconsistent"),
        (lambda sb: sb.members.__setitem__(0, other), "inconsistent"),
    ]
    assert first != other
    for edit, what in cases:
        with pytest.raises(MCACError, match=what):
            Batch(models[:1], states=[broken(edit)])


@pytest.mark.gpu
def test_split_by_aggregate_count_keeps_trajectories():
    """A run stopped at an intermediate aggregate count and resumed under the
    final criterion (mcacg_batch_set_aggregate_limit, the two windows of the
    ensemble benchmark) is the uninterrupted run, bit for bit."""
    models = [PhysicalModel(text=small_ini(n, 120 + k, mode="lognormal", disp=1.25, fv=4e-3, nagg=8))
              for k, n in enumerate([260, 540, 390, 700])]
    with Batch(models) as b:
        b.run(max_steps=0, steps_per_launch=5000)
        ref = b.store_all()
        ref_st = b.stats()
    staged = [PhysicalModel(text=small_ini(n, 120 + k, mode="lognormal", disp=1.25, fv=4e-3, nagg=40))
              for k, n in enumerate([260, 540, 390, 700])]
    with Batch(staged) as b:
        b.run(max_steps=0, steps_per_launch=5000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["n_aggregates"] <= 40)
        assert np.all(st["steps"] < ref_st["steps"])
        b.set_aggregate_limit(8)
        b.run(max_steps=0, steps_per_launch=5000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        assert np.array_equal(st["steps"], ref_st["steps"])
        for s1, s2 in zip(b.store_all(), ref):
            assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64))
            assert np.array_equal(s1.aggregates.view(np.int64), s2.aggregates.view(np.int64))
            assert np.array_equal(s1.members, s2.members)
        # a limit the boxes already meet leaves them where they are
        b.set_aggregate_limit(100)
        b.run(max_steps=0, steps_per_launch=5000)
        assert np.array_equal(b.stats()["steps"], ref_st["steps"])


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [32, 128])
def test_speculative_rounds_give_the_same_runs(threads):
    """Boxes advanced by clusters of 2, 4 or 8 thread blocks (that many
    steps' queries per round, committed in order up to the first conflict or
    merge) end bit for bit where the one-block loop ends, with the same step
    counts: sparse boxes (long runs without an event), dense ones (frequent
    merges and conflicts) and a larger one, to a stop criterion, in launches
    of a fixed step count and in time-capped launches."""
    specs = [(300, 5e-3, 10), (900, 2e-4, 40), (600, 1e-3, 20), (2500, 2e-3, 150)]
    models = [PhysicalModel(text=small_ini(n, 150 + k, mode=("lognormal" if k % 2 else "normal"), disp=1.3, fv=fv,
                                           nagg=nagg))
              for k, (n, fv, nagg) in enumerate(specs)]

    def run(k, mode):
        with Batch(models) as b:
            b.threads = threads
            b.speculation = k
            if mode == "criterion":
                b.run(max_steps=0, steps_per_launch=20000)
            elif mode == "steps":
                b.run(max_steps=3001, steps_per_launch=700)
            else:
                for _ in range(100000):
                    b.run_timed(2.0)
                    if np.all(b.stats()["finished"] == 1):
                        break
            assert b.speculation == k
            st = b.stats()
            assert np.all(st["status"] == 0)
            return st, b.store_all()

    for mode in ("criterion", "steps", "timed"):
        ref_st, ref = run(1, mode)
        for k in (2, 4, 8):
            st, snaps = run(k, mode)
            assert np.array_equal(st["steps"], ref_st["steps"]), (mode, k)
            assert np.array_equal(st["events"], ref_st["events"]), (mode, k)
            assert np.array_equal(st["time"].view(np.int64), ref_st["time"].view(np.int64)), (mode, k)
            for s1, s2 in zip(snaps, ref):
                assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64)), (mode, k)
                assert np.array_equal(s1.aggregates.view(np.int64), s2.aggregates.view(np.int64)), (mode, k)
                assert np.array_equal(s1.members, s2.members), (mode, k)


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [32, 256])
def test_live_list_gives_the_same_runs(threads):
    """Once few aggregates are left the loop picks from, and finds
    neighbours through, a list of the live aggregates in shared memory
    (mcacg_set_live_list_max); the runs are those of the tree and the Verlet
    cells, bit for bit, down to one aggregate."""
    from mcac_gb300.api import set_live_list_max
    specs = [(400, 5e-3), (700, 1e-3), (1500, 3e-3)]
    models = [PhysicalModel(text=small_ini(n, 170 + k, mode=("lognormal" if k % 2 else "normal"), disp=1.3, fv=fv,
                                           nagg=1, wait=20000))
              for k, (n, fv) in enumerate(specs)]
    runs = {}
    for live in (0, 128, 40):
        prev = set_live_list_max(live)
        try:
            with Batch(models) as b:
                b.threads = threads
                b.run(max_steps=0, steps_per_launch=20000)
                st = b.stats()
                assert np.all(st["status"] == 0) and np.all(st["finished"] == 1)
                runs[live] = (st, b.store_all())
        finally:
            set_live_list_max(prev)
    ref_st, ref = runs[0]
    for live in (128, 40):
        st, snaps = runs[live]
        assert np.array_equal(st["steps"], ref_st["steps"]), live
        assert np.array_equal(st["time"].view(np.int64), ref_st["time"].view(np.int64)), live
        for s1, s2 in zip(snaps, ref):
            assert np.array_equal(s1.spheres.view(np.int64), s2.spheres.view(np.int64)), live
            assert np.array_equal(s1.aggregates.view(np.int64), s2.aggregates.view(np.int64)), live
            assert np.array_equal(s1.members, s2.members), live
