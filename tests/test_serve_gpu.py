"""Continuous batching (Server): admission by slot and memory, completion,
and the same result for a request alone and in a mix."""
import numpy as np
import pytest

from mcac_gb300 import Batch, PhysicalModel, Server


def req_ini(n, seed, fv=4e-3, nagg=3, disp=1.3):
    return (f"[monomers]\nnumber = {n}\nmean_diameter = 30\ndispersion_diameter = {disp}\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = {fv}\ntemperature = 1700\n"
            f"[limits]\nnumber_of_aggregates = {nagg}\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n")


def same_state(a, b):
    return (np.array_equal(a.spheres.view(np.int64), b.spheres.view(np.int64))
            and np.array_equal(a.aggregates.view(np.int64), b.aggregates.view(np.int64))
            and np.array_equal(a.members, b.members) and np.array_equal(a.sphere_label, b.sphere_label))


@pytest.mark.gpu
def test_requests_admitted_as_slots_free_and_match_alone():
    sizes = [200, 450, 300, 700, 250, 600, 350, 500, 220, 650]
    models = [PhysicalModel(text=req_ini(n, 900 + k)) for k, n in enumerate(sizes)]
    done = {}
    max_active = 0
    with Server(capacity=4, keep_final_states=True) as srv:
        ids = [srv.submit(m) for m in models[:6]]
        for epoch in range(10_000):
            if epoch == 3:
                ids += [srv.submit(m) for m in models[6:]]  # arrivals while others run
            active, pending = srv.step(800)
            max_active = max(max_active, active)
            for c in srv.poll():
                done[int(c["id"])] = c
            if len(done) == len(models) and active == 0 and pending == 0:
                break
        assert len(done) == len(models)
        assert max_active <= 4
        for rid in ids:
            c = done[rid]
            assert c["status"] == 0 and c["finished"] == 1 and c["n_aggregates"] <= 3
            assert c["submit_s"] <= c["admit_s"] <= c["finish_s"]
        finals = {rid: srv.final_state(rid) for rid in ids[:3] + ids[-2:]}
    # the same requests alone
    for k, rid in enumerate(ids[:3] + ids[-2:]):
        idx = ids.index(rid)
        with Batch([models[idx]]) as b:
            b.run(max_steps=0, steps_per_launch=5000)
            alone = b.store(0)
            assert int(b.stats()["steps"][0]) == int(done[rid]["steps"])
        assert same_state(alone, finals[rid]), rid


@pytest.mark.gpu
def test_memory_budget_limits_concurrency():
    models = [PhysicalModel(text=req_ini(300, 50 + k)) for k in range(4)]
    # the server's footprint model for one box (fine grid at its 128^3 bound)
    one_box = 300 * 760 + 1000 * 4 * 80 + 128 ** 3 * 4 + (3 << 20)
    with Server(capacity=4, memory_budget=int(one_box * 1.5)) as srv:
        for m in models:
            srv.submit(m)
        seen, max_active = 0, 0
        for _ in range(10_000):
            active, pending = srv.step(1000)
            max_active = max(max_active, active)
            seen += len(srv.poll())
            if seen == 4 and pending == 0 and active == 0:
                break
        assert seen == 4 and max_active <= 1


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [64, 0])
def test_time_capped_epochs_give_the_same_runs(threads):
    """Epochs cut by wall time (each box does as many steps as fit) change
    how far a box gets per epoch, never its trajectory; nor does the block
    size, fixed or chosen at each epoch by the number of active runs (0)."""
    models = [PhysicalModel(text=req_ini(n, 950 + k)) for k, n in enumerate([260, 520, 380])]
    done = {}
    with Server(capacity=2, keep_final_states=True) as srv:
        srv.set_epoch_ms(2.0)
        srv.set_threads(threads)
        ids = [srv.submit(m) for m in models]
        for _ in range(100_000):
            active, pending = srv.step(1_000_000)
            for c in srv.poll():
                done[int(c["id"])] = c
            if len(done) == len(models) and active == 0 and pending == 0:
                break
        finals = {rid: srv.final_state(rid) for rid in ids}
    for k, rid in enumerate(ids):
        with Batch([models[k]]) as b:
            b.run(max_steps=0, steps_per_launch=5000)
            assert int(b.stats()["steps"][0]) == int(done[rid]["steps"])
            assert same_state(b.store(0), finals[rid])


@pytest.mark.gpu
def test_oxidising_requests_served_match_alone():
    """Requests that oxidise (spheres shrink and leave; one box loses every
    sphere) beside collision-only ones: each served run ends as it does alone."""
    ox = ("[monomers]\nnumber = {n}\nmean_diameter = 30\ndispersion_diameter = {disp}\n"
          "initialisation_mode = lognormal\n[environment]\nvolume_fraction = 3e-3\ntemperature = 1700\n"
          "[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = -0.5\n"
          "[oxidation]\nrp_min = {rp}\n[limits]\nnumber_of_aggregates = 0\nphysical_time = {tl}\n"
          "[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n")
    models = [PhysicalModel(text=ox.format(n=250, disp=1.0, rp=1e-8, tl=1.0, seed=71)),
              PhysicalModel(text=ox.format(n=400, disp=1.25, rp=1.2e-8, tl=1e-5, seed=72)),
              PhysicalModel(text=req_ini(300, 73)), PhysicalModel(text=req_ini(350, 74))]
    done = {}
    with Server(capacity=2, keep_final_states=True) as srv:
        ids = [srv.submit(m) for m in models]
        for _ in range(10_000):
            active, pending = srv.step(2000)
            for c in srv.poll():
                done[int(c["id"])] = c
            if len(done) == len(models) and active == 0 and pending == 0:
                break
        assert len(done) == len(models)
        finals = [srv.final_state(rid) for rid in ids]
    for rid in ids:
        assert done[rid]["status"] == 0 and done[rid]["finished"] == 1
    assert finals[0].ns == 0 and finals[0].na == 0  # every sphere of the monodisperse box went
    assert 0 < finals[1].ns < 400
    for k, m in enumerate(models):
        with Batch([m]) as b:
            b.run(max_steps=0, steps_per_launch=5000)
            alone = b.store(0)
        assert alone.ns == finals[k].ns and alone.na == finals[k].na
        assert same_state(alone, finals[k]), k
