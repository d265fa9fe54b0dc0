"""Surface growth in the device loop, against the reference's own runs.

With ``with_surface_reactions`` every sphere of a box grows by u_sg dt at
every step and every aggregate is updated (src/calcul.cpp:157-206). The
device loop does the same and follows the reference statistically (its pick
and directions differ in order, as without growth). Checked: every sphere
gained exactly u_sg times the box's physical time, the aggregate fields equal
their definitions over the grown spheres, and 32 seeded boxes match the
reference binary's own runs (tests/golden/growth_ensemble.npz, made by
tests/golden/make_growth_golden.py) in time to 15 aggregates, mean sphere
radius, fractal law and mean aggregate size.
"""
import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import Batch, PhysicalModel
from mcac_gb300.snapshot import A, S
from test_device_loop_gpu import seq_sum


def growth_ini(seed: int) -> str:
    return (f"[monomers]\nnumber = 300\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 5e-3\ntemperature = 1700\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = 0.5\n"
            f"[limits]\nnumber_of_aggregates = 15\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n")


def fractal_fit(npp, dgdp):
    keep = npp >= 3
    slope, icpt = np.polyfit(np.log(dgdp[keep]), np.log(npp[keep]), 1)
    return slope, np.exp(icpt)


@pytest.mark.gpu
def test_spheres_grow_by_u_sg_times_time_and_fields_follow():
    models = [PhysicalModel(text=growth_ini(600 + k)) for k in range(4)]
    with Batch(models) as b:
        before = b.store_all()
        b.run(max_steps=0, steps_per_launch=5000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        after = b.store_all()
    for k, m in enumerate(models):
        u = m.params.u_sg
        grown = after[k].spheres[S["r"]] - before[k].spheres[S["r"]]
        dt_total = after[k].time - before[k].time
        np.testing.assert_allclose(grown, u * dt_total, rtol=1e-6)
        snap = after[k]
        off = snap.member_offsets()
        for a in range(snap.na):
            mem = snap.members[off[a]:off[a + 1]]
            r = snap.spheres[S["r"], mem]
            np.testing.assert_allclose(snap.spheres[S["volume"], mem], 4 * np.pi / 3 * r ** 3, rtol=1e-14)
            assert snap.aggregates[A["volume"], a] == seq_sum(snap.spheres[S["volume"], mem])
            assert snap.aggregates[A["surface"], a] == seq_sum(snap.spheres[S["surface"], mem])
            np.testing.assert_allclose(snap.aggregates[A["dp"], a], 2 * r.mean(), rtol=1e-12)
        assert snap.maxradius >= snap.aggregates[A["rmax"]].max()


@pytest.mark.gpu
def test_growth_ensemble_matches_reference():
    g = load_golden("growth_ensemble.npz")
    seeds = g["seeds"]
    with Batch([PhysicalModel(text=growth_ini(int(s))) for s in seeds]) as b:
        b.run(max_steps=0, steps_per_launch=10000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        snaps = b.store_all()
    t_gpu = np.array([s.time for s in snaps])
    r_gpu = np.array([s.spheres[S["r"]].mean() for s in snaps])
    npp_gpu = np.concatenate([s.n_spheres for s in snaps])
    dg_gpu = np.concatenate([s.aggregates[A["dg_over_dp"]] for s in snaps])

    def close(a, b_, k=4.0):
        se = np.sqrt(a.var(ddof=1) / len(a) + b_.var(ddof=1) / len(b_))
        return abs(a.mean() - b_.mean()) <= k * se

    assert close(np.log(t_gpu), np.log(g["time"])), (t_gpu.mean(), g["time"].mean())
    assert close(r_gpu, g["mean_r"]), (r_gpu.mean(), g["mean_r"].mean())
    dg, kg = fractal_fit(npp_gpu, dg_gpu)
    dr, kr = fractal_fit(g["npp"], g["dg_over_dp"])
    assert abs(dg - dr) < 0.15, (dg, dr)
    assert abs(np.log(kg / kr)) < 0.3, (kg, kr)
    assert abs(npp_gpu.mean() / g["npp"].mean() - 1) < 0.1


@pytest.mark.gpu
def test_individual_growth_matches_reference():
    """individual_surf_reactions: only the moved aggregate grows, by its own
    time step, and only it is updated unless a merge happened
    (calcul.cpp:108, 148, 159-166, 185-201); 32 boxes against the
    reference binary's runs (tests/golden/growth_individual.npz)."""
    g = load_golden("growth_individual.npz")
    ini = str(g["ini"])
    models = [PhysicalModel(text=ini.replace("random_seed = 0", f"random_seed = {int(s)}")) for s in g["seeds"]]
    with Batch(models) as b:
        before = b.store_all()
        b.run(max_steps=0, steps_per_launch=10000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        snaps = b.store_all()
    # the spheres of different aggregates grew by different amounts (each by
    # its aggregates' own time steps, about the box's time on average)
    u = models[0].params.u_sg
    ratio = []
    for s0, s1 in zip(before, snaps):
        grown = s1.spheres[S["r"]] - s0.spheres[S["r"]]
        assert np.all(grown >= 0) and grown.std() > 0
        ratio.append(grown.mean() / (u * (s1.time - s0.time)))
    assert 0.5 < np.mean(ratio) < 2.0, np.mean(ratio)
    t_gpu = np.array([s.time for s in snaps])
    r_gpu = np.array([s.spheres[S["r"]].mean() for s in snaps])
    npp_gpu = np.concatenate([s.n_spheres for s in snaps])
    dg_gpu = np.concatenate([s.aggregates[A["dg_over_dp"]] for s in snaps])

    def close(a, b_, k=4.0):
        se = np.sqrt(a.var(ddof=1) / len(a) + b_.var(ddof=1) / len(b_))
        return abs(a.mean() - b_.mean()) <= k * se

    assert close(np.log(t_gpu), np.log(g["time"])), (t_gpu.mean(), g["time"].mean())
    assert close(r_gpu, g["mean_r"]), (r_gpu.mean(), g["mean_r"].mean())
    dg, kg = fractal_fit(npp_gpu, dg_gpu)
    dr, kr = fractal_fit(g["npp"], g["dg_over_dp"])
    assert abs(dg - dr) < 0.15, (dg, dr)
    assert abs(npp_gpu.mean() / g["npp"].mean() - 1) < 0.1
