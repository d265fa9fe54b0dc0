"""Overlap-corrected volume and surface ("caps", "alphas") with surface growth.

Aggregate::compute_volume_surface (src/aggregats/aggregat.cpp:321-430) takes
the spherical caps of every contact off each sphere ("caps") or corrects the
plain sums by the contact statistics ("alphas"); update_partial then weighs
the centre of mass and Rg with the per-sphere volumes of the last full update
(aggregat.cpp:431-483). The device loop does the same at merges and at full
updates. Checked: (1) with a full update every step, every final aggregate's
volume, surface, overlap and coordination equal the reference formulas
applied to the final spheres (the reference visits a sphere's contacts in its
hash map's order, this library by index: the same terms, summed in another
order, so to 1e-12); (2) 32 seeded boxes of the reference's own
surface-growth validation case match the reference binary's runs
(tests/golden/volsurf_*.npz, made by tests/golden/make_volsurf_golden.py) in
time, sphere radius, aggregate sizes, fractal law and the volume and surface
corrections.
"""
import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import Batch, PhysicalModel
from mcac_gb300.snapshot import A, S
from test_growth_gpu import fractal_fit

EPS = 1e-10


def growth_ini(method: str, seed: int, flux: float = 0.5) -> str:
    return (f"[monomers]\nnumber = 300\nmean_diameter = 30\ndispersion_diameter = 1.25\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 5e-3\ntemperature = 1700\n"
            f"[surface_growth]\nwith_surface_reactions = true\nflux_surfgrowth = {flux}\n"
            f"volsurf_method = {method}\nfull_aggregate_update_frequency = 1\n"
            f"[limits]\nnumber_of_aggregates = 15\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n")


def caps(r1, v1, s1, r2, v2, s2, d):
    """Intersection (src/spheres/sphere_intersection.cpp:29-66)."""
    if d <= 0 or not d < r1 + r2:
        return 0.0, 0.0, 0.0, 0.0
    if d >= max(r1 - r2, 0.0):
        h1 = (r2 * r2 - (r1 - d) ** 2) / (2.0 * d)
        h2 = (r1 * r1 - (r2 - d) ** 2) / (2.0 * d)
        return (np.pi * h1 * h1 * (3 * r1 - h1) / 3.0, np.pi * h2 * h2 * (3 * r2 - h2) / 3.0,
                2 * np.pi * r1 * h1, 2 * np.pi * r2 * h2)
    return (v1, 0.0, s1, 0.0) if r1 < r2 else (0.0, v2, 0.0, s2)


def volume_surface(snap, a, method):
    """compute_volume_surface of one aggregate from its spheres."""
    off = snap.member_offsets()
    mem = snap.members[off[a]:off[a + 1]]
    n = len(mem)
    r = snap.spheres[S["r"], mem]
    vol = snap.spheres[S["volume"], mem].copy()
    sur = snap.spheres[S["surface"], mem].copy()
    rel = snap.spheres[[S["rx"], S["ry"], S["rz"]]][:, mem].T
    pairs = []
    for i in range(n):
        d = np.sqrt(((rel[i] - rel[i + 1:]) ** 2).sum(1))
        for k in np.nonzero(d <= (1 + EPS) * (r[i] + r[i + 1:]))[0]:
            pairs.append((i, i + 1 + int(k), float(d[k])))
    ov = sum(2 * (r[i] + r[j] - d) / (r[i] + r[j]) for i, j, d in pairs)
    inter = 2 * len(pairs)
    overlap = ov / inter if inter else 0.0
    coord = inter / n if inter else 0.0
    v0, s0 = snap.spheres[S["volume"], mem], snap.spheres[S["surface"], mem]
    if method == "caps":
        for i, j, d in pairs:
            c = caps(r[i], v0[i], s0[i], r[j], v0[j], s0[j], d)
            vol[i] -= c[0]
            sur[i] -= c[2]
            vol[j] -= c[1]
            sur[j] -= c[3]
        vol, sur = np.maximum(vol, 0), np.maximum(sur, 0)
    V, Sf = float(np.sum(vol)), float(np.sum(sur))
    if method == "alphas" and pairs:
        c_ij = np.array([(r[i] + r[j] - d) / (r[i] + r[j]) for i, j, d in pairs])
        vp = np.array([r[i] ** 3 + r[j] ** 3 for i, j, _ in pairs])
        sp = np.array([r[i] ** 2 + r[j] ** 2 for i, j, _ in pairs])
        c10 = 2 * np.sum(c_ij * sp) / (2 * np.sum(sp))
        c20 = 2 * np.sum(c_ij ** 2 * vp) / (2 * np.sum(vp))
        c30 = 2 * np.sum(c_ij ** 3 * vp) / (2 * np.sum(vp))
        overlap = 2 * np.sum(c_ij) / inter
        cn_min = 2 * (1 - 1 / n)
        dc = abs(coord - cn_min)
        corr_v = 0.25 * (3 * c20 - c30) * coord - c30 * dc * 0.62741833 - dc ** 1.5 * 0.00332425
        corr_s = 0.5 * c10 * coord - c10 ** 2 * dc * 0.701325 - dc ** 2 * 0.0045
        corr_v = 1.0 if corr_v < 0 else min(corr_v, 1.0)
        corr_s = 1.0 if corr_s < 0 else min(corr_s, 1.0)
        V *= max(1 - corr_v, 1 / n)
        Sf *= max(1 - corr_s, 1 / n)
    return V, Sf, overlap, coord, len(pairs)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["alphas", "caps"])
def test_corrected_fields_follow_their_definitions(method):
    models = [PhysicalModel(text=growth_ini(method, 640 + k)) for k in range(3)]
    with Batch(models) as b:
        b.run(max_steps=0, steps_per_launch=5000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        snaps = b.store_all()
    n_pairs = 0
    for snap in snaps:
        for a in range(snap.na):
            V, Sf, ov, co, npairs = volume_surface(snap, a, method)
            n_pairs += npairs
            np.testing.assert_allclose(snap.aggregates[A["volume"], a], V, rtol=1e-12)
            np.testing.assert_allclose(snap.aggregates[A["surface"], a], Sf, rtol=1e-12)
            np.testing.assert_allclose(snap.aggregates[A["overlapping"], a], ov, rtol=1e-9, atol=1e-15)
            assert snap.aggregates[A["coordination_number"], a] == pytest.approx(co, rel=1e-15)
    assert n_pairs > 100  # the boxes hold many overlapping contacts


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["alphas", "caps"])
def test_validation_case_matches_reference(method):
    g = load_golden(f"volsurf_{method}.npz")
    ini = str(g["ini"])
    models = [PhysicalModel(text=ini.replace("random_seed = 0", f"random_seed = {int(s)}")) for s in g["seeds"]]
    with Batch(models) as b:
        b.run(max_steps=0, steps_per_launch=20000)
        st = b.stats()
        assert np.all(st["finished"] == 1) and np.all(st["status"] == 0)
        snaps = b.store_all()
    t = np.array([s.time for s in snaps])
    r = np.array([s.spheres[S["r"]].mean() for s in snaps])
    npp = np.concatenate([s.n_spheres for s in snaps])
    dg = np.concatenate([s.aggregates[A["dg_over_dp"]] for s in snaps])
    # the corrections per box (the aggregates of one box share its history,
    # so boxes are the independent samples)
    vr, sr = [], []
    for s in snaps:
        off = s.member_offsets()
        v, w = [], []
        for a in range(s.na):
            mem = s.members[off[a]:off[a + 1]]
            v.append(s.aggregates[A["volume"], a] / s.spheres[S["volume"], mem].sum())
            w.append(s.aggregates[A["surface"], a] / s.spheres[S["surface"], mem].sum())
        vr.append(np.mean(v))
        sr.append(np.mean(w))
    vr, sr = np.array(vr), np.array(sr)
    nb = len(g["seeds"])
    ref_vr = np.array([g["vol_ratio"][g["box"] == k].mean() for k in range(nb)])
    ref_sr = np.array([g["surf_ratio"][g["box"] == k].mean() for k in range(nb)])

    def close(x, y, k=4.0):
        se = np.sqrt(x.var(ddof=1) / len(x) + y.var(ddof=1) / len(y))
        return abs(x.mean() - y.mean()) <= k * se + 1e-12 * abs(y.mean())

    assert close(np.log(t), np.log(g["time"])), (t.mean(), g["time"].mean())
    assert close(r, g["mean_r"]), (r.mean(), g["mean_r"].mean())
    assert close(vr, ref_vr), (vr.mean(), ref_vr.mean())
    assert close(sr, ref_sr), (sr.mean(), ref_sr.mean())
    dfit, kfit = fractal_fit(npp, dg)
    dref, kref = fractal_fit(g["npp"], g["dg_over_dp"])
    assert abs(dfit - dref) < 0.2, (dfit, dref)
    assert abs(npp.mean() / g["npp"].mean() - 1) < 0.1
