"""The device loop's random draws against the reference's distributions.

The device-resident loop does not reproduce the reference's draws one for
one (its pick walks a fixed-point sum tree, its directions use FP32 angles),
so its pick and its directions are checked here against the distributions
the reference's code samples:

* AggregatList::pick_random (aggregat_list.cpp:59-66, 124-141) picks label
  i with probability (1/time_step_i) / sum_j (1/time_step_j): a chi-square
  test of 2^21 picks from the loop's own tree descent, on a polydisperse
  state after some merges and on a monodisperse initial state (all weights
  equal, the reference's tie case).
* random_direction (tools.cpp:82-89) is uniform on the unit sphere: 2^22
  directions from the loop's own draw have unit length to 1e-12, the
  sphere's first and second moments within 5 standard errors, and a
  uniform cos(polar angle) and azimuth (Kolmogorov-Smirnov).

The seeds are fixed, so each test's outcome is deterministic; the
thresholds (p > 1e-4, 5 standard errors) are the false-alarm rates a
correct sampler meets with probability about 1 - 1e-4 per check.
"""
import numpy as np
import pytest

from mcac_gb300 import Batch, PhysicalModel
from mcac_gb300.api import draw_directions
from mcac_gb300.snapshot import A

scipy_stats = pytest.importorskip("scipy.stats")


def box_ini(n, seed, disp, nagg=1):
    return (f"[monomers]\nnumber = {n}\nmean_diameter = 30\ndispersion_diameter = {disp}\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = 3e-3\ntemperature = 1700\n"
            f"[limits]\nnumber_of_aggregates = {nagg}\n"
            f"[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n")


def chi_square_p(counts, weights):
    expected = weights / weights.sum() * counts.sum()
    chi2 = float(((counts - expected) ** 2 / expected).sum())
    return float(scipy_stats.chi2.sf(chi2, len(counts) - 1)), chi2


@pytest.mark.gpu
@pytest.mark.parametrize("disp,steps", [(1.5, 3000), (1.0, 0)])
def test_pick_frequencies_follow_inverse_time_steps(disp, steps):
    with Batch([PhysicalModel(text=box_ini(1500, 31, disp))]) as b:
        if steps:
            b.run(max_steps=steps, steps_per_launch=steps)
        snap = b.store(0)
        counts, done = b.pick_histogram(0, 1 << 21, seed=7)
    assert len(counts) == snap.na and counts.sum() == done  # every pick lands on a live aggregate
    w = 1.0 / snap.aggregates[A["time_step"]]
    assert np.all(counts > 0)
    p, chi2 = chi_square_p(counts.astype(np.float64), w)
    assert p > 1e-4, (chi2, len(counts), p)
    if disp == 1.0:
        assert np.all(w == w[0])  # monodisperse: every weight equal, uniform picks


@pytest.mark.gpu
def test_directions_are_isotropic():
    n = 1 << 22
    d = draw_directions(n, seed=11)
    assert np.all(np.abs(np.sqrt((d * d).sum(1)) - 1.0) < 1e-12)
    m = d.mean(0)
    assert np.all(np.abs(m) < 5.0 * np.sqrt(1.0 / 3.0 / n)), m
    # second moments of the uniform sphere: E[x^2] = 1/3 (variance of x^2:
    # 4/45), E[xy] = 0 (variance 1/15)
    sq = (d * d).mean(0)
    assert np.all(np.abs(sq - 1.0 / 3.0) < 5.0 * np.sqrt(4.0 / 45.0 / n)), sq
    for i, j in ((0, 1), (0, 2), (1, 2)):
        assert abs((d[:, i] * d[:, j]).mean()) < 5.0 * np.sqrt(1.0 / 15.0 / n)
    # cos(polar angle) = z uniform on [-1, 1]; azimuth uniform on [-pi, pi]
    assert scipy_stats.kstest(d[:, 2], "uniform", args=(-1.0, 2.0)).pvalue > 1e-4
    phi = np.arctan2(d[:, 1], d[:, 0])
    assert scipy_stats.kstest(phi, "uniform", args=(-np.pi, 2.0 * np.pi)).pvalue > 1e-4
