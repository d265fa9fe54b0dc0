"""The device loop against the reference on boxes of the benchmark ensemble.

tests/golden/ensemble64.npz holds what the reference's own mcac::calcul
(built from its sources, tests/golden/make_ensemble_golden.py) gives for 64
boxes of the 512-box ensemble (boxes 0, 8, ..., 504: 300 to 16 000
monomers, monodisperse and LogNormal(1.25), 100-5000 ppm, 1500-1900 K), each
run from its seeded placement until 20 aggregates are left. The device loop
runs the same boxes to the same criterion; its trajectories differ from the
reference's step by step (its pick walks a sum tree and its directions use
FP32 angles), so the distributions are compared:

* the aggregates' monomer counts and Rg/dp, pooled over the boxes
  (1280 aggregates a side): two-sample Kolmogorov-Smirnov, p > 1e-3;
* the physical time each box takes: two-sample KS over the 64 boxes and a
  Wilcoxon signed-rank test of the per-box log ratio, p > 1e-3;
* the fractal law N = k (2 Rg/dp)^D fitted over the aggregates of at least 3
  monomers (as the reference's validation notebook fits it): D and ln k
  within 4 standard errors of their difference, the standard error derived
  by bootstrap over the reference's boxes (500 resamples, fixed seed) and
  taken as sqrt(2) times it, the two samples being of the same size.

The seeds are fixed, so the outcome is deterministic.
"""
import numpy as np
import pytest

from mcac_gb300 import Batch, PhysicalModel
from mcac_gb300.snapshot import A

from conftest import load_golden

scipy_stats = pytest.importorskip("scipy.stats")


def fractal_fit(npp, dgdp):
    keep = npp >= 3
    slope, icpt = np.polyfit(np.log(dgdp[keep]), np.log(npp[keep]), 1)
    return slope, icpt


@pytest.mark.gpu
def test_ensemble_distributions_match_the_reference():
    import bench
    g = load_golden("ensemble64.npz")
    stop = int(g["stop_aggregates"])
    inis = bench.ensemble_inis(512)
    models = []
    for b in g["boxes"]:
        pm = PhysicalModel(text=inis[int(b)])
        pm.set(number_of_aggregates_limit=stop)
        models.append(pm)
    with Batch(models) as batch:
        batch.run(max_steps=0, steps_per_launch=50000)
        st = batch.stats()
        assert np.all(st["status"] == 0) and np.all(st["finished"] == 1)
        snaps = batch.store_all()
    npp = np.concatenate([s.n_spheres for s in snaps]).astype(np.float64)
    dgdp = np.concatenate([s.aggregates[A["dg_over_dp"]] for s in snaps])
    box = np.concatenate([np.full(s.na, k) for k, s in enumerate(snaps)])
    t_gpu = st["time"]
    # the same stop on both sides
    assert np.array_equal(st["n_aggregates"], g["n_aggregates"])
    ref_npp, ref_dgdp, ref_box = g["npp"].astype(np.float64), g["dg_over_dp"], g["box"]
    assert scipy_stats.ks_2samp(np.log(npp), np.log(ref_npp)).pvalue > 1e-3
    assert scipy_stats.ks_2samp(np.log(dgdp), np.log(ref_dgdp)).pvalue > 1e-3
    assert scipy_stats.ks_2samp(np.log(t_gpu), np.log(g["time"])).pvalue > 1e-3
    assert scipy_stats.wilcoxon(np.log(t_gpu / g["time"])).pvalue > 1e-3
    # fractal law, tolerance by bootstrap over the reference's boxes
    d_ref, c_ref = fractal_fit(ref_npp, ref_dgdp)
    d_gpu, c_gpu = fractal_fit(npp, dgdp)
    rng = np.random.default_rng(12345)
    boxes = np.unique(ref_box)
    fits = []
    for _ in range(500):
        pick = rng.choice(boxes, size=len(boxes), replace=True)
        idx = np.concatenate([np.flatnonzero(ref_box == b) for b in pick])
        fits.append(fractal_fit(ref_npp[idx], ref_dgdp[idx]))
    se = np.sqrt(2.0) * np.std(np.array(fits), axis=0, ddof=1)
    assert abs(d_gpu - d_ref) < 4.0 * se[0], (d_gpu, d_ref, se[0])
    assert abs(c_gpu - c_ref) < 4.0 * se[1], (c_gpu, c_ref, se[1])
    assert len(np.unique(box)) == len(snaps)
