"""Surface growth in the host-driven loop, step by step against the oracle.

With ``with_surface_reactions`` and a positive flux every sphere grows at every step
(or those of the moved aggregate, individual_surf_reactions) and the
aggregates are updated, fully or with update_partial (src/calcul.cpp:157-206).
The host-driven loop grows the spheres and recomputes the geometry on the
GPU and the physics fields on the host; the oracle does the same in C and is
pinned to the reference's own runs of these INIs (tests/test_oracle.py,
tests/golden/growth_exact.npz). Every MC step must pick the same aggregate,
find the same contact and merge the same pair, and the final state must be
identical byte for byte.
"""
import pytest

from conftest import load_golden
from test_calcul_gpu import compare_runs


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["collective", "individual", "partial"])
def test_growth_run_matches_oracle_step_by_step(case):
    g = load_golden("growth_exact.npz")
    st = compare_runs(str(g[f"{case}_ini"]))
    assert st.n_aggregates == int(g[f"{case}_na"])
