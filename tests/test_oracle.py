"""The oracle (C restatement, oracle/mcac_oracle.c) pinned to the reference.

The golden vectors were produced by the reference compiled from its own
sources; these tests run on the CPU only.
"""
import hashlib
import shutil
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300.snapshot import Snapshot
from oracle import oracle_py as O


def digest(snap):
    h = hashlib.sha256()
    for arr in (snap.spheres, snap.sphere_label, snap.aggregates, snap.n_spheres, snap.members):
        h.update(np.ascontiguousarray(arr).tobytes())
    h.update(np.array([snap.maxradius, snap.box_length], dtype=np.float64).tobytes())
    return h.hexdigest()


def test_oracle_initial_state_and_full_run():
    g = load_golden("c1_trace.npz")
    box = O.OracleBox(str(g["ini"]))
    ref = Snapshot.from_npz(g, "init_")
    s = box.store()
    np.testing.assert_array_equal(s.spheres, ref.spheres)
    np.testing.assert_array_equal(s.aggregates, ref.aggregates)
    st, tr = box.calcul(trace=True, trace_capacity=len(g["t_picked"]) + 1)
    assert st.steps == len(g["t_picked"])
    np.testing.assert_array_equal(tr["picked"], g["t_picked"])
    np.testing.assert_array_equal(tr["merged"], g["t_merged"])
    np.testing.assert_array_equal(tr["other_sphere"], g["t_other_sphere"])
    np.testing.assert_array_equal(tr["contact_distance"].view(np.int64), g["t_contact_distance"].view(np.int64))
    np.testing.assert_array_equal(tr["time_after"].view(np.int64), g["t_time_after"].view(np.int64))
    assert digest(box.store()) == str(g["final_digest"])


@pytest.mark.parametrize("case", ["collective", "individual", "partial"])
def test_oracle_surface_growth_runs(case):
    """Surface growth (every aggregate, the moved one only, update_partial
    between full updates): the reference's own runs' final states, byte for
    byte (tests/golden/make_growth_exact_golden.py)."""
    g = load_golden("growth_exact.npz")
    box = O.OracleBox(str(g[f"{case}_ini"]))
    st, _ = box.calcul()
    assert st.n_aggregates == int(g[f"{case}_na"])
    assert st.time == float(g[f"{case}_time"])
    assert digest(box.store()) == str(g[f"{case}_digest"])


@pytest.mark.parametrize("mode", ["coll", "ind"])
@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_oracle_oxidation_runs(mode, k):
    """Oxidation from states the reference grew (spheres shrink, those at or
    below rp_min leave, empty aggregates disappear, disconnected ones split;
    every aggregate at every step, or the moved one): the reference's own
    runs' final states, byte for byte (tests/golden/make_oxidation_golden.py).
    The reference's harness placed one monomer before loading the state, four
    draws of the seeded stream."""
    import ctypes

    from test_oxidation_gpu import oxidation_ini
    g = load_golden("oxidation.npz")
    start = Snapshot.from_npz(g, f"start_{k}_")
    text = oxidation_ini(900 + k, start.time + float(g["ind_dt"]), float(g["ind_rp_min"]), mode == "ind",
                         float(g["flux"]))
    libc = ctypes.CDLL(None)
    libc.srand(900 + k)
    for _ in range(4):
        libc.rand()
    box = O.OracleBox(text, start)
    st, _ = box.calcul()
    out = box.store()
    assert (out.na, out.ns) == (int(g[f"exact_{mode}_{k}_na"]), int(g[f"exact_{mode}_{k}_ns"]))
    assert st.time == float(g[f"exact_{mode}_{k}_time"])
    assert digest(out) == str(g[f"exact_{mode}_{k}_digest"])


def test_oracle_lognormal_run_final_state():
    g = load_golden("ln_late.npz")
    box = O.OracleBox(str(g["ini"]))
    st, tr = box.calcul(trace=True, trace_capacity=int(g["run_steps"]) + 1)
    assert st.steps == int(g["run_steps"]) and st.events == int(g["run_events"])
    np.testing.assert_array_equal(np.flatnonzero(tr["merged"]), g["merge_steps"])
    assert digest(box.store()) == str(g["final_digest"])


@pytest.mark.parametrize("fixture", ["c1_q5000.npz", "ln_late.npz"])
def test_oracle_queries_and_merges(fixture):
    g = load_golden(fixture)
    snap = Snapshot.from_npz(g, "s_")
    box = O.OracleBox(str(g["ini"]), snap)
    for k in range(len(g["q_label"])):
        c = box.distance_to_next_contact(g["q_label"][k], g["q_dir"][k], g["q_distance"][k])
        assert np.float64(c.distance).view(np.int64) == np.float64(g["q_contact_distance"][k]).view(np.int64)
        assert (c.moving_sphere, c.other_sphere, c.other_aggregate) == (
            g["q_moving_sphere"][k], g["q_other_sphere"][k], g["q_other_agg"][k])
    for r, q in enumerate(g["m_index"][:40]):
        b2 = O.OracleBox(str(g["ini"]), snap)
        c = b2.distance_to_next_contact(g["q_label"][q], g["q_dir"][q], g["q_distance"][q])
        b2.translate(g["q_label"][q], np.asarray(g["q_dir"][q]) * c.distance)
        assert b2.merge(c)
        s = b2.store()
        keep = int(g["m_keep"][r])
        np.testing.assert_array_equal(s.aggregates[:, keep].view(np.int64), g["m_record"][r].view(np.int64))
        assert s.maxradius == g["m_maxradius"][r]


SORT_CPP = r"""
#include <algorithm>
#include <cstdio>
#include <numeric>
#include <vector>
int main() {
    size_t n;
    if (std::fread(&n, sizeof n, 1, stdin) != 1) return 1;
    std::vector<double> v(n);
    if (std::fread(v.data(), sizeof(double), n, stdin) != n) return 1;
    std::vector<size_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&v](size_t a, size_t b) { return v[a] < v[b]; });
    std::fwrite(idx.data(), sizeof(size_t), n, stdout);
    return 0;
}
"""


@pytest.fixture(scope="module")
def std_sort_binary(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("stdsort")
    (d / "s.cpp").write_text(SORT_CPP)
    subprocess.run(["g++", "-O2", "-o", str(d / "s"), str(d / "s.cpp")], check=True)
    return d / "s"


@pytest.mark.parametrize("case", ["ties", "few_values", "random", "sorted", "reversed", "organ", "small"])
def test_sort_order_matches_libstdcxx(std_sort_binary, case):
    rng = np.random.default_rng(hash(case) % 2**32)
    n = {"small": 13}.get(case, 5000)
    keys = {
        "ties": np.full(n, 0.5),
        "few_values": rng.integers(0, 4, n).astype(float),
        "random": rng.random(n),
        "sorted": np.arange(n, dtype=float),
        "reversed": np.arange(n, 0, -1, dtype=float),
        "organ": np.concatenate([np.arange(n // 2), np.arange(n - n // 2, 0, -1)]).astype(float),
        "small": rng.integers(0, 3, n).astype(float),
    }[case]
    payload = np.array([n], dtype=np.uint64).tobytes() + keys.astype(np.float64).tobytes()
    out = subprocess.run([str(std_sort_binary)], input=payload, capture_output=True, check=True).stdout
    expect = np.frombuffer(out, dtype=np.uint64).astype(np.int64)
    np.testing.assert_array_equal(O.sort_indices(keys), expect)
