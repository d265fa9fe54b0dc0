"""distance_to_next_contact and merge on the GPU against the reference.

Each fixture holds a state produced by the reference binary, seeded queries
(source label, direction from the reference's random_direction, distance =
the source's lpm) and the reference's answers. The bar is bit equality:
same contact spheres, same aggregate, same FP64 distance bits (stronger than
the 1e-9 relative tolerance the benchmark asks for). The contact search and
the merge geometry use only +, -, *, /, sqrt, fmod and floor, so their
results do not depend on the machine; the physics fields of a merged
aggregate go through libm (erf, exp, pow) and are compared with the oracle
run on the same machine, and with the reference within 4 ulp.
"""
import numpy as np
import pytest

from conftest import load_golden
from mcac_gb300 import AggregatList, PhysicalModel
from mcac_gb300.snapshot import A, Snapshot
from oracle import oracle_py as O

LIBM_FIELDS = [A["f_agg"], A["lpm"], A["time_step"], A["d_m"]]
GEOMETRY_FIELDS = [f for f in range(21) if f not in LIBM_FIELDS]

FIXTURES = ["c1_q5000.npz", "ln_late.npz"]


def same_double(a: float, b: float) -> bool:
    return np.float64(a).view(np.int64) == np.float64(b).view(np.int64)


@pytest.mark.gpu
@pytest.mark.parametrize("fixture", FIXTURES)
def test_queries_match_reference_bitwise(fixture):
    g = load_golden(fixture)
    snap = Snapshot.from_npz(g, "s_")
    pm = PhysicalModel(text=str(g["ini"]))
    with AggregatList(pm, snap) as box:
        bad = []
        for k in range(len(g["q_label"])):
            info = box.distance_to_next_contact(int(g["q_label"][k]), g["q_dir"][k], float(g["q_distance"][k]))
            ok = (same_double(info.distance, g["q_contact_distance"][k])
                  and info.moving_sphere == g["q_moving_sphere"][k]
                  and info.other_sphere == g["q_other_sphere"][k]
                  and info.other_aggregate == g["q_other_agg"][k]
                  and (info.moving_aggregate == g["q_label"][k] or info.moving_sphere < 0))
            if not ok:
                bad.append((k, info, g["q_contact_distance"][k], g["q_moving_sphere"][k], g["q_other_sphere"][k],
                            g["q_other_agg"][k]))
        assert not bad, bad[:5]
        assert int(g["q_contact"].sum()) > 50  # the fixture exercises contacts


@pytest.mark.gpu
@pytest.mark.parametrize("fixture", FIXTURES)
def test_merges_match_reference_bitwise(fixture):
    g = load_golden(fixture)
    snap = Snapshot.from_npz(g, "s_")
    pm = PhysicalModel(text=str(g["ini"]))
    offsets = np.concatenate([[0], np.cumsum(g["m_n"])])
    assert len(g["m_index"]) > 50
    for r, q in enumerate(g["m_index"]):
        with AggregatList(pm, snap) as box:
            d = g["q_dir"][q]
            info = box.distance_to_next_contact(int(g["q_label"][q]), d, float(g["q_distance"][q]))
            box.translate(int(g["q_label"][q]), np.asarray(d) * info.distance)
            assert box.merge(info) == bool(g["m_merged"][r])
            keep = int(g["m_keep"][r])
            fields, n = box.aggregate(keep)
            assert n == g["m_n"][r]
            ref = g["m_record"][r]
            np.testing.assert_array_equal(fields[GEOMETRY_FIELDS].view(np.int64), ref[GEOMETRY_FIELDS].view(np.int64))
            np.testing.assert_allclose(fields[LIBM_FIELDS], ref[LIBM_FIELDS], rtol=4 * 2.0**-52, atol=0)
            if r < 30:
                ob = O.OracleBox(str(g["ini"]), snap)
                c = ob.distance_to_next_contact(g["q_label"][q], d, g["q_distance"][q])
                ob.translate(g["q_label"][q], np.asarray(d) * c.distance)
                assert ob.merge(c)
                np.testing.assert_array_equal(fields.view(np.int64), ob.store().aggregates[:, keep].view(np.int64))
            st = box.store()
            assert st.maxradius == g["m_maxradius"][r]
            ids = g["m_sphere_ids"][offsets[r]:offsets[r + 1]]
            np.testing.assert_array_equal(st.members_of(keep), ids)
            rows = st.spheres[:, ids].T
            np.testing.assert_array_equal(rows.view(np.int64), g["m_sphere_rows"][offsets[r]:offsets[r + 1]].view(np.int64))
