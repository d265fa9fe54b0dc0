"""The batched contact query that allocates no device memory.

mcacg_distance_to_next_contacts_static keeps every device buffer in a
file-scope array, for callers that cannot allocate device memory while they
run. Called through the C-ABI twice in a row, it must give the same answers,
byte for byte, as mcacg_distance_to_next_contacts on the same box; it must
leave the device's free memory unchanged, also on boxes that the allocating
entry point never touched; requests beyond its fixed limits must fail with a
clear error. The file is named to be collected last, and it passes alone in
a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest

from mcac_gb300 import CONTACT_DTYPE, AggregatList
from mcac_gb300._lib import Contact, MCACError, check, lib, ptr
from mcac_gb300.workloads import contact_search_case


def static_queries(box, sources, directions, distances):
    src = np.ascontiguousarray(sources, dtype=np.int64)
    d = np.ascontiguousarray(directions, dtype=np.float64).reshape(len(src), 3)
    dist = np.ascontiguousarray(distances, dtype=np.float64)
    out = np.zeros(len(src), dtype=CONTACT_DTYPE)
    check(lib().mcacg_distance_to_next_contacts_static(box._box, len(src), ptr(src, C.c_int64), ptr(d, C.c_double),
                                                       ptr(dist, C.c_double), out.ctypes.data_as(C.POINTER(Contact))))
    return out


@pytest.mark.gpu
def test_static_scratch_queries_equal_allocating_queries():
    case = contact_search_case(n_spheres=30_000, n_aggregates=600, n_queries=3000, seed=21)
    with AggregatList(case.model, case.state) as box:
        for scale in (1.0, 6.0):
            ref, _ = box.distance_to_next_contacts(case.sources, case.directions, scale * case.distances)
            first = static_queries(box, case.sources, case.directions, scale * case.distances)
            second = static_queries(box, case.sources, case.directions, scale * case.distances)
            assert np.array_equal(first.view(np.uint8), ref.view(np.uint8))
            assert np.array_equal(second.view(np.uint8), ref.view(np.uint8))
        assert (ref["moving_sphere"] >= 0).sum() > 50


@pytest.mark.gpu
def test_static_scratch_allocates_nothing():
    """After the first call on the device (which loads the module holding
    the array), calls on fresh boxes and on used ones leave the device's free
    memory as it was; the allocating entry point runs only afterwards, as
    the check of the answers."""
    import torch
    case = contact_search_case(n_spheres=20_000, n_aggregates=400, n_queries=2000, seed=23)
    with AggregatList(case.model, case.state) as a, AggregatList(case.model, case.state) as b:
        first = static_queries(a, case.sources, case.directions, case.distances)  # set-up call on this device
        torch.cuda.synchronize()
        torch.cuda.mem_get_info()
        free0, _ = torch.cuda.mem_get_info()
        outs = [static_queries(b, case.sources, case.directions, case.distances) for _ in range(3)]
        outs += [static_queries(a, case.sources, case.directions, 3.0 * case.distances) for _ in range(2)]
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, (free0, free1)
        for o in outs[:3]:
            assert np.array_equal(o.view(np.uint8), first.view(np.uint8))
        assert np.array_equal(outs[3].view(np.uint8), outs[4].view(np.uint8))
        ref, _ = b.distance_to_next_contacts(case.sources, case.directions, case.distances)
        assert np.array_equal(first.view(np.uint8), ref.view(np.uint8))
        ref3, _ = a.distance_to_next_contacts(case.sources, case.directions, 3.0 * case.distances)
        assert np.array_equal(outs[3].view(np.uint8), ref3.view(np.uint8))


@pytest.mark.gpu
def test_static_scratch_limits():
    case = contact_search_case(n_spheres=5_000, n_aggregates=100, n_queries=4, seed=22)
    with AggregatList(case.model, case.state) as box:
        assert len(static_queries(box, [], np.zeros((0, 3)), [])) == 0
        with pytest.raises(MCACError, match="out of range"):
            static_queries(box, [len(box)], [[1.0, 0.0, 0.0]], [1e-7])
        n = (1 << 16) + 1
        with pytest.raises(MCACError, match="queries per call"):
            static_queries(box, np.zeros(n, np.int64), np.tile([1.0, 0.0, 0.0], (n, 1)), np.full(n, 1e-7))
        # still usable after the refusals
        ref, _ = box.distance_to_next_contacts(case.sources, case.directions, case.distances)
        out = static_queries(box, case.sources, case.directions, case.distances)
        assert np.array_equal(out.view(np.uint8), ref.view(np.uint8))


@pytest.mark.gpu
def test_static_scratch_refuses_a_box_too_large_for_it():
    # 1,000,000 aggregate slots need 44 MB of candidate lists per block, more
    # than the whole 32 MiB array
    from mcac_gb300 import PhysicalModel, synthetic_state
    from mcac_gb300.workloads import contact_search_ini
    pm = PhysicalModel(text=contact_search_ini(1_000_000, seed=3, sigma_geo=1.25, volume_fraction=1e-3))
    sb = synthetic_state(pm, 1_000_000, 1)
    with AggregatList(pm, sb) as box:
        with pytest.raises(MCACError, match="too large for the static scratch"):
            static_queries(box, [0], [[1.0, 0.0, 0.0]], [1e-8])
