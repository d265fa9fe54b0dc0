"""ctypes binding of include/mcacg.h (the library's C-ABI).

Loads ``mcac_gb300/_build/libmcacg.so`` (built by ``mcac_gb300.build`` /
``__graft_entry__.build()``). There is no fallback: when the library is
missing, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libmcacg.so"

i32, i64, f64, vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p


class Params(C.Structure):
    _fields_ = [
        ("n_monomeres", i64), ("density", f64), ("mean_diameter", f64), ("dispersion_diameter", f64),
        ("initialisation_mode", i32), ("pick_method", i32),
        ("initial_time", f64), ("volume_fraction", f64), ("temperature", f64), ("pressure", f64),
        ("fractal_prefactor", f64), ("fractal_dimension", f64),
        ("with_surface_reactions", i32), ("volsurf_method", i32), ("flux_surfgrowth", f64), ("rp_min_oxid", f64),
        ("full_aggregate_update_frequency", i64),
        ("number_of_aggregates_limit", i64), ("n_iter_without_event_limit", i64), ("cpu_limit", f64),
        ("physical_time_limit", f64), ("mean_monomere_per_aggregate_limit", i64),
        ("with_domain_duplication", i32), ("with_domain_reduction", i32), ("with_collisions", i32),
        ("enforce_volume_fraction", i32), ("individual_surf_reactions", i32), ("random_seed", i32),
        ("n_verlet_divisions", i64),
        ("with_nucleation", i32), ("with_potentials", i32), ("with_flame_coupling", i32),
        ("with_electric_charges", i32),
        ("box_length", f64), ("box_volume", f64), ("viscosity", f64), ("gaz_mean_free_path", f64),
        ("mean_massic_radius", f64), ("friction_exponnant", f64), ("u_sg", f64),
        ("write_events_frequency", i64), ("write_between_event_frequency", i64), ("write_delta_t", f64),
        ("cpu_event_limit", f64),
    ]


class Contact(C.Structure):
    _fields_ = [("distance", f64), ("moving_sphere", i64), ("other_sphere", i64),
                ("moving_aggregate", i64), ("other_aggregate", i64)]


class State(C.Structure):
    _fields_ = [("n_spheres", i64), ("n_aggregates", i64), ("n_verlet_divisions", i64),
                ("box_length", f64), ("maxradius", f64), ("time", f64),
                ("spheres", C.POINTER(f64)), ("sphere_label", C.POINTER(i64)), ("aggregates", C.POINTER(f64)),
                ("n_spheres_per_aggregate", C.POINTER(i64)), ("members", C.POINTER(i64))]


class StepRecord(C.Structure):
    _fields_ = [("step", i64), ("picked", i64), ("contact", i64), ("merged", i64), ("moving_sphere", i64),
                ("other_sphere", i64), ("moving_agg", i64), ("other_agg", i64), ("n_agg_after", i64),
                ("deltatemps", f64), ("full_distance", f64), ("dir", f64 * 3), ("contact_distance", f64),
                ("move_distance", f64), ("time_after", f64), ("reserved", f64)]


class RunOpts(C.Structure):
    _fields_ = [("max_steps", i64), ("trace", C.POINTER(StepRecord)), ("trace_capacity", i64),
                ("advancement_path", C.c_char_p)]


class RunStats(C.Structure):
    _fields_ = [("steps", i64), ("events", i64), ("n_aggregates", i64), ("time", f64),
                ("finished", i32), ("reserved", i32)]


class Profile(C.Structure):
    _fields_ = [("queries", i64), ("merges", i64), ("translates", i64), ("query_ms", f64), ("merge_ms", f64),
                ("mov_spheres", i64), ("scanned", i64), ("cells", i64), ("candidates", i64),
                ("cand_spheres", i64), ("refined", i64), ("merged_spheres", i64), ("merge_pairs", i64),
                ("cycles_pick", i64), ("cycles_query", i64), ("cycles_move", i64), ("cycles_merge", i64),
                ("cycles_query_scan", i64), ("cycles_query_pairs", i64)]


# every exported symbol with its argument types (restype is int unless noted)
SIGNATURES = {
    "mcacg_abi_version": [],
    "mcacg_last_error": [],
    "mcacg_device_count": [C.POINTER(C.c_int)],
    "mcacg_params_default": [C.POINTER(Params)],
    "mcacg_params_from_ini": [C.c_char_p, C.POINTER(Params)],
    "mcacg_params_from_ini_text": [C.c_char_p, C.POINTER(Params)],
    "mcacg_state_init_random": [C.POINTER(Params), C.POINTER(State)],
    "mcacg_state_synthetic": [C.POINTER(Params), i32, i32, C.POINTER(State)],
    "mcacg_box_create": [C.POINTER(Params), C.POINTER(vp)],
    "mcacg_box_create_from_state": [C.POINTER(Params), C.POINTER(State), C.POINTER(vp)],
    "mcacg_box_destroy": [vp],
    "mcacg_box_set_stream": [vp, vp],
    "mcacg_box_sizes": [vp, C.POINTER(i64), C.POINTER(i64)],
    "mcacg_box_store_state": [vp, C.POINTER(State)],
    "mcacg_box_get_time": [vp, C.POINTER(f64)],
    "mcacg_box_set_time": [vp, f64],
    "mcacg_box_set_profiling": [vp, C.c_int],
    "mcacg_box_take_profile": [vp, C.POINTER(Profile)],
    "mcacg_distance_to_next_contact": [vp, i64, C.POINTER(f64), f64, C.POINTER(Contact)],
    "mcacg_distance_to_next_contacts": [vp, i32, C.POINTER(i64), C.POINTER(f64), C.POINTER(f64),
                                        C.POINTER(Contact), C.POINTER(f64)],
    "mcacg_distance_to_next_contacts_static": [vp, i32, C.POINTER(i64), C.POINTER(f64), C.POINTER(f64),
                                               C.POINTER(Contact)],
    "mcacg_translate": [vp, i64, C.POINTER(f64)],
    "mcacg_time_forward": [vp, i64, f64],
    "mcacg_merge": [vp, C.POINTER(Contact), C.POINTER(i32)],
    "mcacg_sort_time_steps": [vp, f64],
    "mcacg_pick_random": [vp, C.POINTER(i64)],
    "mcacg_get_time_step": [vp, f64, C.POINTER(f64)],
    "mcacg_get_max_time_step": [vp, C.POINTER(f64)],
    "mcacg_refresh": [vp],
    "mcacg_size": [vp, C.POINTER(i64)],
    "mcacg_get_avg_npp": [vp, C.POINTER(f64)],
    "mcacg_get_total_volume": [vp, C.POINTER(f64)],
    "mcacg_get_total_surface": [vp, C.POINTER(f64)],
    "mcacg_get_aggregate": [vp, i64, C.POINTER(f64), C.POINTER(i64)],
    "mcacg_calcul": [vp, C.POINTER(RunOpts), C.POINTER(RunStats)],
    "mcacg_run_device": [vp, i64, C.POINTER(RunStats)],
    "mcacg_batch_create": [C.POINTER(Params), i32, vp, C.POINTER(vp)],
    "mcacg_batch_create_from_states": [C.POINTER(Params), C.POINTER(State), i32, vp, C.POINTER(vp)],
    "mcacg_batch_destroy": [vp],
    "mcacg_host_alloc": [i64, C.POINTER(vp)],
    "mcacg_set_merge_grid_min": [C.c_int32, C.POINTER(C.c_int32)],
    "mcacg_set_live_list_max": [C.c_int32, C.POINTER(C.c_int32)],
    "mcacg_host_free": [vp],
    "mcacg_resident_boxes": [i32, C.POINTER(i32)],
    "mcacg_batch_set_threads": [vp, i32],
    "mcacg_batch_threads": [vp, C.POINTER(i32)],
    "mcacg_batch_set_aggregate_limit": [vp, i64],
    "mcacg_batch_set_speculation": [vp, i32],
    "mcacg_batch_speculation": [vp, C.POINTER(i32)],
    "mcacg_batch_pick_histogram": [vp, i32, i64, C.c_uint32, C.POINTER(i64), i64, C.POINTER(i64), C.POINTER(i64)],
    "mcacg_draw_directions": [i64, C.c_uint32, C.POINTER(f64)],
    "mcacg_batch_run": [vp, i64, i64],
    "mcacg_batch_run_timed": [vp, f64],
    "mcacg_batch_stats": [vp, C.POINTER(RunStats)],
    "mcacg_batch_size": [vp, C.POINTER(i32)],
    "mcacg_batch_box_sizes": [vp, i32, C.POINTER(i64), C.POINTER(i64)],
    "mcacg_batch_store_state": [vp, i32, C.POINTER(State)],
    "mcacg_batch_store_states": [vp, C.POINTER(State), i32],
    "mcacg_batch_last_run": [vp, C.POINTER(f64), C.POINTER(i32)],
    "mcacg_batch_work": [vp, C.POINTER(Profile)],
    "mcacg_batch_box_work": [vp, i32, C.POINTER(Profile)],
    "mcacg_server_create": [i32, i64, vp, i32, C.POINTER(vp)],
    "mcacg_server_destroy": [vp],
    "mcacg_server_set_threads": [vp, i32],
    "mcacg_server_set_epoch_ms": [vp, f64],
    "mcacg_server_submit": [vp, C.POINTER(Params), C.POINTER(i64)],
    "mcacg_server_step": [vp, i64, C.POINTER(i32), C.POINTER(i32)],
    "mcacg_server_poll": [vp, C.c_void_p, i32, C.POINTER(i32)],
    "mcacg_server_final_sizes": [vp, i64, C.POINTER(i64), C.POINTER(i64)],
    "mcacg_server_final_state": [vp, i64, C.POINTER(State)],
    "mcacg_server_kernel_time": [vp, C.POINTER(f64), C.POINTER(i32)],
}

COMPLETION_DTYPE = np.dtype([("id", "<i8"), ("steps", "<i8"), ("events", "<i8"), ("n_aggregates", "<i8"),
                             ("time", "<f8"), ("status", "<i4"), ("finished", "<i4"), ("submit_s", "<f8"),
                             ("admit_s", "<f8"), ("finish_s", "<f8")])

_lock = threading.Lock()
_lib = None


def lib() -> C.CDLL:
    """The loaded C-ABI library; raises when it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
            handle = C.CDLL(str(LIB_PATH))
            for name, args in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.argtypes = args
                fn.restype = C.c_char_p if name == "mcacg_last_error" else C.c_int
            _lib = handle
        return _lib


# -- errors: the reference's exception classes, by ErrorCodes value ---------
class MCACError(RuntimeError):
    code = 1
    name = "Unknown Error"


def _exc(name: str, code: int):
    return type(name, (MCACError,), {"code": code, "name": name})


IOError_ = _exc("IOError", 2)
VerletError = _exc("VerletError", 3)
InputError = _exc("InputError", 4)
AbandonError = _exc("AbandonError", 5)
TooDenseError = _exc("TooDenseError", 6)
SBLError = _exc("SBLError", 7)
VolSurfError = _exc("VolSurfError", 8)
MergeError = _exc("MergeError", 9)
ARVOError = _exc("ARVOError", 10)
CudaError = _exc("CudaError", 100)
CapacityError = _exc("CapacityError", 101)
DeviceTimeout = _exc("DeviceTimeout", 102)
BadArgument = _exc("BadArgument", 103)
NoDevice = _exc("NoDevice", 104)
_BY_CODE = {c.code: c for c in (IOError_, VerletError, InputError, AbandonError, TooDenseError, SBLError,
                                VolSurfError, MergeError, ARVOError, CudaError, CapacityError, DeviceTimeout,
                                BadArgument, NoDevice)}


def check(rc: int) -> None:
    if rc == 0:
        return
    msg = lib().mcacg_last_error().decode(errors="replace")
    raise _BY_CODE.get(rc, MCACError)(f"[{rc}] {msg}")


def ptr(arr: np.ndarray, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


class _PinnedBlock:
    """Page-locked host memory from the library, freed with the last array
    that views it."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        check(lib().mcacg_host_alloc(int(nbytes), C.byref(p)))
        self.ptr, self.nbytes = p.value, int(nbytes)

    def __del__(self):
        if self.ptr:
            lib().mcacg_host_free(C.c_void_p(self.ptr))
            self.ptr = None

    def buffer(self):
        buf = (C.c_char * self.nbytes).from_address(self.ptr)
        buf._owner = self  # the numpy views keep the block alive through buf
        return buf


class StateBuffers:
    """Host arrays behind an mcacg_state (keeps them alive). With
    pinned=True they sit in one page-locked block, so loading and storing
    the state moves them by DMA."""

    @staticmethod
    def _layout(ns: int, na: int):
        return [("spheres", np.float64, (9, ns)), ("sphere_label", np.int64, (ns,)),
                ("aggregates", np.float64, (21, na)), ("n_spheres", np.int64, (na,)), ("members", np.int64, (ns,))]

    @staticmethod
    def _bytes(ns: int, na: int) -> int:
        return 8 * (11 * ns + 22 * na)

    def __init__(self, n_spheres: int, n_aggregates: int, pinned: bool = False, _buf=None, _offset: int = 0):
        ns, na = int(n_spheres), int(n_aggregates)
        if pinned or _buf is not None:
            buf = _buf if _buf is not None else _PinnedBlock(max(self._bytes(ns, na), 8)).buffer()
            off = _offset
            for name, dt, shape in self._layout(ns, na):
                count = int(np.prod(shape))
                setattr(self, name, np.frombuffer(buf, dtype=dt, count=count, offset=off).reshape(shape))
                off += 8 * count
        else:
            self.spheres = np.zeros((9, ns), dtype=np.float64)
            self.sphere_label = np.zeros(ns, dtype=np.int64)
            self.aggregates = np.zeros((21, na), dtype=np.float64)
            self.n_spheres = np.zeros(na, dtype=np.int64)
            self.members = np.zeros(ns, dtype=np.int64)
        self.state = State(ns, na, 0, 0.0, 0.0, 0.0,
                           ptr(self.spheres, f64), ptr(self.sphere_label, i64), ptr(self.aggregates, f64),
                           ptr(self.n_spheres, i64), ptr(self.members, i64))

    @classmethod
    def many(cls, sizes, pinned: bool = True) -> list:
        """StateBuffers for many boxes ((n_spheres, n_aggregates) each); with
        pinned=True all of them in one page-locked block, allocated at once
        (large page-locked blocks made before the host memory fragments copy
        fastest)."""
        sizes = [(int(a), int(b)) for a, b in sizes]
        if not pinned:
            return [cls(ns, na) for ns, na in sizes]
        buf = _PinnedBlock(max(8, sum(cls._bytes(ns, na) for ns, na in sizes))).buffer()
        out, off = [], 0
        for ns, na in sizes:
            out.append(cls(ns, na, _buf=buf, _offset=off))
            off += cls._bytes(ns, na)
        return out

    @classmethod
    def from_snapshot(cls, snap, pinned: bool = False) -> "StateBuffers":
        sb = cls(snap.ns, snap.na, pinned=pinned)
        sb.spheres[...] = snap.spheres
        sb.sphere_label[...] = snap.sphere_label
        sb.aggregates[...] = snap.aggregates
        sb.n_spheres[...] = snap.n_spheres
        sb.members[...] = snap.members
        sb.state.n_verlet_divisions = snap.n_div
        sb.state.box_length = snap.box_length
        sb.state.maxradius = snap.maxradius
        sb.state.time = snap.time
        return sb

    def to_snapshot(self, physics=None, volsurf_method: int = 4):
        from .snapshot import Snapshot
        st = self.state
        ns, na = int(st.n_spheres), int(st.n_aggregates)
        nsph = self.n_spheres[:na].copy()
        cells = np.zeros((na, 3), dtype=np.int64)
        step = st.n_verlet_divisions / st.box_length if st.box_length > 0 else 0.0
        agg = self.aggregates.reshape(-1)[:21 * na].reshape(21, na)  # stored packed as [21][na]
        for k, f in enumerate((7, 8, 9)):
            cells[:, k] = np.floor(agg[f] * step).astype(np.int64)
        return Snapshot(
            n_div=int(st.n_verlet_divisions), box_length=float(st.box_length), maxradius=float(st.maxradius),
            time=float(st.time), physics=np.zeros(9) if physics is None else np.asarray(physics, float),
            volsurf_method=volsurf_method, spheres=self.spheres.reshape(-1)[:9 * ns].reshape(9, ns).copy(),
            sphere_label=self.sphere_label[:ns].copy(),
            aggregates=self.aggregates.reshape(-1)[:21 * na].reshape(21, na).copy(),
            n_spheres=nsph, members=self.members[:int(nsph.sum())].copy(), cells=cells)
