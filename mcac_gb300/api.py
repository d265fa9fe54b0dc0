"""Python face of the library, named after the reference's C++ interface.

``PhysicalModel`` is the parameter file (src/physical_model/physical_model.cpp),
``AggregatList`` one device-resident box with the methods src/calcul.cpp calls
each step (include/aggregats/aggregat_list.hpp), and ``calcul`` the MC loop.
Everything runs through the C-ABI in include/mcacg.h; nothing here computes
physics itself.
"""
from __future__ import annotations

import ctypes as C
import os
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import Contact, Params, RunOpts, RunStats, StateBuffers, StepRecord, check, lib, ptr
from .snapshot import STEP_DTYPE, Snapshot


class PhysicalModel:
    """The INI parameter file with the reference's keys, defaults and derived values."""

    def __init__(self, path: str | Path | None = None, text: str | None = None, **overrides):
        self.params = Params()
        if path is not None:
            check(lib().mcacg_params_from_ini(str(path).encode(), C.byref(self.params)))
        elif text is not None:
            check(lib().mcacg_params_from_ini_text(text.encode(), C.byref(self.params)))
        else:
            check(lib().mcacg_params_default(C.byref(self.params)))
        if overrides:
            self.set(**overrides)

    def set(self, **values) -> "PhysicalModel":
        """Change parameters and recompute the derived block through the library."""
        for k, v in values.items():
            if not hasattr(self.params, k):
                raise KeyError(k)
            setattr(self.params, k, v)
        # re-derive from the INI-level values
        text = self.to_ini()
        derived = Params()
        check(lib().mcacg_params_from_ini_text(text.encode(), C.byref(derived)))
        for name in ("box_length", "box_volume", "viscosity", "gaz_mean_free_path", "mean_massic_radius",
                     "friction_exponnant", "u_sg"):
            setattr(self.params, name, getattr(derived, name))
        return self

    def __getattr__(self, name):
        if name == "params":
            raise AttributeError(name)
        return getattr(self.params, name)

    def to_ini(self) -> str:
        p = self.params
        b = lambda v: "true" if v else "false"  # noqa: E731
        modes = {0: "lognormal", 1: "normal"}
        volsurf = {0: "caps", 1: "sbl", 2: "arvo", 3: "alphas", 4: "none"}
        return "\n".join([
            "[monomers]", f"number = {p.n_monomeres}", f"density = {p.density!r}",
            f"mean_diameter = {p.mean_diameter!r}", f"dispersion_diameter = {p.dispersion_diameter!r}",
            f"initialisation_mode = {modes[p.initialisation_mode]}",
            "[environment]", f"initial_time = {p.initial_time!r}", f"volume_fraction = {p.volume_fraction!r}",
            f"temperature = {p.temperature!r}", f"pressure = {p.pressure!r}",
            f"fractal_prefactor = {p.fractal_prefactor!r}", f"fractal_dimension = {p.fractal_dimension!r}",
            "[surface_growth]", f"with_surface_reactions = {b(p.with_surface_reactions)}",
            f"flux_surfgrowth = {p.flux_surfgrowth!r}", f"volsurf_method = {volsurf[p.volsurf_method]}",
            f"full_aggregate_update_frequency = {p.full_aggregate_update_frequency}",
            "[oxidation]", f"rp_min = {p.rp_min_oxid!r}",
            "[limits]", f"number_of_aggregates = {p.number_of_aggregates_limit}",
            f"n_iter_without_event = {p.n_iter_without_event_limit}", f"cpu = {p.cpu_limit!r}",
            f"cpu_event = {p.cpu_event_limit!r}",
            f"physical_time = {p.physical_time_limit!r}",
            f"mean_monomere_per_aggregate = {p.mean_monomere_per_aggregate_limit}",
            "[numerics]", f"with_domain_duplication = {b(p.with_domain_duplication)}",
            f"with_domain_reduction = {b(p.with_domain_reduction)}",
            f"with_collisions = {b(p.with_collisions)}",
            f"enforce_volume_fraction = {b(p.enforce_volume_fraction)}",
            f"individual_surf_reactions = {b(p.individual_surf_reactions)}",
            f"n_verlet_divisions = {p.n_verlet_divisions}",
            f"pick_method = {'random' if p.pick_method == 0 else 'last'}",
            f"random_seed = {p.random_seed}", "",
        ])


def init_state(model: PhysicalModel) -> StateBuffers:
    """The reference constructor's random placement, on the host (no GPU)."""
    n = int(model.params.n_monomeres)
    sb = StateBuffers(n, n)
    check(lib().mcacg_state_init_random(C.byref(model.params), C.byref(sb.state)))
    return sb


def synthetic_state(model: PhysicalModel, n_aggregates: int, max_size: int) -> StateBuffers:
    """A seeded synthetic snapshot of ballistic aggregates (host, no GPU):
    model.n_monomeres spheres in n_aggregates aggregates of 1..max_size
    spheres, in a periodic cube sized for model.volume_fraction."""
    n = int(model.params.n_monomeres)
    sb = StateBuffers(n, int(n_aggregates))
    check(lib().mcacg_state_synthetic(C.byref(model.params), int(n_aggregates), int(max_size),
                                      C.byref(sb.state)))
    return sb


# one mcacg_contact per row
CONTACT_DTYPE = np.dtype([("distance", np.float64), ("moving_sphere", np.int64), ("other_sphere", np.int64),
                          ("moving_aggregate", np.int64), ("other_aggregate", np.int64)])


@dataclass
class AggregateContactInfo:
    """include/tools/contact_info.hpp:73-85 with indices for the weak pointers."""
    distance: float
    moving_sphere: int
    other_sphere: int
    moving_aggregate: int
    other_aggregate: int

    def __le__(self, d: float) -> bool:  # SphereContactInfo::operator<=
        return self.distance <= d

    def to_c(self) -> Contact:
        return Contact(self.distance, self.moving_sphere, self.other_sphere, self.moving_aggregate,
                       self.other_aggregate)


class AggregatList:
    """One box on the GPU behind the reference's AggregatList interface."""

    def __init__(self, model: PhysicalModel, state: Snapshot | StateBuffers | None = None,
                 stream: int | None = None):
        self.model = model
        self._box = C.c_void_p()
        if state is None:
            check(lib().mcacg_box_create(C.byref(model.params), C.byref(self._box)))
        else:
            sb = state if isinstance(state, StateBuffers) else StateBuffers.from_snapshot(state)
            check(lib().mcacg_box_create_from_state(C.byref(model.params), C.byref(sb.state), C.byref(self._box)))
        if stream is not None:
            check(lib().mcacg_box_set_stream(self._box, C.c_void_p(stream)))

    def close(self) -> None:
        if self._box:
            check(lib().mcacg_box_destroy(self._box))
            self._box = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- getters
    def size(self) -> int:
        v = C.c_int64()
        check(lib().mcacg_size(self._box, C.byref(v)))
        return v.value

    def __len__(self) -> int:
        return self.size()

    @property
    def time(self) -> float:
        v = C.c_double()
        check(lib().mcacg_box_get_time(self._box, C.byref(v)))
        return v.value

    @time.setter
    def time(self, t: float) -> None:
        check(lib().mcacg_box_set_time(self._box, float(t)))

    def get_avg_npp(self) -> float:
        v = C.c_double()
        check(lib().mcacg_get_avg_npp(self._box, C.byref(v)))
        return v.value

    def get_max_time_step(self) -> float:
        v = C.c_double()
        check(lib().mcacg_get_max_time_step(self._box, C.byref(v)))
        return v.value

    def get_time_step(self, factor: float) -> float:
        v = C.c_double()
        check(lib().mcacg_get_time_step(self._box, float(factor), C.byref(v)))
        return v.value

    def get_total_volume(self) -> float:
        v = C.c_double()
        check(lib().mcacg_get_total_volume(self._box, C.byref(v)))
        return v.value

    def get_total_surface(self) -> float:
        v = C.c_double()
        check(lib().mcacg_get_total_surface(self._box, C.byref(v)))
        return v.value

    def aggregate(self, label: int) -> tuple[np.ndarray, int]:
        f = np.zeros(21)
        n = C.c_int64()
        check(lib().mcacg_get_aggregate(self._box, int(label), ptr(f, C.c_double), C.byref(n)))
        return f, n.value

    # -- per-step interface
    def distance_to_next_contact(self, source: int, direction, distance: float) -> AggregateContactInfo:
        d = np.ascontiguousarray(direction, dtype=np.float64)
        c = Contact()
        check(lib().mcacg_distance_to_next_contact(self._box, int(source), ptr(d, C.c_double), float(distance),
                                                    C.byref(c)))
        return AggregateContactInfo(c.distance, c.moving_sphere, c.other_sphere, c.moving_aggregate,
                                    c.other_aggregate)

    def distance_to_next_contacts(self, sources, directions, distances) -> tuple[np.ndarray, float]:
        """Many independent queries on the current state, run concurrently on
        the GPU. Returns (CONTACT_DTYPE array, kernel milliseconds)."""
        src = np.ascontiguousarray(sources, dtype=np.int64)
        d = np.ascontiguousarray(directions, dtype=np.float64).reshape(len(src), 3)
        dist = np.ascontiguousarray(distances, dtype=np.float64)
        if dist.shape != src.shape:
            raise ValueError("sources and distances differ in length")
        out = np.zeros(len(src), dtype=CONTACT_DTYPE)
        ms = C.c_double(0.0)
        check(lib().mcacg_distance_to_next_contacts(self._box, len(src), ptr(src, C.c_int64), ptr(d, C.c_double),
                                                     ptr(dist, C.c_double),
                                                     out.ctypes.data_as(C.POINTER(Contact)), C.byref(ms)))
        return out, ms.value

    def translate(self, label: int, vector) -> None:
        v = np.ascontiguousarray(vector, dtype=np.float64)
        check(lib().mcacg_translate(self._box, int(label), ptr(v, C.c_double)))

    def time_forward(self, label: int, deltatemps: float) -> None:
        check(lib().mcacg_time_forward(self._box, int(label), float(deltatemps)))

    def merge(self, info: AggregateContactInfo) -> bool:
        c = info.to_c()
        m = C.c_int32()
        check(lib().mcacg_merge(self._box, C.byref(c), C.byref(m)))
        return bool(m.value)

    def sort_time_steps(self, factor: float) -> None:
        check(lib().mcacg_sort_time_steps(self._box, float(factor)))

    def pick_random(self) -> int:
        v = C.c_int64()
        check(lib().mcacg_pick_random(self._box, C.byref(v)))
        return v.value

    def refresh(self) -> None:
        check(lib().mcacg_refresh(self._box))

    # -- instrumentation
    def set_profiling(self, on: bool = True) -> None:
        check(lib().mcacg_box_set_profiling(self._box, 1 if on else 0))

    def take_profile(self) -> dict:
        p = _lib.Profile()
        check(lib().mcacg_box_take_profile(self._box, C.byref(p)))
        return {name: getattr(p, name) for name, _ in _lib.Profile._fields_}

    # -- whole runs and state
    def calcul(self, max_steps: int = 0, trace: bool = False, trace_capacity: int = 0,
               advancement: str | os.PathLike | None = None):
        """The reference MC loop; returns (stats, records or None). With
        'advancement', the reference's time-resolved lines are appended to
        that file (advancement.dat of the reference's output directory)."""
        recs = None
        opts = RunOpts(int(max_steps), None, 0, os.fsencode(advancement) if advancement is not None else None)
        if trace:
            cap = int(trace_capacity or max_steps or 1_000_000)
            recs = (StepRecord * cap)()
            opts.trace = C.cast(recs, C.POINTER(StepRecord))
            opts.trace_capacity = cap
        stats = RunStats()
        check(lib().mcacg_calcul(self._box, C.byref(opts), C.byref(stats)))
        out = None
        if trace:
            n = min(int(stats.steps), opts.trace_capacity)
            out = np.frombuffer(bytes(memoryview(recs).cast("B")[: n * C.sizeof(StepRecord)]), dtype=STEP_DTYPE)
        return stats, out

    def store(self) -> Snapshot:
        ns, na = C.c_int64(), C.c_int64()
        check(lib().mcacg_box_sizes(self._box, C.byref(ns), C.byref(na)))
        sb = StateBuffers(ns.value, na.value)
        check(lib().mcacg_box_store_state(self._box, C.byref(sb.state)))
        return sb.to_snapshot(volsurf_method=int(self.model.params.volsurf_method))


def set_merge_grid_min(n_spheres: int) -> int:
    """Merged aggregates of at least n_spheres spheres find their contact
    pairs on a hashed cell grid, smaller ones by testing all pairs (the same
    pairs either way). Read by boxes created afterwards; returns the previous
    value (default 2048)."""
    prev = C.c_int32(0)
    check(lib().mcacg_set_merge_grid_min(int(n_spheres), C.byref(prev)))
    return prev.value


def draw_directions(n: int, seed: int = 1) -> np.ndarray:
    """n unit vectors from the device loop's direction draw (n x 3)."""
    out = np.zeros((int(n), 3), dtype=np.float64)
    check(lib().mcacg_draw_directions(int(n), int(seed) & 0xffffffff, ptr(out, C.c_double)))
    return out


def set_live_list_max(n_aggregates: int) -> int:
    """Live aggregates from which the device loop lists them in shared memory
    (0: never, at most 128); process-wide, for batches made afterwards.
    Returns the previous value."""
    prev = C.c_int32()
    check(lib().mcacg_set_live_list_max(int(n_aggregates), C.byref(prev)))
    return prev.value


def device_count() -> int:
    n = C.c_int()
    check(lib().mcacg_device_count(C.byref(n)))
    return n.value


def resident_boxes(threads: int = 256) -> int:
    """Boxes the device-resident loop runs at once on the current device with
    'threads' threads per box."""
    n = C.c_int32(0)
    check(lib().mcacg_resident_boxes(int(threads), C.byref(n)))
    return n.value


def _run_stats(box_run) -> RunStats:
    return box_run


class Batch:
    """Independent boxes advanced together by the device-resident loop.

    Box i is placed exactly as ``AggregatList(models[i])`` would place it;
    afterwards every step runs on the GPU (one thread block per box) with the
    statistics of the reference's loop (see include/mcacg.h).
    """

    def __init__(self, models, stream: int | None = None, states=None):
        models = list(models)
        arr = (Params * len(models))(*[m.params for m in models])
        self.models = models
        self._b = C.c_void_p()
        s = C.c_void_p(stream) if stream else None
        if states is None:
            check(lib().mcacg_batch_create(arr, len(models), s, C.byref(self._b)))
        else:
            bufs = [st if isinstance(st, StateBuffers) else StateBuffers.from_snapshot(st) for st in states]
            sarr = (_lib.State * len(bufs))(*[b.state for b in bufs])
            check(lib().mcacg_batch_create_from_states(arr, sarr, len(models), s, C.byref(self._b)))

    def close(self) -> None:
        if self._b:
            check(lib().mcacg_batch_destroy(self._b))
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self) -> int:
        return len(self.models)

    @property
    def threads(self) -> int:
        """Threads per box of the loop (0 until chosen at the first run: the
        largest size at which every unfinished box is resident)."""
        n = C.c_int32(0)
        check(lib().mcacg_batch_threads(self._b, C.byref(n)))
        return n.value

    @threads.setter
    def threads(self, value: int) -> None:
        check(lib().mcacg_batch_set_threads(self._b, int(value)))

    @property
    def speculation(self) -> int:
        """Thread blocks per box of the loop's speculative rounds (1: none)."""
        n = C.c_int32(0)
        check(lib().mcacg_batch_speculation(self._b, C.byref(n)))
        return n.value

    @speculation.setter
    def speculation(self, value: int) -> None:
        """1 (the default) or 0: none; 2, 4 or 8 blocks per box."""
        check(lib().mcacg_batch_set_speculation(self._b, int(value)))

    def run_timed(self, wall_ms: float) -> None:
        """Runs every unfinished box for about wall_ms of wall time, each as
        fast as it goes (returns early when all are done)."""
        check(lib().mcacg_batch_run_timed(self._b, float(wall_ms)))

    def run(self, max_steps: int = 0, steps_per_launch: int = 20000) -> None:
        check(lib().mcacg_batch_run(self._b, int(max_steps), int(steps_per_launch)))

    def set_aggregate_limit(self, limit: int) -> None:
        """Every box's number_of_aggregates stop criterion becomes 'limit';
        boxes that stopped without an error continue at the next run (each
        re-checks all of its criteria first)."""
        check(lib().mcacg_batch_set_aggregate_limit(self._b, int(limit)))

    def pick_histogram(self, box: int, n_picks: int, seed: int = 1) -> tuple[np.ndarray, int]:
        """Counts per label of n_picks (at least) picks from box 'box''s
        current pick tree by the device loop's own descent (nothing moves),
        and the number of picks made."""
        na = self.box_sizes(box)[1]
        counts = np.zeros(max(na, 1), dtype=np.int64)
        n_lab, done = C.c_int64(), C.c_int64()
        check(lib().mcacg_batch_pick_histogram(self._b, int(box), int(n_picks), int(seed) & 0xffffffff,
                                               ptr(counts, C.c_int64), len(counts), C.byref(n_lab), C.byref(done)))
        return counts[:n_lab.value], done.value

    def stats(self) -> np.ndarray:
        n = len(self.models)
        arr = (RunStats * n)()
        check(lib().mcacg_batch_stats(self._b, arr))
        out = np.zeros(n, dtype=[("steps", "i8"), ("events", "i8"), ("n_aggregates", "i8"), ("time", "f8"),
                                 ("finished", "i4"), ("status", "i4")])
        for i, s in enumerate(arr):
            out[i] = (s.steps, s.events, s.n_aggregates, s.time, s.finished, s.reserved)
        return out

    def box_work(self, box: int) -> dict:
        """Work counters and phase cycles of one box since creation."""
        p = _lib.Profile()
        check(lib().mcacg_batch_box_work(self._b, int(box), C.byref(p)))
        return {name: getattr(p, name) for name, _ in _lib.Profile._fields_}

    def work(self) -> dict:
        p = _lib.Profile()
        check(lib().mcacg_batch_work(self._b, C.byref(p)))
        return {name: getattr(p, name) for name, _ in _lib.Profile._fields_}

    def last_run(self) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_int32()
        check(lib().mcacg_batch_last_run(self._b, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def box_sizes(self, box: int) -> tuple[int, int]:
        """(spheres, live aggregates) of one box: the sizes its stored state needs."""
        ns, na = C.c_int64(), C.c_int64()
        check(lib().mcacg_batch_box_sizes(self._b, int(box), C.byref(ns), C.byref(na)))
        return ns.value, max(na.value, 1)

    def store_all(self, raw: bool = False, out: list | None = None, pinned: bool = False) -> list:
        """The state of every box (one call, converted in parallel): as
        Snapshots, or with raw=True as the filled host arrays
        (StateBuffers), without further copies. 'out' may supply the
        StateBuffers to fill (one per box, large enough), e.g. buffers kept
        from an earlier call; new buffers are page-locked with pinned=True."""
        if out is not None:
            bufs = list(out)
            for b in bufs:
                b.state.n_spheres, b.state.n_aggregates = b.spheres.shape[1], b.aggregates.shape[1]
        else:
            bufs = StateBuffers.many([self.box_sizes(box) for box in range(len(self.models))], pinned=pinned)
        arr = (_lib.State * len(bufs))(*[b.state for b in bufs])
        check(lib().mcacg_batch_store_states(self._b, arr, len(bufs)))
        for k, b in enumerate(bufs):
            b.state = arr[k]
            na = int(b.state.n_aggregates)
            if na != b.aggregates.shape[1]:  # the table is stored packed as [21][na]
                b.aggregates = b.aggregates.reshape(-1)[:21 * na].reshape(21, na)
            ns = int(b.state.n_spheres)
            if ns != b.spheres.shape[1]:  # spheres removed by oxidation: packed as [9][ns]
                b.spheres = b.spheres.reshape(-1)[:9 * ns].reshape(9, ns)
                b.sphere_label = b.sphere_label[:ns]
        if raw:
            return bufs
        return [b.to_snapshot(volsurf_method=int(self.models[k].params.volsurf_method)) for k, b in enumerate(bufs)]

    def store(self, box: int) -> Snapshot:
        sb = StateBuffers(*self.box_sizes(box))
        check(lib().mcacg_batch_store_state(self._b, int(box), C.byref(sb.state)))
        return sb.to_snapshot(volsurf_method=int(self.models[box].params.volsurf_method))


class Server:
    """Continuous batching of aggregation runs on one GPU (see include/mcacg.h)."""

    def __init__(self, capacity: int, memory_budget: int = 0, stream: int | None = None,
                 keep_final_states: bool = False):
        self._s = C.c_void_p()
        check(lib().mcacg_server_create(int(capacity), int(memory_budget), C.c_void_p(stream) if stream else None,
                                        1 if keep_final_states else 0, C.byref(self._s)))

    def close(self) -> None:
        if self._s:
            check(lib().mcacg_server_destroy(self._s))
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_threads(self, threads: int) -> None:
        """Threads per box of the epochs (32, 64, 128, 256 or 512; 0: at each
        epoch the largest size at which every active run is resident)."""
        check(lib().mcacg_server_set_threads(self._s, int(threads)))

    def set_epoch_ms(self, ms: float) -> None:
        """Wall-time cap of an epoch (0: each box does all its epoch steps)."""
        check(lib().mcacg_server_set_epoch_ms(self._s, float(ms)))

    def submit(self, model: PhysicalModel) -> int:
        rid = C.c_int64()
        check(lib().mcacg_server_submit(self._s, C.byref(model.params), C.byref(rid)))
        return rid.value

    def step(self, epoch_steps: int) -> tuple[int, int]:
        a, p = C.c_int32(), C.c_int32()
        check(lib().mcacg_server_step(self._s, int(epoch_steps), C.byref(a), C.byref(p)))
        return a.value, p.value

    def poll(self, max_items: int = 4096) -> np.ndarray:
        buf = np.zeros(max_items, dtype=_lib.COMPLETION_DTYPE)
        n = C.c_int32()
        check(lib().mcacg_server_poll(self._s, buf.ctypes.data, int(max_items), C.byref(n)))
        return buf[:n.value].copy()

    def final_state(self, rid: int) -> Snapshot:
        ns, na = C.c_int64(), C.c_int64()
        check(lib().mcacg_server_final_sizes(self._s, int(rid), C.byref(ns), C.byref(na)))
        sb = StateBuffers(ns.value, max(na.value, 1))
        check(lib().mcacg_server_final_state(self._s, int(rid), C.byref(sb.state)))
        return sb.to_snapshot()

    def kernel_time(self) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_int32()
        check(lib().mcacg_server_kernel_time(self._s, C.byref(ms), C.byref(n)))
        return ms.value, n.value


def run_device(aggregates: AggregatList, max_steps: int = 0) -> RunStats:
    """Advance one box with the device-resident loop."""
    s = RunStats()
    check(lib().mcacg_run_device(aggregates._box, int(max_steps), C.byref(s)))
    return s


def calcul(model: PhysicalModel, aggregates: AggregatList, max_steps: int = 0, advancement=None):
    """mcac::calcul (src/calcul.cpp:55-290): collisions, with surface growth or
    oxidation when the model asks for them."""
    return aggregates.calcul(max_steps=max_steps, advancement=advancement)


__all__ = ["PhysicalModel", "AggregatList", "AggregateContactInfo", "init_state", "calcul", "device_count",
           "_lib", "math"]
