"""ctypes wrapper of the C restatement in oracle/mcac_oracle.c.

TEST INFRASTRUCTURE ONLY: the checker of the test suite and the CPU baseline
of bench.py; the product never imports it. The INI reader here follows the
reference's PhysicalModel constructor (src/physical_model/physical_model.cpp:
99-187): first definition of a key wins, missing keys leave defaults.
"""
from __future__ import annotations

import ctypes as C
import multiprocessing as mp
import os
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = ROOT / "oracle" / "_build" / "libmcac_oracle.so"

i32, i64, f64 = C.c_int32, C.c_int64, C.c_double


class MoParams(C.Structure):
    _fields_ = [("n_monomeres", i64), ("density", f64), ("mean_diameter", f64), ("dispersion_diameter", f64),
                ("initialisation_mode", i32), ("random_seed", i32), ("initial_time", f64),
                ("volume_fraction", f64), ("temperature", f64), ("fractal_dimension", f64), ("viscosity", f64),
                ("gaz_mean_free_path", f64), ("box_length", f64), ("n_verlet_divisions", i64),
                ("enforce_volume_fraction", i32), ("with_collisions", i32),
                ("number_of_aggregates_limit", i64), ("n_iter_without_event_limit", i64),
                ("mean_monomere_per_aggregate_limit", i64), ("physical_time_limit", f64),
                ("with_surface_reactions", i32), ("individual_surf_reactions", i32), ("flux_surfgrowth", f64),
                ("u_sg", f64), ("full_aggregate_update_frequency", i64), ("rp_min_oxid", f64)]


class MoContact(C.Structure):
    _fields_ = [("distance", f64), ("moving_sphere", i64), ("other_sphere", i64), ("moving_aggregate", i64),
                ("other_aggregate", i64)]


class MoStats(C.Structure):
    _fields_ = [("steps", i64), ("events", i64), ("n_aggregates", i64), ("time", f64), ("finished", i32),
                ("reserved", i32)]


# one traced MC step: mo_step_record of mcac_oracle.h
STEP_DTYPE = np.dtype([
    ("step", "<i8"), ("picked", "<i8"), ("contact", "<i8"), ("merged", "<i8"),
    ("moving_sphere", "<i8"), ("other_sphere", "<i8"), ("moving_agg", "<i8"), ("other_agg", "<i8"),
    ("n_agg_after", "<i8"), ("deltatemps", "<f8"), ("full_distance", "<f8"), ("dir", "<f8", 3),
    ("contact_distance", "<f8"), ("move_distance", "<f8"), ("time_after", "<f8"), ("reserved", "<f8"),
])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from mcac_gb300 import build
            build.build_oracle()
        L = C.CDLL(str(LIB_PATH))
        P = C.POINTER
        sig = {
            "mo_params_derive": (None, [P(MoParams), f64]),
            "mo_box_new_random": (C.c_int, [P(MoParams), P(C.c_void_p)]),
            "mo_box_new_state": (C.c_int, [P(MoParams), i64, i64, i64, f64, f64, f64, P(f64), P(i64), P(f64),
                                           P(i64), P(i64), P(C.c_void_p)]),
            "mo_box_free": (None, [C.c_void_p]),
            "mo_size": (i64, [C.c_void_p]),
            "mo_n_spheres": (i64, [C.c_void_p]),
            "mo_store": (None, [C.c_void_p, P(f64), P(i64), P(f64), P(i64), P(i64), P(f64)]),
            "mo_distance_to_next_contact": (C.c_int, [C.c_void_p, i64, P(f64), f64, P(MoContact)]),
            "mo_translate": (None, [C.c_void_p, i64, P(f64)]),
            "mo_merge": (C.c_int, [C.c_void_p, P(MoContact), P(i32)]),
            "mo_sort_indices": (None, [P(f64), P(i64), i64]),
            "mo_time": (f64, [C.c_void_p]),
            "mo_set_time": (None, [C.c_void_p, f64]),
            "mo_set_aggregate_limit": (None, [C.c_void_p, i64]),
            "mo_calcul": (C.c_int, [C.c_void_p, i64, C.c_void_p, i64, P(MoStats)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


def parse_ini(text: str) -> dict:
    data: dict = {}
    section = ""
    for raw in text.splitlines():
        line = raw.strip()
        if not line or line[0] in ";#":
            continue
        if line[0] == "[":
            section = line[1:line.index("]")].strip() if "]" in line else section
            continue
        if "=" not in line:
            continue
        k, v = line.split("=", 1)
        data.setdefault(section, {}).setdefault(k.strip(), v.strip())
    return data


def params_from_ini(text: str) -> MoParams:
    ini = parse_ini(text)

    def get(sec, key, conv, default):
        v = ini.get(sec, {}).get(key)
        if v is None or v == "":
            return default
        try:
            if conv is bool:
                if v not in ("true", "false"):
                    return default
                return v == "true"
            return conv(v)
        except ValueError:
            return default

    p = MoParams()
    p.n_monomeres = get("monomers", "number", int, 2500)
    p.density = get("monomers", "density", float, 1800.0)
    p.mean_diameter = get("monomers", "mean_diameter", float, 30.0)
    p.dispersion_diameter = get("monomers", "dispersion_diameter", float, 1.0)
    p.initialisation_mode = {"lognormal": 0, "normal": 1}[get("monomers", "initialisation_mode", str, "lognormal")]
    p.initial_time = get("environment", "initial_time", float, 0.0)
    p.volume_fraction = get("environment", "volume_fraction", float, 1e-3)
    p.temperature = get("environment", "temperature", float, 293.15)
    pressure = get("environment", "pressure", float, 101300.0)
    p.fractal_dimension = get("environment", "fractal_dimension", float, 1.4)
    p.number_of_aggregates_limit = get("limits", "number_of_aggregates", int, 1)
    p.n_iter_without_event_limit = get("limits", "n_iter_without_event", int, -1)
    p.physical_time_limit = get("limits", "physical_time", float, -1.0)
    p.mean_monomere_per_aggregate_limit = get("limits", "mean_monomere_per_aggregate", int, -1)
    p.with_collisions = get("numerics", "with_collisions", bool, True)
    p.enforce_volume_fraction = get("numerics", "enforce_volume_fraction", bool, True)
    p.n_verlet_divisions = get("numerics", "n_verlet_divisions", int, 10)
    p.random_seed = get("numerics", "random_seed", int, -1)
    p.with_surface_reactions = get("surface_growth", "with_surface_reactions", bool, False)
    p.flux_surfgrowth = get("surface_growth", "flux_surfgrowth", float, 0.0)
    p.full_aggregate_update_frequency = get("surface_growth", "full_aggregate_update_frequency", int, 1)
    p.individual_surf_reactions = get("numerics", "individual_surf_reactions", bool, False)
    p.rp_min_oxid = get("oxidation", "rp_min", float, 0.166e-09)
    lib().mo_params_derive(C.byref(p), pressure)
    return p


class OracleBox:
    """One box of the C restatement."""

    def __init__(self, ini_text: str, snap=None):
        self.params = params_from_ini(ini_text)
        self.h = C.c_void_p()
        if snap is None:
            rc = lib().mo_box_new_random(C.byref(self.params), C.byref(self.h))
        else:
            self._keep = [np.ascontiguousarray(a) for a in (snap.spheres, snap.sphere_label, snap.aggregates,
                                                          snap.n_spheres, snap.members)]
            sp, sl, ag, nsph, mem = self._keep
            rc = lib().mo_box_new_state(C.byref(self.params), snap.ns, snap.na, snap.n_div, snap.box_length,
                                        snap.maxradius, snap.time, _p(sp, f64), _p(sl, i64), _p(ag, f64),
                                        _p(nsph, i64), _p(mem, i64), C.byref(self.h))
        if rc != 0:
            raise RuntimeError(f"oracle error {rc}")

    def close(self):
        if self.h:
            lib().mo_box_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        self.close()

    def size(self) -> int:
        return int(lib().mo_size(self.h))

    def distance_to_next_contact(self, label, direction, distance):
        d = np.ascontiguousarray(direction, dtype=np.float64)
        c = MoContact()
        rc = lib().mo_distance_to_next_contact(self.h, int(label), _p(d, f64), float(distance), C.byref(c))
        if rc:
            raise RuntimeError(f"oracle error {rc}")
        return c

    def translate(self, label, vec):
        v = np.ascontiguousarray(vec, dtype=np.float64)
        lib().mo_translate(self.h, int(label), _p(v, f64))

    def merge(self, c: MoContact) -> bool:
        m = C.c_int32()
        rc = lib().mo_merge(self.h, C.byref(c), C.byref(m))
        if rc:
            raise RuntimeError(f"oracle error {rc}")
        return bool(m.value)

    def set_aggregate_limit(self, limit: int) -> None:
        lib().mo_set_aggregate_limit(self.h, int(limit))

    def calcul(self, max_steps=0, trace=False, trace_capacity=0):
        st = MoStats()
        buf = None
        cap = 0
        if trace:
            cap = int(trace_capacity or max_steps or 1_000_000)
            buf = np.zeros(cap, dtype=STEP_DTYPE)
        rc = lib().mo_calcul(self.h, int(max_steps), buf.ctypes.data if buf is not None else None, cap,
                             C.byref(st))
        if rc:
            raise RuntimeError(f"oracle error {rc}")
        return st, (buf[:min(int(st.steps), cap)] if buf is not None else None)

    def store(self):
        from mcac_gb300.snapshot import Snapshot
        ns, na = int(lib().mo_n_spheres(self.h)), self.size()
        sp = np.zeros((9, ns))
        sl = np.zeros(ns, np.int64)
        ag = np.zeros((21, na))
        nsph = np.zeros(na, np.int64)
        mem = np.zeros(ns, np.int64)
        sc = np.zeros(3)
        lib().mo_store(self.h, _p(sp, f64), _p(sl, i64), _p(ag, f64), _p(nsph, i64), _p(mem, i64), _p(sc, f64))
        step = self.params.n_verlet_divisions / sc[2]
        cells = np.stack([np.floor(ag[f] * step) for f in (7, 8, 9)], axis=1).astype(np.int64)
        return Snapshot(n_div=int(self.params.n_verlet_divisions), box_length=float(sc[2]), maxradius=float(sc[0]),
                        time=float(sc[1]), physics=np.zeros(9), volsurf_method=4, spheres=sp, sphere_label=sl,
                        aggregates=ag, n_spheres=nsph, members=mem, cells=cells)


def sort_indices(keys: np.ndarray) -> np.ndarray:
    k = np.ascontiguousarray(keys, dtype=np.float64)
    idx = np.zeros(len(k), dtype=np.int64)
    lib().mo_sort_indices(_p(k, f64), _p(idx, i64), len(k))
    return idx


# ---------------------------------------------------------------- bench
# The CPU legs of bench.py. They use nothing of the product: each box is
# placed by this restatement's own copy of the reference placement
# (mo_box_new_random, bit-identical with the reference's).

def _worker(args):
    ini_text, seconds, chunk = args
    box = OracleBox(ini_text)
    steps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        st, _ = box.calcul(max_steps=chunk)
        steps += int(st.steps)
        if st.finished:
            break
    dt = time.perf_counter() - t0
    box.close()
    return steps, dt


def bench_sample(ini_text: str, seconds: float = 15.0, processes: int = 1, steps: int = 1, warmup: int = 0,
                 chunk: int = 200) -> dict:
    """MC steps/s of the restatement on a bounded sample of the workload.

    Each process places its own copy of the box (the reference placement)
    and advances it for 'seconds' of wall time; with several processes the
    value is the sum of their rates (independent boxes, one per core).
    """
    jobs = [(ini_text, seconds, chunk)] * processes
    if processes == 1:
        res = [_worker(jobs[0])]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(processes) as pool:
            res = pool.map(_worker, jobs)
    total_steps = sum(r[0] for r in res)
    value = sum(r[0] / r[1] for r in res)
    return {"value": value, "unit": "MC steps/s", "cores": processes, "kind": "port",
            "sample": f"{processes} independent copies of the box from the reference initial state, "
                      f"~{seconds:.0f} s of MC steps each ({total_steps} steps in total)",
            "host_cpus": os.cpu_count()}


def run_windows(ini_text: str, agg_limit_a: int, steps_a: int, steps_b: int, final_limit: int) -> dict:
    """One box through the two benchmark windows (calcul.cpp:66-281 each).

    Window a: from the initial placement until at most agg_limit_a
    aggregates are left, steps_a steps are done or a stop criterion of the
    parameters is met. Window b: from there, the next steps_b steps under the
    box's own aggregate criterion final_limit (or fewer, if the box stops).
    Placement is not timed; the steps are (process CPU wall time).
    """
    box = OracleBox(ini_text)
    n0 = box.size()
    box.set_aggregate_limit(agg_limit_a)
    t0 = time.perf_counter()
    sa, _ = box.calcul(max_steps=steps_a)
    t1 = time.perf_counter()
    na = int(sa.n_aggregates)
    box.set_aggregate_limit(final_limit)
    sb, _ = box.calcul(max_steps=steps_b)
    t2 = time.perf_counter()
    out = {"n_aggregates_0": n0, "steps_a": int(sa.steps), "events_a": int(sa.events), "s_a": t1 - t0,
           "n_aggregates_a": na, "steps_b": int(sb.steps), "events_b": int(sb.events), "s_b": t2 - t1,
           "n_aggregates_b": int(sb.n_aggregates), "finished": int(sb.finished)}
    box.close()
    return out


def _window_job(job):
    k, ini_text, agg_limit_a, steps_a, steps_b, final_limit = job
    return k, run_windows(ini_text, agg_limit_a, steps_a, steps_b, final_limit)


def farm_windows(jobs: list, processes: int, pool=None) -> list:
    """run_windows over many boxes on 'processes' host processes (a spawn
    pool: the workers load only this restatement). jobs: (key, ini_text,
    agg_limit_a, steps_a, steps_b, final_limit), submitted in the given order
    (largest first keeps the cores busy to the end); returns (key, result)
    in completion order."""
    if processes <= 1 and pool is None:
        return [_window_job(j) for j in jobs]
    if pool is not None:
        return list(pool.imap_unordered(_window_job, jobs))
    with mp.get_context("spawn").Pool(processes) as p:
        return list(p.imap_unordered(_window_job, jobs))


def window_pool(processes: int):
    """A spawn pool for farm_windows, started before any GPU work."""
    return mp.get_context("spawn").Pool(processes)
