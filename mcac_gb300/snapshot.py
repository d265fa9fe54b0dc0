"""Box state ("snapshot") layout shared by the C-ABI, the tests and the oracle.

A snapshot is the complete state of one MCAC box: the sphere storage
(9 FP64 columns, ``SpheresFields`` in the reference's include/constants.hpp:34-45),
the owning aggregate of every sphere, the aggregate storage (21 FP64 columns,
``AggregatesFields``, include/constants.hpp:46-69), each aggregate's ordered
sphere list (``Aggregate::myspheres``, include/aggregats/aggregat.hpp:110) and
its Verlet cell (aggregat.cpp:699-705).

Binary layout (little endian), identical to what the oracle harness writes:

    char[8]  "MCSNAP01"
    int64    n_spheres, n_aggregates, n_verlet_divisions
    float64  box_length, maxradius, time
    float64  temperature, pressure, density, viscosity, gaz_mean_free_path,
             fractal_dimension, fractal_prefactor, mean_massic_radius,
             friction_exponnant
    int64    volsurf_method
    float64  spheres[9][n_spheres]        (field-major)
    int64    sphere_label[n_spheres]
    float64  aggregates[21][n_aggregates] (field-major)
    int64    n_spheres_per_aggregate[n_aggregates]
    int64    members[sum(n_spheres_per_aggregate)]
    int64    verlet_cell[n_aggregates][3]
"""
from __future__ import annotations

import dataclasses
import io
from pathlib import Path

import numpy as np

MAGIC = b"MCSNAP01"

SPHERE_FIELDS = ("x", "y", "z", "r", "volume", "surface", "rx", "ry", "rz")
AGGREGATE_FIELDS = (
    "rg", "f_agg", "lpm", "time_step", "rmax", "volume", "surface",
    "x", "y", "z", "rx", "ry", "rz", "time", "dp", "dg_over_dp",
    "overlapping", "coordination_number", "electric_charge", "d_m", "ch_ratio",
)
PHYSICS_FIELDS = (
    "temperature", "pressure", "density", "viscosity", "gaz_mean_free_path",
    "fractal_dimension", "fractal_prefactor", "mean_massic_radius", "friction_exponnant",
)
A = {name: i for i, name in enumerate(AGGREGATE_FIELDS)}
S = {name: i for i, name in enumerate(SPHERE_FIELDS)}


@dataclasses.dataclass
class Snapshot:
    n_div: int
    box_length: float
    maxradius: float
    time: float
    physics: np.ndarray          # float64[9], PHYSICS_FIELDS order
    volsurf_method: int
    spheres: np.ndarray          # float64[9, n_spheres]
    sphere_label: np.ndarray     # int64[n_spheres]
    aggregates: np.ndarray       # float64[21, n_aggregates]
    n_spheres: np.ndarray        # int64[n_aggregates]
    members: np.ndarray          # int64[sum(n_spheres)]
    cells: np.ndarray            # int64[n_aggregates, 3]

    @property
    def ns(self) -> int:
        return int(self.spheres.shape[1])

    @property
    def na(self) -> int:
        return int(self.aggregates.shape[1])

    def member_offsets(self) -> np.ndarray:
        off = np.zeros(self.na + 1, dtype=np.int64)
        np.cumsum(self.n_spheres, out=off[1:])
        return off

    def members_of(self, label: int) -> np.ndarray:
        off = self.member_offsets()
        return self.members[off[label]:off[label + 1]]

    def copy(self) -> "Snapshot":
        return dataclasses.replace(
            self,
            physics=self.physics.copy(), spheres=self.spheres.copy(),
            sphere_label=self.sphere_label.copy(), aggregates=self.aggregates.copy(),
            n_spheres=self.n_spheres.copy(), members=self.members.copy(), cells=self.cells.copy(),
        )

    # -- (de)serialisation -------------------------------------------------
    def to_bytes(self) -> bytes:
        out = io.BytesIO()
        out.write(MAGIC)
        out.write(np.array([self.ns, self.na, self.n_div], dtype="<i8").tobytes())
        out.write(np.array([self.box_length, self.maxradius, self.time], dtype="<f8").tobytes())
        out.write(np.asarray(self.physics, dtype="<f8").tobytes())
        out.write(np.array([self.volsurf_method], dtype="<i8").tobytes())
        out.write(np.ascontiguousarray(self.spheres, dtype="<f8").tobytes())
        out.write(np.ascontiguousarray(self.sphere_label, dtype="<i8").tobytes())
        out.write(np.ascontiguousarray(self.aggregates, dtype="<f8").tobytes())
        out.write(np.ascontiguousarray(self.n_spheres, dtype="<i8").tobytes())
        out.write(np.ascontiguousarray(self.members, dtype="<i8").tobytes())
        out.write(np.ascontiguousarray(self.cells, dtype="<i8").tobytes())
        return out.getvalue()

    def save(self, path: str | Path) -> None:
        Path(path).write_bytes(self.to_bytes())

    def to_npz_dict(self, prefix: str = "") -> dict:
        return {
            prefix + "header_i": np.array([self.n_div, self.volsurf_method], dtype=np.int64),
            prefix + "header_f": np.array([self.box_length, self.maxradius, self.time], dtype=np.float64),
            prefix + "physics": self.physics,
            prefix + "spheres": self.spheres,
            prefix + "sphere_label": self.sphere_label,
            prefix + "aggregates": self.aggregates,
            prefix + "n_spheres": self.n_spheres,
            prefix + "members": self.members,
            prefix + "cells": self.cells,
        }

    @classmethod
    def from_npz(cls, data, prefix: str = "") -> "Snapshot":
        hi = data[prefix + "header_i"]
        hf = data[prefix + "header_f"]
        return cls(
            n_div=int(hi[0]), volsurf_method=int(hi[1]),
            box_length=float(hf[0]), maxradius=float(hf[1]), time=float(hf[2]),
            physics=np.array(data[prefix + "physics"], dtype=np.float64),
            spheres=np.array(data[prefix + "spheres"], dtype=np.float64),
            sphere_label=np.array(data[prefix + "sphere_label"], dtype=np.int64),
            aggregates=np.array(data[prefix + "aggregates"], dtype=np.float64),
            n_spheres=np.array(data[prefix + "n_spheres"], dtype=np.int64),
            members=np.array(data[prefix + "members"], dtype=np.int64),
            cells=np.array(data[prefix + "cells"], dtype=np.int64).reshape(-1, 3),
        )

    @classmethod
    def from_bytes(cls, buf: bytes) -> "Snapshot":
        if buf[:8] != MAGIC:
            raise ValueError("not an MCAC snapshot")
        pos = 8

        def take(dtype, count):
            nonlocal pos
            arr = np.frombuffer(buf, dtype=dtype, count=count, offset=pos)
            pos += arr.nbytes
            return arr.copy()

        ns, na, n_div = (int(v) for v in take("<i8", 3))
        box_length, maxradius, time = (float(v) for v in take("<f8", 3))
        physics = take("<f8", 9)
        volsurf = int(take("<i8", 1)[0])
        spheres = take("<f8", 9 * ns).reshape(9, ns)
        sphere_label = take("<i8", ns)
        aggregates = take("<f8", 21 * na).reshape(21, na)
        n_spheres = take("<i8", na)
        members = take("<i8", int(n_spheres.sum()))
        cells = take("<i8", 3 * na).reshape(na, 3)
        return cls(n_div, box_length, maxradius, time, physics, volsurf, spheres, sphere_label,
                   aggregates, n_spheres, members, cells)

    @classmethod
    def load(cls, path: str | Path) -> "Snapshot":
        return cls.from_bytes(Path(path).read_bytes())


# Per-step record written by the oracle harness (trace mode) and by the
# C-ABI's traced runs: one fixed-size row per MC step.
STEP_DTYPE = np.dtype([
    ("step", "<i8"), ("picked", "<i8"), ("contact", "<i8"), ("merged", "<i8"),
    ("moving_sphere", "<i8"), ("other_sphere", "<i8"), ("moving_agg", "<i8"), ("other_agg", "<i8"),
    ("n_agg_after", "<i8"), ("deltatemps", "<f8"), ("full_distance", "<f8"), ("dir", "<f8", 3),
    ("contact_distance", "<f8"), ("move_distance", "<f8"), ("time_after", "<f8"), ("reserved", "<f8"),
])

# Query record: inputs of AggregatList::distance_to_next_contact and its answer.
QUERY_DTYPE = np.dtype([
    ("label", "<i8"), ("moving_sphere", "<i8"), ("other_sphere", "<i8"),
    ("moving_agg", "<i8"), ("other_agg", "<i8"), ("contact", "<i8"),
    ("dir", "<f8", 3), ("distance", "<f8"), ("contact_distance", "<f8"), ("reserved", "<f8"),
])


def read_merge_records(path: str | Path, with_spheres: bool) -> list[dict]:
    """Merge records of the oracle harness ('merges' mode when with_spheres)."""
    buf = Path(path).read_bytes()
    pos = 0
    out = []
    while pos < len(buf):
        if with_spheres:
            q, merged, keep, n = np.frombuffer(buf, "<i8", 4, pos)
            pos += 32
        else:
            q, keep, n = np.frombuffer(buf, "<i8", 3, pos)
            merged = 1
            pos += 24
        rec = np.frombuffer(buf, "<f8", 21, pos).copy()
        pos += 21 * 8
        maxradius = float(np.frombuffer(buf, "<f8", 1, pos)[0])
        pos += 8
        item = {"index": int(q), "merged": int(merged), "keep": int(keep), "n": int(n),
                "record": rec, "maxradius": maxradius}
        if with_spheres:
            item["time"] = float(np.frombuffer(buf, "<f8", 1, pos)[0])
            pos += 8
            rows = np.frombuffer(buf, dtype=np.dtype([("id", "<i8"), ("f", "<f8", 9)]), count=int(n), offset=pos)
            pos += rows.nbytes
            item["sphere_ids"] = rows["id"].copy()
            item["sphere_rows"] = rows["f"].copy()
        out.append(item)
    return out
