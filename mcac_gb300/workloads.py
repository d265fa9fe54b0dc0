"""Seeded synthetic workloads with the shapes of the benchmark cases.

``contact_search_case`` is the contact-search microbenchmark: a snapshot of
ballistic aggregates (``synthetic_state``) and a list of queries, each an
aggregate label drawn uniformly, a unit direction drawn with the reference's
``random_direction`` formula (src/tools/tools.cpp:82-89: theta = 2 pi u1,
phi = acos(1 - 2 u2)) and a length equal to that aggregate's mean free path
``lpm`` (aggregat.cpp:247-282). Random numbers come from numpy's PCG64, not
the C library, so the queries are the same on every host.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .api import PhysicalModel, synthetic_state
from ._lib import StateBuffers
from .snapshot import A


def contact_search_ini(n_spheres: int, seed: int = 1, sigma_geo: float = 1.5, volume_fraction: float = 5e-3) -> str:
    return (f"[monomers]\nnumber = {n_spheres}\nmean_diameter = 30\ndispersion_diameter = {sigma_geo}\n"
            f"initialisation_mode = lognormal\n[environment]\nvolume_fraction = {volume_fraction}\n"
            f"temperature = 1700\n[numerics]\nrandom_seed = {seed}\nwith_domain_duplication = false\n")


@dataclass
class ContactSearchCase:
    model: PhysicalModel
    state: StateBuffers
    sources: np.ndarray     # int64 labels
    directions: np.ndarray  # [n, 3]
    distances: np.ndarray


def random_directions(rng: np.random.Generator, n: int) -> np.ndarray:
    u1, u2 = rng.random(n), rng.random(n)
    theta = u1 * 2 * np.pi
    phi = np.arccos(1 - 2 * u2)
    return np.stack([np.sin(phi) * np.cos(theta), np.sin(phi) * np.sin(theta), np.cos(phi)], axis=1)


def contact_search_case(n_spheres: int = 1_000_000, n_aggregates: int = 20_000, max_size: int = 500,
                        n_queries: int = 10_000, seed: int = 1, sigma_geo: float = 1.5,
                        volume_fraction: float = 5e-3) -> ContactSearchCase:
    model = PhysicalModel(text=contact_search_ini(n_spheres, seed, sigma_geo, volume_fraction))
    sb = synthetic_state(model, n_aggregates, max_size)
    rng = np.random.Generator(np.random.PCG64(seed))
    na = int(sb.state.n_aggregates)
    src = rng.integers(0, na, n_queries).astype(np.int64)
    dirs = random_directions(rng, n_queries)
    dist = sb.aggregates[A["lpm"], src].copy()
    return ContactSearchCase(model, sb, src, dirs, dist)
