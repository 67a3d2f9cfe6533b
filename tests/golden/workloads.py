"""The benchmark workloads as parity cases, shared by the fixture generator and the GPU tests.

Each workload is one of ``open_analysis_gb300.structures``' builders at the size a parity test runs
it (the configured size where the reference's NumPy engine finishes it in minutes on one host
thread), with the number of time steps and whether it starts from seeded fields:

* ``microstrip_120x60x40``: the plain microstrip exactly as configured, 2000 steps from rest;
* ``via_transition_400x400x120``: the via transition at full size (Debye stack, SIBC copper,
  10-cell CPML, batch 2, 256 frequencies), 200 steps from seeded fields, so that every CPML
  slab, Debye edge and surface-impedance edge is active from the first step;
* ``large_board_200x150x80``: the large-board structure (eight Debye layers, SIBC traces and vias,
  12-cell CPML, eight ports driven as a batch of eight, 512 frequencies) on a 200 x 150 x 80
  grid, 20 steps from seeded fields.

``convert`` rebuilds a model from another set of problem types (the reference's, when the fixtures
are made), field by field. ``seeded_values`` gives field values from a counter-based generator
(SplitMix64 over the element index, Steele, Lea and Flood 2014) in integer arithmetic, so the
same seed gives the same float32 values on every host and NumPy version.
"""

from __future__ import annotations

import dataclasses
from typing import Any

import numpy as np

NAMES = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _structures() -> Any:
    from open_analysis_gb300 import structures

    return structures


def workloads() -> dict[str, dict[str, Any]]:
    """name -> {"model": builder (no arguments), "steps": int, "seed": int or None}."""
    st = _structures()
    return {
        "microstrip_120x60x40": {"model": st.microstrip, "steps": 2000, "seed": None},
        "via_transition_400x400x120": {"model": st.via_transition, "steps": 200, "seed": 2026},
        "large_board_200x150x80": {
            "model": lambda: st.large_board(nx=200, ny=150, nz=80),
            "steps": 20,
            "seed": 2027,
        },
    }


def _splitmix64(x: np.ndarray) -> np.ndarray:
    z = x + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def seeded_values(shape: tuple[int, ...], seed: int, stream: int) -> np.ndarray:
    """float32 values uniform in [-1, 1) on a 2^-23 lattice for one field component."""
    n = int(np.prod(shape))
    base = np.uint64((seed * 64 + stream) << 36)
    with np.errstate(over="ignore"):
        z = _splitmix64(np.arange(n, dtype=np.uint64) + base)
    v = (z >> np.uint64(40)).astype(np.float32) * np.float32(2.0**-23) - np.float32(1.0)
    return v.reshape(shape)


def sample_index(size: int, count: int, seed: int) -> np.ndarray:
    """``count`` distinct flat indices below ``size`` (sorted), from the same generator."""
    with np.errstate(over="ignore"):
        z = _splitmix64(np.arange(4 * count, dtype=np.uint64) + np.uint64(seed << 40))
    vals = (z % np.uint64(size)).astype(np.int64)
    _, first = np.unique(vals, return_index=True)
    return np.sort(vals[np.sort(first)][:count])


def convert(obj: Any, ns: Any) -> Any:
    """A copy of ``obj`` (a model or one of its parts) built from the types in ``ns``; objects of
    other types (a waveform class of the caller's own, NumPy arrays, numbers) are kept."""
    if isinstance(obj, (list, tuple)) and not isinstance(obj, str):
        out = [convert(v, ns) for v in obj]
        return out if isinstance(obj, list) else tuple(out)
    name = type(obj).__name__
    if name == "Grid" and hasattr(obj, "lines"):
        return ns.Grid(*[np.asarray(v) for v in obj.lines])
    if dataclasses.is_dataclass(obj) and not isinstance(obj, type) and hasattr(ns, name):
        kw = {f.name: convert(getattr(obj, f.name), ns) for f in dataclasses.fields(obj) if f.init}
        return getattr(ns, name)(**kw)
    return obj
