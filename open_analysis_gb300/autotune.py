"""Launch-shape autotuner for the sweeps.

The sweeps march every thread up ``tile_z`` planes (bulk launch) or ``tile_z_slab`` planes (CPML
slab launches). Longer marches amortise the carried-plane reload, shorter ones expose more blocks;
the best point depends on the grid and the batch. :func:`tune` times each candidate on the
engine itself with CUDA events (a few 64-step chunks after one warm-up chunk, which also captures
the graph of that shape) and leaves the fastest shape set on the engine. Timing steps advance
the engine: tune a scratch engine of the same problem, or account for the steps taken.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any

BULK = (8, 16, 24, 32, 48)
SLAB = (2, 4, 8)
VARIANTS = (1, 0)  # shared-memory staged bulk sweeps, register marching


@dataclass(frozen=True)
class TuneResult:
    tile_z: int
    tile_z_slab: int
    variant: int
    ms_per_step: float
    table: dict[tuple[int, int, int], float]


def _candidates(bulk: tuple[int, ...], slab: tuple[int, ...], variants: tuple[int, ...]) -> list[tuple[int, int, int]]:
    return [(tz, ts, v) for v in variants for tz in bulk for ts in slab]


def tune(
    engine: Any,
    chunks: int = 2,
    bulk: tuple[int, ...] = BULK,
    slab: tuple[int, ...] = SLAB,
    variants: tuple[int, ...] = VARIANTS,
) -> TuneResult:
    """Time every (bulk tile, slab tile, variant); needs ``(1 + chunks) * 64`` steps each."""
    table: dict[tuple[int, int, int], float] = {}
    for cand in _candidates(bulk, slab, variants):
        engine.set_tuning(*cand)
        engine.step_timed(64)  # capture the graph of this shape
        ms = sum(engine.step_timed(64) for _ in range(chunks))
        table[cand] = ms / (64 * chunks)
    best = min(table, key=table.__getitem__)
    engine.set_tuning(*best)
    return TuneResult(best[0], best[1], best[2], table[best], table)


def steps_needed(
    chunks: int = 2, bulk: tuple[int, ...] = BULK, slab: tuple[int, ...] = SLAB, variants: tuple[int, ...] = VARIANTS
) -> int:
    return len(_candidates(bulk, slab, variants)) * (1 + chunks) * 64
