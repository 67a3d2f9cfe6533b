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

BULK = (8, 12, 16, 24, 32, 48)
SLAB = (2, 4, 8)


@dataclass(frozen=True)
class TuneResult:
    tile_z: int
    tile_z_slab: int
    ms_per_step: float
    table: dict[tuple[int, int], float]


def tune(engine: Any, chunks: int = 2, bulk: tuple[int, ...] = BULK, slab: tuple[int, ...] = SLAB) -> TuneResult:
    """Time every (bulk, slab) pair; needs ``(1 + chunks) * 64`` free steps per pair."""
    table: dict[tuple[int, int], float] = {}
    for tz in bulk:
        for ts in slab:
            engine.set_tuning(tz, ts)
            engine.step_timed(64)  # capture the graph of this shape
            ms = sum(engine.step_timed(64) for _ in range(chunks))
            table[(tz, ts)] = ms / (64 * chunks)
    best = min(table, key=table.__getitem__)
    engine.set_tuning(*best)
    return TuneResult(best[0], best[1], table[best], table)


def steps_needed(chunks: int = 2, bulk: tuple[int, ...] = BULK, slab: tuple[int, ...] = SLAB) -> int:
    return len(bulk) * len(slab) * (1 + chunks) * 64
