"""Launch-shape autotuner for the sweeps.

Each block of a sweep marches ``tile_z`` planes; longer marches amortise the pipeline prologue
and the carried-plane reload, shorter ones expose more blocks. Four sweep variants exist: the
fused H + E sweep of the interior (3), planes staged through shared memory by TMA tensor copies
(2) or by cp.async (1), or marched in registers (0). The best point depends on the grid and the
batch. :func:`tune` times each candidate on the
engine itself with CUDA events (a few 64-step chunks after one warm-up chunk, which also captures
the graph of that shape) and leaves the fastest shape set on the engine. Timing steps advance
the engine: tune a scratch engine of the same problem, or account for the steps taken.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any

TILES = (4, 8, 16, 24, 32, 64)
FUSED_TILES = (8, 16, 32, 64, 128)  # the fused sweep recomputes one plane per march: longer ones
VARIANTS = (3, 2, 1, 0)  # fused, staged by TMA, staged by cp.async, register marching


@dataclass(frozen=True)
class TuneResult:
    tile_z: int
    variant: int
    ms_per_step: float
    table: dict[tuple[int, int], float]


def _candidates(tiles: tuple[int, ...], variants: tuple[int, ...]) -> list[tuple[int, int]]:
    # variant 0 runs the slab kernel alone, whose march does not depend on the tile; the fused
    # sweep takes its own, longer marches unless the caller gives tiles
    out = []
    for v in variants:
        vt = tiles[:1] if v == 0 else (FUSED_TILES if v == 3 and tiles == TILES else tiles)
        out.extend((tz, v) for tz in vt)
    return out


def tune(engine: Any, chunks: int = 2, tiles: tuple[int, ...] = TILES, variants: tuple[int, ...] = VARIANTS) -> TuneResult:
    """Time every (tile, variant); needs ``(1 + chunks) * 64`` steps each. A variant the engine
    refuses (TMA staging where the driver encoded no descriptors, the fused sweep where the
    interior is empty) is skipped."""
    from open_analysis_gb300.model import ModelError

    table: dict[tuple[int, int], float] = {}
    for cand in _candidates(tiles, variants):
        try:
            engine.set_tuning(*cand)
        except ModelError:
            continue
        engine.step_timed(64)  # capture the graph of this shape
        ms = sum(engine.step_timed(64) for _ in range(chunks))
        table[cand] = ms / (64 * chunks)
    best = min(table, key=table.__getitem__)
    engine.set_tuning(*best)
    return TuneResult(best[0], best[1], table[best], table)


def steps_needed(chunks: int = 2, tiles: tuple[int, ...] = TILES, variants: tuple[int, ...] = VARIANTS) -> int:
    return len(_candidates(tiles, variants)) * (1 + chunks) * 64
