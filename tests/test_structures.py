"""The synthetic benchmark structures build and compile (CPU): the shapes, batches and lists the
bench workloads rely on."""

from __future__ import annotations

import numpy as np

from open_analysis_gb300.model import compile_model
from open_analysis_gb300.structures import large_board, microstrip, via_transition


def test_large_board_has_every_part() -> None:
    m = large_board(nx=200, ny=150, nz=80, n_freq=16)
    c = compile_model(m, "float32")
    assert c.batch == 8 and len(c.ports) == 8
    assert len([r for r in m.regions if not r.pec]) == 8  # eight dielectric layers
    assert len(m.conductors) == 12 * 2 + 40  # 12 L-shaped traces, 40 vias
    assert c.ade is not None and c.ade.tau.size == 1 and sum(f.size for f in c.ade.flat) > 0
    assert c.sibc is not None and c.sibc.flat.size > 1000
    assert len(c.pml.corrections) > 0 and c.frequencies[0] == 0.05e9 and c.frequencies[-1] == 40e9
    eps = {round(r.eps_r, 12) for r in m.regions if not r.pec}
    assert all(3.4 <= e <= 4.2 for e in eps) and len(eps) > 1
    # seeded: the same seed builds the same board
    assert compile_model(large_board(nx=200, ny=150, nz=80, n_freq=16), "float32").sibc.flat.size == c.sibc.flat.size


def test_benchmark_structures_compile() -> None:
    c = compile_model(via_transition(nx=80, ny=80, nz=48, n_freq=8), "float32")
    assert c.batch == 2 and c.ade is not None and c.sibc is not None
    c = compile_model(microstrip(), "float32")
    assert c.batch == 2 and np.isclose(c.frequencies[-1], 20e9)
