"""Batched sweeps: the seeded instance set, and (``-m gpu``) batched = looped = ``run`` bit for
bit, since each instance's arithmetic does not depend on what runs beside it."""

from __future__ import annotations

import numpy as np
import pytest

from open_analysis_gb300.structures import line_instance, sweep_instances, sweep_params


def test_sweep_parameters_are_seeded_and_in_range() -> None:
    a, b = sweep_params(64), sweep_params(64)
    assert a == b and sweep_params(8, seed=1) != sweep_params(8, seed=2)
    for p in a:
        assert 80 <= p.nx <= 240 and 40 <= p.ny <= 120 and 30 <= p.nz <= 80
        assert 0.1e-3 <= p.width <= 0.6e-3 and 0.1e-3 <= p.height <= 0.4e-3
        assert 3.0 <= p.eps_inf <= 4.8 and 0.1 <= p.delta_eps <= 0.5 and 2e-12 <= p.tau <= 20e-12
    assert {p.stripline for p in a} == {True, False}


def test_instances_compile_with_debye_cpml_and_two_ports() -> None:
    from open_analysis_gb300.model import compile_model

    for m in sweep_instances(3):
        c = compile_model(m, "float32")
        assert c.batch == 2 and c.ade is not None and c.frequencies.size == 128
        assert len(c.pml.corrections) > 0


@pytest.mark.gpu
def test_batched_equals_looped_equals_run() -> None:
    from open_analysis_gb300.batch import SWEEP_TILES, compile_all, run_batched, run_looped, tune_shape
    from open_analysis_gb300.run import run, sparams

    params = sweep_params(6, seed=7)
    small = [p.__class__(**{**p.__dict__, "nx": p.nx // 2, "ny": p.ny // 2, "nz": p.nz // 2 + 8}) for p in params]
    models = [line_instance(p, n_freq=16) for p in small]
    compiled = compile_all(models, workers=1)
    steps = 300
    shape = tune_shape(compiled)
    assert shape is not None and shape.tile_z in SWEEP_TILES and shape.variant == 2
    a = run_batched(models, compiled, steps, shape=shape)
    b = run_looped(models, compiled, steps)  # default shape: launch shapes do not change results
    for sa, sb in zip(a.s, b.s, strict=True):
        assert np.array_equal(sa, sb)
    one = run(models[0], engine="gb300", dtype="float32", end_db=None, max_steps=steps)
    assert np.array_equal(sparams(models[0], one), a.s[0])
    assert a.cell_updates == b.cell_updates > 0
