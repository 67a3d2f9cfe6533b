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
    assert shape is not None and shape.tile_z in SWEEP_TILES and shape.variant in (2, 3)
    a = run_batched(models, compiled, steps, shape=shape)
    b = run_looped(models, compiled, steps)  # default shape: launch shapes do not change results
    for sa, sb in zip(a.s, b.s, strict=True):
        assert np.array_equal(sa, sb)
    one = run(models[0], engine="gb300", dtype="float32", end_db=None, max_steps=steps)
    assert np.array_equal(sparams(models[0], one), a.s[0])
    assert a.cell_updates == b.cell_updates > 0


def _mode_sweep(n: int = 3) -> list:  # type: ignore[type-arg]
    """Mode-port striplines with wave planes (the ``mode_stripline`` case), the fill's eps_inf
    varied per instance."""
    from dataclasses import replace

    from cases import CASES, namespace

    out = []
    for i in range(n):
        m = CASES["mode_stripline"][0](namespace("gb300"))
        m.regions[0] = replace(m.regions[0], eps_r=3.0 + 0.4 * i)
        out.append(m)
    return out


def test_sweep_results_use_wave_planes_and_write_worker_files(tmp_path) -> None:  # type: ignore[no-untyped-def]
    """On the oracle: a sweep instance with mode ports and wave planes reports the wave-plane S
    (the worker's choice, ``adapter/sim.py:184-198``), and each instance's ``ports.npz``,
    ``run.json`` and Touchstone file carry that S as the adapter reads it."""
    import json

    from open_analysis_gb300.batch import collect, finish_sweep, instance_sparams
    from open_analysis_gb300.deembed import wave_sparams
    from open_analysis_gb300.run import port_voltage_factor, sparams
    from oracle.numpy_engine import OracleEngine

    models = _mode_sweep(2)
    compiled = [compile_model_f32(m) for m in models]
    steps = 300
    engines = []
    for c in compiled:
        e = OracleEngine(c, "float32")
        e.step(steps)
        engines.append(e)
    res = [collect(m, c, e, steps, "float32") for m, c, e in zip(models, compiled, engines, strict=True)]
    run = finish_sweep(models, compiled, engines, steps, "float32", 1.0, 0.0, wire_dir=tmp_path)
    for m, r, s in zip(models, res, run.s, strict=True):
        s_port = sparams(m, r)
        fac = port_voltage_factor(r.dt, m.frequencies)
        want, _ = wave_sparams({k: v * fac for k, v in r.probes.items()}, m.plane_sets, r.port_r, s_port=s_port,
                               freqs=m.frequencies)
        assert np.array_equal(s, want) and np.array_equal(instance_sparams(m, r), want)
        assert not np.array_equal(s, s_port)
    for n, files in enumerate(run.extra["wire"]):
        with np.load(files["wire"]) as z:
            assert np.array_equal(z["s"], np.moveaxis(run.s[n], -1, 0))
            assert np.array_equal(z["freqs"], models[n].frequencies)
            assert list(z["names"]) == [p.name for p in models[n].ports]
        meta = json.loads(open(files["run_json"]).read())
        assert meta["steps"] == steps and meta["port_names"] == ["p1", "p2"]
        assert files["touchstone"].endswith(".s2p")


def compile_model_f32(m):  # type: ignore[no-untyped-def]
    from open_analysis_gb300.model import compile_model

    return compile_model(m, "float32")


@pytest.mark.gpu
def test_batched_mode_port_sweep_equals_looped(tmp_path) -> None:  # type: ignore[no-untyped-def]
    """Wave planes on the batched path: batched = looped bit for bit, wire files included."""
    from open_analysis_gb300.batch import compile_all, run_batched, run_looped

    models = _mode_sweep(3)
    compiled = compile_all(models, workers=1)
    a = run_batched(models, compiled, 400, wire_dir=tmp_path / "batched")
    b = run_looped(models, compiled, 400, wire_dir=tmp_path / "looped")
    for sa, sb in zip(a.s, b.s, strict=True):
        assert np.array_equal(sa, sb)
    for fa, fb in zip(a.extra["wire"], b.extra["wire"], strict=True):
        with np.load(fa["wire"]) as za, np.load(fb["wire"]) as zb:
            assert np.array_equal(za["s"], zb["s"])


def _small_instances(n: int, seed: int = 11):  # type: ignore[no-untyped-def]
    params = sweep_params(n, seed=seed)
    small = [p.__class__(**{**p.__dict__, "nx": p.nx // 2, "ny": p.ny // 2, "nz": p.nz // 2 + 8}) for p in params]
    return [line_instance(p, n_freq=16) for p in small]


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [150, 71])
def test_engine_batch_fields_equal_engines_stepped_alone(steps: int) -> None:
    """The native batch (one launch per kernel class over all instances) against every engine
    stepped on its own: all six fields, the probe DFTs and the energy bit for bit. The instances
    differ in size and in sweep variant (fused, TMA-staged, register marching, one tile height
    each), so the batch splits into one native batch per variant; 150 steps take two graph
    chunks and 22 eager steps (an even and an odd count leave the fused variant's buffers
    swapped differently)."""
    from open_analysis_gb300.batch import EngineBatch, compile_all
    from open_analysis_gb300.engine import Gb300Engine
    from open_analysis_gb300.model import ModelError

    models = _small_instances(5)
    compiled = compile_all(models, workers=1)
    shapes = [(16, 3), (8, 3), (8, 2), (4, 2), (16, 0)]

    def make() -> list:  # type: ignore[type-arg]
        out = []
        for c, (tz, v) in zip(compiled, shapes, strict=True):
            e = Gb300Engine(c, "float32", max_steps=steps + 10)
            try:
                e.set_tuning(tz, v)
            except ModelError:  # no fused box in this instance: the TMA-staged sweeps
                e.set_tuning(tz, 2)
            out.append(e)
        return out

    alone, grouped = make(), make()
    for e in alone:
        e.step(steps)
    batch = EngineBatch(grouped)
    assert len(batch.handles) == len({e.get_tuning()[1] for e in grouped}) >= 2
    batch.step_async(steps - 7)
    batch.step(7)
    assert batch.graph_kernels() > 0
    for a, b in zip(alone, grouped, strict=True):
        assert a.step_count == b.step_count == steps
        for k in range(6):
            assert np.array_equal(a.field(k), b.field(k)), k
        ra, rb = a.results(), b.results()
        assert ra.keys() == rb.keys()
        for key in ra:
            assert np.array_equal(ra[key], rb[key]), key
        assert a.energy() == b.energy()
    batch.close()
    for e in alone + grouped:
        e.close()


@pytest.mark.gpu
def test_engine_batch_refuses_out_of_step_engines() -> None:
    """Host-side checks: engines at different steps cannot form a batch, and an engine stepped on
    its own while in a batch stops the batch with FDTD_BAD_INPUT instead of racing it."""
    from open_analysis_gb300.batch import EngineBatch, compile_all
    from open_analysis_gb300.engine import Gb300Engine
    from open_analysis_gb300.model import ModelError

    compiled = compile_all(_small_instances(2), workers=1)
    e1, e2 = (Gb300Engine(c, "float32", max_steps=200) for c in compiled)
    e1.set_tuning(8, 2)
    e2.set_tuning(8, 2)
    e1.step(3)
    with pytest.raises(ModelError):
        EngineBatch([e1, e2])
    e2.step(3)
    batch = EngineBatch([e1, e2])
    batch.step(5)
    e1.step(1)
    with pytest.raises(ModelError):
        batch.step(1)
    batch.close()
    e1.close()
    e2.close()


@pytest.mark.gpu
def test_stream_launches_equal_batched_launches() -> None:
    from open_analysis_gb300.batch import compile_all, run_batched

    models = _small_instances(4, seed=5)
    compiled = compile_all(models, workers=1)
    a = run_batched(models, compiled, 200, launch="batch")
    b = run_batched(models, compiled, 200, launch="streams")
    assert a.extra["launch"] == "batch" and a.extra["graph_kernels_per_chunk"] > 0
    for sa, sb in zip(a.s, b.s, strict=True):
        assert np.array_equal(sa, sb)
