"""Batched parameter sweeps: many independent FDTD instances on one GPU at the same time.

A sweep (the reference runs one problem at a time) is a list of models with different grids.
Each instance gets its own engine, stream and captured 64-step graphs; ``run_batched`` queues all
their steps (``Gb300Engine.step_async``) before waiting on any, so the GPU runs kernels of many
small grids side by side instead of one small grid at a time; ``run_looped`` is the plain way,
one instance after the other (``step`` synchronises). Both give the same S-parameters bit for
bit (each instance's arithmetic does not depend on what runs beside it).

The host compiles the instances in a ``spawn`` process pool before any CUDA call. The launch
shape (planes per block, sweep variant) comes from the project's autotuner
(:func:`open_analysis_gb300.autotune.tune`), run once per sweep on a scratch engine of the
median-size instance (:func:`tune_shape`) and applied to every instance.
"""

from __future__ import annotations

import os
import time
from collections.abc import Sequence
from concurrent.futures import ProcessPoolExecutor
from dataclasses import dataclass, field
from multiprocessing import get_context
from pathlib import Path
from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.model import Compiled, ModePort, Model, compile_model
from open_analysis_gb300.run import RunResult, port_voltage_factor, source_spectrum, sparams

ComplexArray = npt.NDArray[np.complex128]

# Many engines run on many streams; CUDA maps streams onto this many hardware work queues (8 by
# default, so streams beyond 8 share queues and serialise). Takes effect when set before the
# process first uses CUDA.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")


def _compile(args: tuple[Model, str]) -> Compiled:
    return compile_model(*args)


def compile_all(models: Sequence[Model], dtype: str = "float32", workers: int = 8) -> list[Compiled]:
    """Compile every model on the host, in parallel processes (``spawn``: safe before or after
    the process has touched the GPU)."""
    if workers <= 1 or len(models) < 2:
        return [compile_model(m, dtype) for m in models]
    with ProcessPoolExecutor(max_workers=workers, mp_context=get_context("spawn")) as pool:
        return list(pool.map(_compile, [(m, dtype) for m in models]))


def collect(model: Model, c: Compiled, eng: Any, steps: int, dtype: str) -> RunResult:
    """The ``RunResult`` of an engine that ran ``steps`` steps (as ``run`` assembles it: port
    voltage sums, source spectrum, port resistances)."""
    probes = eng.results()
    sums = {f"V:{q['name']}": q["probe_parts"] for q in c.ports if q.get("probe_parts")}
    sums.update(c.probe_sums)
    for name, parts in sums.items():
        probes[name] = sum(probes.pop(q) for q in parts)
    return RunResult(
        probes=probes,
        source_dft=source_spectrum(c, steps),
        steps=steps,
        dt=c.dt,
        engine=eng.name,
        dtype=dtype,
        stopped_by="max_steps",
        energy_db=0.0,
        peak_bytes=eng.peak_bytes(),
        port_r=np.array([float(q["r_ohm"]) for q in c.ports]),
    )


def instance_sparams(model: Model, res: RunResult) -> ComplexArray:
    """S-parameters of one instance as the worker reports them (``adapter/sim.py:184-198``): the
    port S, or, where every port is a mode port and the model has wave planes
    (``deembed.add_wave_planes``), the wave-plane S (``deembed.wave_sparams``, the port voltages
    mapped by the port voltage factor) with the port S where the planes are ill-conditioned."""
    s_port = sparams(model, res)
    planes = getattr(model, "plane_sets", None)
    if not planes or not model.ports or not all(isinstance(p, ModePort) for p in model.ports):
        return s_port
    from open_analysis_gb300.deembed import wave_sparams

    fac = port_voltage_factor(res.dt, model.frequencies)
    probes = {k: v * fac for k, v in res.probes.items()}
    s_wave, _ = wave_sparams(probes, planes, res.port_r, s_port=s_port, freqs=model.frequencies)
    return s_wave


@dataclass
class SweepRun:
    """S-parameters of every instance (``(N, N, F)`` each), the time of the stepping and of the
    result read-back [s], the time to create the engines [s], and the cell-updates done."""

    s: list[ComplexArray]
    seconds: float
    create_seconds: float
    cell_updates: float
    extra: dict[str, Any] = field(default_factory=dict)

    @property
    def sweeps_per_s(self) -> float:
        return len(self.s) / self.seconds


SWEEP_TILES = (4, 8, 16)


def tune_shape(compiled: Sequence[Compiled], dtype: str = "float32") -> Any:
    """The autotuner's launch shape for a sweep: the fused or the TMA-staged sweeps with 4, 8 or
    16 planes per block, each timed for one 64-step chunk on a scratch engine of the median-size
    instance.
    Returns the :class:`~open_analysis_gb300.autotune.TuneResult`, or None when no TMA shape is
    available (the engines then keep their default)."""
    from open_analysis_gb300.autotune import steps_needed, tune
    from open_analysis_gb300.engine import Gb300Engine

    c = sorted(compiled, key=lambda x: x.grid.cells)[len(compiled) // 2]
    eng = Gb300Engine(c, dtype, max_steps=steps_needed(1, SWEEP_TILES, (3, 2)))
    try:
        return tune(eng, chunks=1, tiles=SWEEP_TILES, variants=(3, 2))
    except ValueError:  # every candidate refused
        return None
    finally:
        eng.close()


def _engines(compiled: Sequence[Compiled], steps: int, dtype: str, shape: Any = None) -> tuple[list[Any], float]:
    from open_analysis_gb300.engine import Gb300Engine
    from open_analysis_gb300.model import ModelError

    t0 = time.perf_counter()
    engines = []
    for c in compiled:
        e = Gb300Engine(c, dtype, max_steps=steps)
        if shape is not None:
            try:
                e.set_tuning(shape.tile_z, shape.variant)
            except ModelError:  # this instance cannot take the shape: keep its default
                pass
        engines.append(e)
    return engines, time.perf_counter() - t0


def finish_sweep(models: Sequence[Model], compiled: Sequence[Compiled], engines: Sequence[Any], steps: int,
                 dtype: str, seconds: float, create: float, wire_dir: str | Path | None = None) -> SweepRun:
    """Read every instance's results back (``instance_sparams``), close the engines and, with
    ``wire_dir``, write each instance's worker files (``ports.npz`` with ``(F, N, N)`` S,
    ``run.json``, Touchstone; ``adapter/worker.py:47-52``) into ``wire_dir/instance_<n>``."""
    t0 = time.perf_counter()
    results = [collect(m, c, e, steps, dtype) for m, c, e in zip(models, compiled, engines, strict=True)]
    s = [instance_sparams(m, r) for m, r in zip(models, results, strict=True)]
    read = time.perf_counter() - t0
    for e in engines:
        close = getattr(e, "close", None)
        if close is not None:
            close()
    updates = float(sum(c.grid.cells * c.batch for c in compiled)) * steps
    extra: dict[str, Any] = {"readback_seconds": read}
    if wire_dir is not None:
        from open_analysis_gb300.jobs import write_wire

        share = (seconds + read) / max(len(models), 1)
        extra["wire"] = [
            write_wire(Path(wire_dir) / f"instance_{n:03d}", "sweep", m, sn, r, 0.0, share)
            for n, (m, sn, r) in enumerate(zip(models, s, results, strict=True))
        ]
    return SweepRun(s, seconds + read, create, updates, extra)


def run_batched(models: Sequence[Model], compiled: Sequence[Compiled], steps: int, dtype: str = "float32",
                shape: Any = None, wire_dir: str | Path | None = None) -> SweepRun:
    """All instances at once: every engine's steps queued on its own stream, then waited on.

    The first 64-step chunk goes first on every engine (each captures its graph there), the
    rest after: capturing a graph while other engines' work is queued would wait for that work
    and run the instances one after the other. ``shape``: a launch shape from
    :func:`tune_shape` (None: the engines' default). ``wire_dir``: write each instance's worker
    files there (:func:`finish_sweep`)."""
    engines, create = _engines(compiled, steps, dtype, shape)
    t0 = time.perf_counter()
    first = min(64, steps)
    for e in engines:
        e.step_async(first)
    for e in engines:
        e.wait()
    if steps > first:
        for e in engines:
            e.step_async(steps - first)
        for e in engines:
            e.wait()
    return finish_sweep(models, compiled, engines, steps, dtype, time.perf_counter() - t0, create, wire_dir)


def run_looped(models: Sequence[Model], compiled: Sequence[Compiled], steps: int, dtype: str = "float32",
               shape: Any = None, wire_dir: str | Path | None = None) -> SweepRun:
    """The plain way: one instance after the other."""
    engines, create = _engines(compiled, steps, dtype, shape)
    t0 = time.perf_counter()
    for e in engines:
        e.step(steps)
    return finish_sweep(models, compiled, engines, steps, dtype, time.perf_counter() - t0, create, wire_dir)
