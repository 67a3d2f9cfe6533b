"""Batched parameter sweeps: many independent FDTD instances on one GPU at the same time.

A sweep (the reference runs one problem at a time) is a list of models with different grids.
Each instance gets its own engine (its own device state). ``run_batched`` steps them as one
:class:`EngineBatch` (``oafdtd_batch_*``): every kernel class of a time step is a single launch
over the blocks of all instances, each block finding its instance and its own arguments through
a table, and whole 64-step chunks replay one captured graph for the whole sweep, so small grids
fill the GPU together. ``run_looped`` is the plain way, one instance after the other.
``run_batched(..., launch="streams")`` keeps the earlier form: every engine's own graphs queued
on its own stream. All three give the same S-parameters bit for bit (the batched launches run the
same kernel bodies on each instance's own arguments).

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


class EngineBatch:
    """Engines stepped as one (``oafdtd_batch_*``): engines of one sweep variant form one native
    batch each (instances that could not take a sweep's launch shape may run another variant).
    Every engine's results stay readable through the engine; the engines must outlive the batch
    and are stepped only through it while it exists."""

    def __init__(self, engines: Sequence[Any]) -> None:
        import ctypes as C

        from open_analysis_gb300 import native

        self._lib = native.load()
        self._C = C
        groups: dict[int, list[Any]] = {}
        for e in engines:
            groups.setdefault(e.get_tuning()[1], []).append(e)
        self.engines = list(engines)
        self.handles: list[Any] = []
        try:
            for members in groups.values():
                arr = (C.c_void_p * len(members))(*[m._h.value for m in members])
                h = C.c_void_p()
                native.check(self._lib.oafdtd_batch_create(arr, len(members), C.byref(h)), "batch_create")
                self.handles.append(h)
        except Exception:
            self.close()
            raise

    def step_async(self, n: int) -> None:
        from open_analysis_gb300 import native

        for h in self.handles:
            native.check(self._lib.oafdtd_batch_step_async(h, int(n)), "batch_step_async")

    def wait(self) -> None:
        from open_analysis_gb300 import native

        for h in self.handles:
            native.check(self._lib.oafdtd_batch_wait(h), "batch_wait")

    def step(self, n: int) -> None:
        self.step_async(n)
        self.wait()

    def graph_kernels(self) -> int:
        """Kernel launches in one replay of the batches' 64-step graphs (0 before a capture)."""
        from open_analysis_gb300 import native

        total = 0
        for h in self.handles:
            out = self._C.c_int64()
            native.check(self._lib.oafdtd_batch_graph_kernels(h, self._C.byref(out)), "batch_graph_kernels")
            total += int(out.value)
        return total

    def close(self) -> None:
        for h in self.handles:
            if h:
                self._lib.oafdtd_batch_destroy(h)
        self.handles = []

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


def run_batched(models: Sequence[Model], compiled: Sequence[Compiled], steps: int, dtype: str = "float32",
                shape: Any = None, wire_dir: str | Path | None = None, launch: str = "batch") -> SweepRun:
    """All instances at once. ``launch="batch"`` (the default): one :class:`EngineBatch`, every
    kernel class one launch over all instances. ``launch="streams"``: every engine's steps queued
    on its own stream, then waited on; the first 64-step chunk goes first on every engine (each
    captures its graph there), the rest after, since capturing a graph while other engines' work
    is queued would wait for that work. ``shape``: a launch shape from :func:`tune_shape` (None:
    the engines' default). ``wire_dir``: write each instance's worker files there
    (:func:`finish_sweep`)."""
    if launch not in ("batch", "streams"):
        raise ValueError(f"launch {launch!r}: 'batch' or 'streams'")
    engines, create = _engines(compiled, steps, dtype, shape)
    extra: dict[str, Any] = {"launch": launch}
    if launch == "batch":
        t_b = time.perf_counter()
        batch = EngineBatch(engines)
        create += time.perf_counter() - t_b
        t0 = time.perf_counter()
        batch.step(steps)
        extra["graph_kernels_per_chunk"] = batch.graph_kernels()
        extra["native_batches"] = len(batch.handles)
        batch.close()
    else:
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
    run = finish_sweep(models, compiled, engines, steps, dtype, time.perf_counter() - t0, create, wire_dir)
    run.extra.update(extra)
    return run


def run_looped(models: Sequence[Model], compiled: Sequence[Compiled], steps: int, dtype: str = "float32",
               shape: Any = None, wire_dir: str | Path | None = None) -> SweepRun:
    """The plain way: one instance after the other."""
    engines, create = _engines(compiled, steps, dtype, shape)
    t0 = time.perf_counter()
    for e in engines:
        e.step(steps)
    return finish_sweep(models, compiled, engines, steps, dtype, time.perf_counter() - t0, create, wire_dir)
