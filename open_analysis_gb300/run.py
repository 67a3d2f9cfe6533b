"""Run driver: engine creation, memory check, energy end criterion, source spectra, S-parameters.

Mirrors ``packages/oa-fdtd/src/oa_fdtd/run.py``: ``RunResult :19-33``, ``source_spectrum :36-43``,
``make_engine :46-75``, ``run :78-160``, ``port_voltage_factor :203-215`` and ``sparams :218-246``.
The loop is the reference's: ``check_every`` steps per engine call, the energy checked against its
peak for the ``end_db`` criterion, and the ``FDTD.UNSTABLE`` detector (non-finite energy, or growth
above the post-pulse minimum by ``growth_db``).

Engine choice: ``"gb300"``, ``"cuda"`` and ``"auto"`` all select :class:`Gb300Engine` (the only
engine of this package); there is no CPU fallback. ``engine`` may also be an engine class or
factory with the reference constructor signature ``(compiled, dtype, record_series=...,
max_steps=...)``; the tests pass the CPU oracle that way.
"""

from __future__ import annotations

from collections.abc import Callable
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.errors import AccelError, ErrorInfo
from open_analysis_gb300.model import Compiled, Model, ModelError, compile_model

FloatArray = npt.NDArray[np.float64]
ComplexArray = npt.NDArray[np.complex128]
GIB = 1024**3


@dataclass
class RunResult:
    probes: dict[str, ComplexArray]  # name -> (B, F) DFT
    source_dft: ComplexArray  # (channels, F)
    steps: int
    dt: float
    engine: str
    dtype: str
    stopped_by: str  # "end_criterion" | "max_steps"
    energy_db: float
    peak_bytes: int
    report: dict[str, Any] = field(default_factory=dict)
    series: dict[str, FloatArray] = field(default_factory=dict)
    port_r: FloatArray = field(default_factory=lambda: np.zeros(0))
    tail: dict[str, Any] = field(default_factory=dict)


def source_spectrum(c: Compiled, steps: int) -> ComplexArray:
    """``sum_n s_c(t_{n+1/2}) exp(-j w t_{n+1/2}) dt`` for every channel."""
    t = (np.arange(steps) + 0.5) * c.dt
    ph = np.exp(-1j * 2.0 * np.pi * c.frequencies[:, None] * t[None, :]) * c.dt
    out = np.zeros((len(c.channels), c.frequencies.size), np.complex128)
    for ci, ch in enumerate(c.channels):
        out[ci] = ph @ ch["waveform"](t)
    return out


def _budget_bytes(total: int) -> int:
    """Device budget: ``min(0.75 total, total - 2 GiB)``, overridable by ``OA_GPU_MEM_GB``."""
    import os

    env = os.environ.get("OA_GPU_MEM_GB")
    if env:
        return min(int(float(env) * GIB), total)
    return max(0, int(min(0.75 * total, total - 2 * GIB)))


def make_engine(
    c: Compiled,
    engine: str | Callable[..., Any],
    dtype: str,
    record_series: bool,
    max_steps: int,
) -> tuple[Any, dict[str, Any]]:
    """Build the engine and an AccelReport-shaped report."""
    if callable(engine):
        eng = engine(c, dtype, record_series=record_series, max_steps=max_steps)
        return eng, {"backend": getattr(eng, "name", "custom")}
    if engine not in ("gb300", "cuda", "auto"):
        raise ModelError(
            "FDTD_BAD_ENGINE",
            f"engine {engine!r} is not available",
            "This package runs the GB300 engine only: use engine='gb300'.",
        )
    from open_analysis_gb300 import native
    from open_analysis_gb300.engine import Gb300Engine, estimate_bytes

    info = native.device_info()
    need = estimate_bytes(c, np.dtype(dtype).itemsize, max_steps=max_steps, record_series=record_series)
    budget = _budget_bytes(info["total_bytes"])
    if need > budget:
        raise AccelError(
            ErrorInfo(
                "ACCEL_OUT_OF_MEMORY",
                f"fdtd needs about {need / GIB:.2f} GiB on the GPU; the budget is {budget / GIB:.2f} GiB.",
                "fdtd",
                f"estimate={need} B, budget={budget} B. Raise OA_GPU_MEM_GB or reduce the problem.",
            )
        )
    eng = Gb300Engine(c, dtype, record_series, max_steps=max_steps)
    report = {
        "backend": "cuda",
        "device_name": info["device_name"],
        "device_id": 0,
        "compute_capability": info["compute_capability"],
        "runtime_version": info["runtime_version"],
        "library_versions": {"oafdtd": str(native.ABI_VERSION)},
        "peak_bytes": 0,
        "budget_bytes": budget,
        "fallbacks": [],
        "deterministic": True,
        "untested_on_hardware": False,
    }
    return eng, report


def run(
    model: Model,
    *,
    engine: str | Callable[..., Any] = "auto",
    dtype: str = "float32",
    max_steps: int = 100_000,
    end_db: float | None = -50.0,
    min_steps: int = 0,
    check_every: int = 64,
    record_series: bool = False,
    tail: bool = False,
    growth_db: float = 20.0,
) -> RunResult:
    """Run until the field energy is ``end_db`` below its peak (checked every ``check_every``
    steps once ``min_steps`` have run) or ``max_steps``; ``end_db=None`` runs ``max_steps``."""
    c = compile_model(model, dtype)
    eng, report = make_engine(c, engine, dtype, record_series or tail, max_steps)
    t_src = 2.0 * model.waveform.delay_tau * model.waveform.tau
    e_min = float("inf")
    peak = 0.0
    e_db = 0.0
    stopped = "max_steps"
    done = 0
    import time

    t_run = time.perf_counter()
    while done < max_steps:
        n = min(check_every, max_steps - done)
        eng.step(n)
        done += n
        if end_db is None:
            continue
        e = eng.energy()
        peak = max(peak, e)
        e_db = 10.0 * np.log10(e / peak) if peak > 0 and e > 0 else 0.0
        if not np.isfinite(e):
            raise ModelError(
                "FDTD.UNSTABLE",
                f"field energy is not finite after {done} steps",
                "Lower the Courant number, check for a PEC/material corner or refine the mesh.",
            )
        if done * c.dt > 1.2 * t_src:
            e_min = min(e_min, e) if e > 0 else e_min
            if np.isfinite(e_min) and e > e_min * 10.0 ** (growth_db / 10.0):
                raise ModelError(
                    "FDTD.UNSTABLE",
                    f"late-time energy grew {10.0 * np.log10(e / e_min):.1f} dB above its minimum "
                    f"after {done} steps",
                    "Lower the Courant number, check for a PEC/material corner or refine the mesh.",
                )
        if done >= min_steps and peak > 0 and e_db <= end_db:
            stopped = "end_criterion"
            break
    wall = time.perf_counter() - t_run
    if isinstance(report, dict) and wall > 0 and done > 0:
        # the run's own rate and, where the engine counts it, its algorithmic DRAM traffic
        report["gcell_updates_per_s"] = float(c.grid.cells) * c.batch * done / wall / 1e9
        if hasattr(eng, "model_bytes"):
            report["bytes_per_step"] = float(eng.model_bytes())
            report["gb_per_s"] = report["bytes_per_step"] * done / wall / 1e9
    probes = eng.results()
    sums = {f"V:{q['name']}": q["probe_parts"] for q in c.ports if q.get("probe_parts")}
    sums.update(c.probe_sums)
    tail_report: dict[str, Any] = {}
    series = eng.series() if (record_series or tail) else {}
    if tail and stopped == "max_steps" and end_db is not None and done > 0:
        from open_analysis_gb300.tail import extend_tails

        tail_report = extend_tails(c, probes, series, sums, done)
    for name, parts in sums.items():
        probes[name] = sum(probes.pop(q) for q in parts)
    peak_bytes = eng.peak_bytes()
    if isinstance(report, dict) and "peak_bytes" in report:
        report["peak_bytes"] = peak_bytes
    return RunResult(
        probes=probes,
        source_dft=source_spectrum(c, done),
        steps=done,
        dt=c.dt,
        engine=eng.name,
        dtype=dtype,
        stopped_by=stopped,
        energy_db=e_db,
        peak_bytes=peak_bytes,
        report=report,
        series=series if record_series else {},
        port_r=np.array([float(q["r_ohm"]) for q in c.ports]),
        tail=tail_report,
    )


def port_voltage_factor(dt: float, frequencies: FloatArray) -> ComplexArray:
    """``cos(w dt / 2)``: maps the recorded E^{n+1} DFT to the time-averaged voltage the
    semi-implicit port resistor sees at t_{n+1/2}."""
    x = np.pi * np.asarray(frequencies, dtype=np.float64) * dt
    return np.cos(x).astype(np.complex128)


def sparams(model: Model, res: RunResult, *, reciprocal: bool = False) -> ComplexArray:
    """Power-wave ``S[i, j, f]``; batch member ``k`` drives port ``model.excited_indices()[k]``.
    Undriven columns are NaN, or filled from ``S[j, i]`` with ``reciprocal=True``."""
    ports = model.ports
    n = len(ports)
    if n == 0:
        raise ModelError("FDTD_NO_PORTS", "S-parameters need at least one port")
    cols = model.excited_indices()
    nf = res.source_dft.shape[1]
    fac = port_voltage_factor(res.dt, model.frequencies)
    s = np.full((n, n, nf), np.nan + 0j, np.complex128)
    for k, j in enumerate(cols):
        v = np.zeros((n, nf), np.complex128)
        for i in range(n):
            v[i] = res.probes[f"V:{ports[i].name}"][k] * fac
        a_j = res.source_dft[j] / (2.0 * np.sqrt(res.port_r[j]))
        for i in range(n):
            s[i, j] = (v[i] / np.sqrt(res.port_r[i]) - (a_j if i == j else 0.0)) / a_j
    if reciprocal:
        for j in range(n):
            if j in cols:
                continue
            for i in cols:
                s[i, j] = s[j, i]
    return s
