"""Engine-level jobs and the worker's output files.

``python -m open_analysis_gb300.jobs run job.json`` runs the reference's engine-level job format
(``packages/oa-fdtd/src/oa_fdtd/cli.py:1-20``: mesh lines, waveform, frequencies, walls, CPML,
regions, lumped ports, soft sources, probes, run options, output name) on the GB300 engine and
writes the reference's outputs:

* ``output`` (default ``ports.npz``) with ``frequencies``, ``s`` as ``(N, N, F)`` when the job has
  ports, and ``probe_<name>`` DFTs (``cli.py:118-128``);
* with ``"wire": true`` also the FDTD worker's files (``adapter/worker.py:47-52``) in the
  directory ``wire_dir`` (default ``worker``) beside the job: ``ports.npz`` with ``freqs``, ``s``
  as ``(F, N, N)``, ``z0`` and ``names`` (the file the adapter's collect step reads), ``run.json``
  with the run statistics (``adapter/sim.py:204-220``) and a Touchstone file
  ``<output stem>.s<N>p``.

The summary goes to stdout as one JSON object; failures print an ``ErrorInfo``-shaped object
(``code``, ``message``, ``path``, ``hint``) and exit with status 2, as the reference's CLI does.
"""

from __future__ import annotations

import argparse
import json
import sys
import time
from collections.abc import Callable
from pathlib import Path
from typing import Any

import numpy as np

from open_analysis_gb300.grid import Grid
from open_analysis_gb300.model import LumpedPort, Model, ModelError, Probe, Region, SoftSource, Waveform
from open_analysis_gb300.pml import CpmlSpec
from open_analysis_gb300.run import RunResult, run, sparams
from open_analysis_gb300.touchstone import write_touchstone


def _xyz(v: Any) -> tuple[float, float, float]:
    a = [float(x) for x in v]
    if len(a) != 3:
        raise ModelError("FDTD_BAD_JOB", "boxes need three coordinates")
    return (a[0], a[1], a[2])


def model_from_job(job: dict[str, Any]) -> Model:
    """The ``Model`` of a parsed job (the reference's keys and defaults). Raises ``ModelError``."""
    try:
        m = Model(
            Grid(*(np.asarray(job["grid"][k], dtype=np.float64) for k in "xyz")),
            Waveform(**job["waveform"]),
            np.asarray(job["frequencies"], dtype=np.float64),
        )
        if "walls" in job:
            m.walls = tuple(job["walls"])
        if "cpml" in job:
            m.cpml = CpmlSpec(**job["cpml"])
        if "courant" in job:
            m.courant = float(job["courant"])
        for r in job.get("regions", []):
            m.regions.append(Region(_xyz(r["lo"]), _xyz(r["hi"]), r.get("eps_r", 1.0), r.get("sigma", 0.0), r.get("pec", False)))
        for p in job.get("ports", []):
            m.ports.append(
                LumpedPort(p["name"], int(p["axis"]), _xyz(p["lo"]), _xyz(p["hi"]), p.get("r_ohm", 50.0), p.get("sign", 1.0))
            )
        for s in job.get("sources", []):
            m.sources.append(SoftSource(s["name"], int(s["axis"]), _xyz(s["lo"]), _xyz(s["hi"]), s.get("amplitude", 1.0)))
        for p in job.get("probes", []):
            m.probes.append(Probe(p["name"], p["kind"], int(p["axis"]), _xyz(p["lo"]), _xyz(p["hi"]), p.get("weight", "sum")))
    except (KeyError, TypeError) as exc:
        raise ModelError("FDTD_BAD_JOB", f"malformed job: {exc!r}", "See open_analysis_gb300.jobs.") from exc
    return m


def run_meta(res: RunResult, model: Model, wall_build_s: float, wall_run_s: float) -> dict[str, Any]:
    """Run statistics in the worker's ``run.json`` shape."""
    return {
        "engine": res.engine,
        "dtype": res.dtype,
        "steps": res.steps,
        "stopped_by": res.stopped_by,
        "energy_db": res.energy_db,
        "dt_s": res.dt,
        "peak_gpu_bytes": res.peak_bytes,
        "wall_build_s": wall_build_s,
        "wall_run_s": wall_run_s,
        "cells": int(model.grid.cells),
        "diagnostics": [],
        "accel": res.report,
        "tail": res.tail,
    }


def write_wire(
    directory: Path, stem: str, model: Model, s_nnf: np.ndarray, res: RunResult, wall_build_s: float, wall_run_s: float
) -> dict[str, str]:
    """The worker's files in ``directory``: ``ports.npz`` (freqs, s (F, N, N), z0, names),
    ``run.json`` and a Touchstone file. Returns their paths. ``z0`` is the run's port resistances
    (the lumped ports' R, the mode ports' modal impedance), as the reference's adapter takes it
    (``adapter/sim.py:194``)."""
    names = [p.name for p in model.ports]
    z0 = np.asarray(res.port_r, dtype=np.float64)
    s_fnn = np.moveaxis(np.asarray(s_nnf), -1, 0)
    freqs = np.asarray(model.frequencies, dtype=np.float64)
    directory.mkdir(parents=True, exist_ok=True)
    npz = directory / "ports.npz"
    np.savez(npz, freqs=freqs, s=s_fnn, z0=z0, names=np.array(names))
    meta = run_meta(res, model, wall_build_s, wall_run_s)
    meta["port_names"] = names
    meta["fdtd_version"] = "open_analysis_gb300"
    run_json = directory / "run.json"
    run_json.write_text(json.dumps(meta, indent=1, default=str) + "\n", encoding="utf-8")
    ts = directory / f"{stem}.s{len(names)}p"
    write_touchstone(ts, freqs, s_fnn, list(z0), names, [f"{res.engine} {res.dtype}, {res.steps} steps"])
    return {"wire": str(npz), "run_json": str(run_json), "touchstone": str(ts)}


def run_job(path: Path, engine: str | Callable[..., Any] | None = None) -> dict[str, Any]:
    """Run a job file; ``engine`` overrides the job's (a factory, or ``"gb300"``)."""
    job = json.loads(Path(path).read_text(encoding="utf-8"))
    t0 = time.perf_counter()
    model = model_from_job(job)
    opts = job.get("run", {})
    wall_build = time.perf_counter() - t0
    t1 = time.perf_counter()
    res = run(
        model,
        engine=engine if engine is not None else opts.get("engine", "auto"),
        dtype=opts.get("dtype", "float32"),
        max_steps=int(opts.get("max_steps", 100_000)),
        end_db=opts.get("end_db", -50.0),
    )
    wall_run = time.perf_counter() - t1
    out: dict[str, Any] = {"frequencies": model.frequencies}
    s = sparams(model, res) if model.ports else None
    if s is not None:
        out["s"] = s
    for name, v in res.probes.items():
        out["probe_" + name.replace(":", "_")] = v
    target = Path(path).parent / job.get("output", "ports.npz")
    np.savez(target, **out)
    summary: dict[str, Any] = {
        "output": str(target),
        "steps": res.steps,
        "stopped_by": res.stopped_by,
        "engine": res.engine,
        "dtype": res.dtype,
        "energy_db": res.energy_db,
        "dt_s": res.dt,
        "peak_gpu_bytes": res.peak_bytes,
        "accel": res.report,
    }
    if job.get("wire") and s is not None:
        wire_dir = Path(path).parent / job.get("wire_dir", "worker")
        summary.update(write_wire(wire_dir, target.stem, model, s, res, wall_build, wall_run))
    return summary


def _error(code: str, message: str, path: str, hint: str = "") -> dict[str, str]:
    return {"code": code, "message": message, "path": path, "hint": hint}


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(prog="python -m open_analysis_gb300.jobs")
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run", help="run a job file")
    r.add_argument("job", type=Path)
    args = ap.parse_args(argv)
    try:
        summary = run_job(args.job)
    except ModelError as exc:
        print(json.dumps(_error(exc.code, exc.message, str(args.job), exc.hint)))
        return 2
    except OSError as exc:
        print(json.dumps(_error("FDTD_IO", str(exc), str(args.job))))
        return 2
    except Exception as exc:  # AccelError carries an ErrorInfo
        info = getattr(exc, "info", None)
        print(json.dumps(info.to_dict() if info is not None else _error("FDTD_ERROR", str(exc), "")))
        return 2
    print(json.dumps(summary, default=str))
    return 0


if __name__ == "__main__":
    sys.exit(main())
