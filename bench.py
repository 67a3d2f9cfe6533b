#!/usr/bin/env python
"""FDTD time-stepping throughput on GB300: Gcell-updates/s and the HBM roofline.

``python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]``

Workload (default): the via-transition problem, 400 x 400 x 120 cells of 25 um (19.2 M cells),
single-pole Debye dielectric, surface-impedance copper, 10-cell CPML, two lumped ports (batch of
two excitations), 256 DFT frequencies (``open_analysis_gb300.structures.via_transition``),
synthetic geometry. One bench step = one 64-time-step chunk, the unit the reference run loop
advances between energy checks. Gcell-updates/s = interior cells x batch x time steps / time.

* ``value``: device time (CUDA events on the engine's stream) of K chunks, fields resident in HBM
  (the fields, 0.98 GB, are far larger than the 129 MB L2, so no flush is needed).
* ``e2e``: the same metric through the public API from host buffers: engine creation (the host
  ``Compiled`` arrays copied to the device), K chunks each followed by the energy check (a device
  to host read, as the run loop does), the probe DFTs read back at the end; host wall clock.
* ``roofline``: the dominant kernel's algorithmic bytes per launch (the engine's traffic model,
  ``Gb300Engine.kernel_bytes``) over its average launch time measured with CUDA events inside the
  timed region.
* ``cpu_baseline``: the CPU oracle (the reference's NumPy engine restated) in float32 on the same
  compiled problem, a bounded sample of time steps, one host thread.
* ``sweeps``: S-parameter sweeps/s of a seeded sweep of uneven microstrip/stripline instances
  (``structures.sweep_instances``), all instances batched on the GPU at once against looping the
  plain engine over them (``open_analysis_gb300.batch``); wall clock of the stepping and the
  S-parameter read-back, engines created beforehand; both give identical S-parameters.
  ``sweeps.surrogate``: batched + learned surrogate against batched alone and against the plain
  loop, on a three-parameter sweep of small via transitions (``surrogate.experiment``: data from
  the batched engine, the ensemble trained on the GPU, held-out answers judged against FDTD).
* ``large_board``: the 1600 x 1200 x 160 board region (307 M cells, eight ports as a batch of
  eight, 512 frequencies) on the same GPU after the sweeps: ``--board-chunks`` timed 64-step
  chunks, the per-class fractions of the measured copy bandwidth, compile time and device bytes.

``--impl reference`` times the reference's CPU path (the oracle port; the reference is a Python
package and is not installed on the GPU host) on the same workload, one time step per bench step.
For N > 1 (torchrun) every rank runs its own replica (independent instances: weak scaling, no
collective on the data path); rank 0 prints the line with the max time over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path
from typing import Any

import numpy as np

# batched sweeps run many engines on many streams: more hardware work queues (before CUDA starts)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

CHUNK = 64


# ---------------------------------------------------------------------------- distributed plumbing
class Ranks:
    """Rank bookkeeping; torch.distributed (gloo, host-side only) for barrier and max."""

    def __init__(self, gpus: int) -> None:
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.gpus = gpus
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.dist is None:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi SM clock and throttle-reason samples every 200 ms during the timed region."""

    QUERY = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, gpu: int) -> None:
        self.gpu = gpu
        self.proc: subprocess.Popen[bytes] | None = None
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])

    def start(self) -> None:
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)],
                stdout=open(self.path, "wb"),
                stderr=subprocess.DEVNULL,
            )
        except OSError:
            self.proc = None

    def stop(self) -> dict[str, Any] | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.strip()]
        self.path.unlink(missing_ok=True)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, flag in zip(names, r[5:9], strict=False):
                if flag.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {
            "sm_mhz": statistics.median(sm),
            "sm_max_mhz": max(smax),
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


# ---------------------------------------------------------------------------- roofline inputs
def measured_peak() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        try:
            return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def profiled_traffic(kernel: str) -> float | None:
    """DRAM bytes per launch of ``kernel`` from the committed ncu summary, scaled to this
    workload, or None when no capture exists."""
    path = ROOT / "profiles" / f"{kernel}_via_transition_traffic.txt"
    if not path.exists():
        return None
    vals: dict[str, float] = {}
    for line in path.read_text().splitlines():
        if "=" in line and not line.lstrip().startswith("#"):
            k, v = line.split("=", 1)
            try:
                vals[k.strip()] = float(v.split()[0])
            except (ValueError, IndexError):
                continue
    if "bytes_per_launch_full_workload" in vals:
        return vals["bytes_per_launch_full_workload"]
    return None


# ---------------------------------------------------------------------------- arms
def build_problem(args: argparse.Namespace, native: bool | None = None) -> tuple[Any, Any]:
    """The workload's model and its compiled arrays. ``native=False`` compiles with the NumPy
    stages only (bit for bit the same arrays), so no engine library is loaded."""
    from open_analysis_gb300.model import compile_model
    from open_analysis_gb300.structures import large_board, microstrip, via_transition

    if args.workload == "microstrip":
        m = microstrip()
    elif args.workload == "large_board":
        m = large_board()
    elif args.cells:
        nx, ny, nz = (int(v) for v in args.cells.split(","))
        m = via_transition(nx=nx, ny=ny, nz=nz)
    else:
        m = via_transition()
    return m, compile_model(m, "float32", native=native)


def workload_config(args: argparse.Namespace, c: Any, world: int) -> dict[str, Any]:
    """The workload keys both arms print (the launch shape and the time steps per bench step are
    reported beside them: they describe how an arm steps, not what it computes)."""
    nx, ny, nz = c.grid.n
    names = {"microstrip": f"microstrip_{nx}x{ny}x{nz}", "large_board": f"large_board_{nx}x{ny}x{nz}"}
    return {
        "workload": names.get(args.workload, f"via_transition_{nx}x{ny}x{nz}"),
        "cells": [nx, ny, nz],
        "batch": c.batch,
        "dft_frequencies": int(c.frequencies.size),
        "ade_poles": 0 if c.ade is None else int(c.ade.tau.size),
        "sibc_edges": 0 if c.sibc is None else int(c.sibc.flat.size),
        "l2": "inputs larger than L2 (fields 6 x batch x 4 B per storage cell), no flush",
        "parallelism": f"replicas{world}",
    }


def cpu_sample(c: Any, target_s: float) -> dict[str, Any]:
    """The oracle in float32 on the same problem: one untimed step, then as many steps as fit
    about ``target_s`` seconds (at least two)."""
    from oracle.numpy_engine import OracleEngine

    eng = OracleEngine(c, "float32")
    t0 = time.perf_counter()
    eng.step(1)
    one = time.perf_counter() - t0
    n = max(2, int(target_s / max(one, 1e-6)))
    t0 = time.perf_counter()
    eng.step(n)
    dt = time.perf_counter() - t0
    nx, ny, nz = c.grid.n
    rate = nx * ny * nz * c.batch * n / dt / 1e9
    return {
        "value": rate,
        "unit": "Gcell-updates/s",
        "cores": 1,
        "kind": "port",
        "sample": f"{n} time steps of the full {nx}x{ny}x{nz} grid, batch {c.batch}, float32, "
        f"after 1 untimed step ({dt:.1f} s); NumPy elementwise runs on one thread",
    }


def sweep_measure(n: int, steps: int) -> dict[str, Any]:
    """Batched against looped S-parameter sweeps over ``n`` seeded instances (2 ports, 128
    frequencies each), ``steps`` time steps each."""
    from open_analysis_gb300.batch import compile_all, run_batched, run_looped, tune_shape
    from open_analysis_gb300.structures import sweep_instances

    models = sweep_instances(n)
    compiled = compile_all(models)
    t0 = time.perf_counter()
    shape = tune_shape(compiled)
    tune_s = time.perf_counter() - t0
    batched = run_batched(models, compiled, steps, shape=shape)
    streams = run_batched(models, compiled, steps, shape=shape, launch="streams")
    looped = run_looped(models, compiled, steps, shape=shape)
    same = all(np.array_equal(a, b) and np.array_equal(a, c)
               for a, b, c in zip(batched.s, looped.s, streams.s, strict=True))
    return {
        "metric": "S-parameter sweeps/s",
        "instances": n,
        "steps": steps,
        "cells_total": int(sum(x.grid.cells for x in compiled)),
        "batched": batched.sweeps_per_s,
        "looped": looped.sweeps_per_s,
        "streams": streams.sweeps_per_s,
        "batched_over_looped": batched.sweeps_per_s / looped.sweeps_per_s,
        "batched_over_streams": batched.sweeps_per_s / streams.sweeps_per_s,
        "batched_gcell_s": batched.cell_updates / batched.seconds / 1e9,
        "looped_gcell_s": looped.cell_updates / looped.seconds / 1e9,
        "streams_gcell_s": streams.cell_updates / streams.seconds / 1e9,
        "batched_launch": {k: batched.extra[k] for k in ("graph_kernels_per_chunk", "native_batches")},
        "identical_s": same,
        "launch_shape": None if shape is None else {"tile_z": shape.tile_z, "variant": shape.variant,
                                                    "tune_seconds": tune_s},
    }


def surrogate_measure(n: int) -> dict[str, Any]:
    """The learned surrogate on a sweep of small via transitions (48 x 48 x 60 cells; stack
    height, eps_inf and delta_eps free, the rest fixed): generate ``n`` instances with the
    batched engine, train a 32-member ensemble on the GPU (BF16 tensor-core kernels), answer the
    held-out instances with FDTD fallback, judge every answer against FDTD, and compare the sweep
    rates."""
    from open_analysis_gb300.surrogate import ViaGrid, experiment

    g = ViaGrid(nx=48, ny=48, nz=60, h=50e-6, dz=100e-6, n_freq=32, cpml=6, span=560e-12)
    fixed = {"drill": 0.3e-3, "pad": 0.5e-3, "antipad": 0.9e-3, "stub": 0.6e-3}
    n_tr, n_vc = (n * 2) // 3, n // 12
    # 32 members: on this sweep the strict gate accepted 70 % with 8, 80 % with 16 and 81 % with 32
    # (every answer within 0.05 dB each time), training 8 / 7 / 12 s
    rep = experiment(g, n, seed=21, fixed=fixed, split=(n_tr / n, n_vc / n, n_vc / n), batch=64, epochs=3000,
                     lrs=(1e-3,), chunk=64, members=32)
    keep = ("grid", "steps", "folds", "network", "activation", "members", "train_seconds", "tol_db", "accepted",
            "accepted_worst_db", "answers_within_tol", "answers_worst_db", "network_alone_median_db",
            "network_alone_within_tol", "plain_sweeps_per_s", "batched_sweeps_per_s", "surrogate_sweeps_per_s",
            "network_sweeps_per_s",
            "gain_vs_plain", "gain_vs_batched")
    out = {k: rep[k] for k in keep}
    out["free_parameters"] = ["stack", "eps_inf", "delta_eps"]
    return out


def board_measure(chunks: int, warmup: int = 2) -> dict[str, Any]:
    """The large board region on one GPU: 1600 x 1200 x 160 cells of 20 um (307 M cells), eight
    Debye layers, 12 traces and 40 vias of surface-impedance copper at seeded positions, 12-cell
    CPML, eight ports driven as a batch of eight, 512 frequencies 0.05-40 GHz
    (``structures.large_board``), the engine's default launch shape. ``chunks`` timed 64-step
    chunks after ``warmup`` untimed ones, then one profiled chunk for the per-class times."""
    from open_analysis_gb300.engine import Gb300Engine
    from open_analysis_gb300.model import compile_model
    from open_analysis_gb300.structures import large_board

    t0 = time.perf_counter()
    c = compile_model(large_board(), "float32")
    compile_s = time.perf_counter() - t0
    nx, ny, nz = c.grid.n
    batch = c.batch
    t0 = time.perf_counter()
    eng = Gb300Engine(c, "float32", max_steps=(warmup + chunks + 3) * CHUNK)
    create_s = time.perf_counter() - t0
    del c
    for _ in range(warmup):
        eng.step(CHUNK)
    sampler = ClockSampler(0)
    sampler.start()
    times = [eng.step_timed(CHUNK) for _ in range(chunks)]
    clocks = sampler.stop()
    ms_step = sum(times) / (chunks * CHUNK)
    eng.set_profiling(True)
    eng.step(CHUNK)  # capture the profiled graph
    eng.step(CHUNK)
    kt = eng.kernel_times()
    eng.set_profiling(False)
    kb = eng.kernel_bytes()
    model_bytes = eng.model_bytes()
    device_bytes = eng.peak_bytes()
    eng.close()
    peak, peak_kind = measured_peak()
    classes = {k: {"ms_per_time_step": kt[k], "algorithmic_gb": kb[k] / 1e9,
                   "frac": kb[k] / (kt[k] / 1e3) / 1e9 / peak}
               for k in kb if k != "step" and kb[k] > 0 and kt.get(k, 0.0) > 0}
    return {
        "workload": f"large_board_{nx}x{ny}x{nz}",
        "batch": batch,
        "value": float(nx) * ny * nz * batch / (ms_step / 1e3) / 1e9,
        "unit": "Gcell-updates/s",
        "timed_chunks": chunks,
        "warmup_chunks": warmup,
        "ms_per_time_step": ms_step,
        "step_frac": model_bytes / (ms_step / 1e3) / 1e9 / peak,
        "peak": peak,
        "peak_source": peak_kind,
        "classes": classes,
        "compile_seconds": compile_s,
        "create_seconds": create_s,
        "device_bytes": device_bytes,
        "clocks": clocks,
    }


def run_gb300(args: argparse.Namespace, ranks: Ranks) -> None:
    from open_analysis_gb300 import native
    from open_analysis_gb300.engine import Gb300Engine

    native.set_device(ranks.local)
    model, c = build_problem(args)
    nx, ny, nz = c.grid.n
    cells = nx * ny * nz
    prof_chunks = 3
    max_steps = (args.warmup + args.steps + prof_chunks + 3) * CHUNK
    tiles: dict[str, Any] = {}
    if args.tile_z or args.variant >= 0:
        tiles = {"tile_z": args.tile_z, "variant": args.variant, "source": "flags"}
    elif not args.no_tune:
        from open_analysis_gb300.autotune import steps_needed, tune

        scratch = Gb300Engine(c, "float32", max_steps=steps_needed() + CHUNK)
        tr = tune(scratch)
        scratch.close()
        tiles = {"tile_z": tr.tile_z, "variant": tr.variant, "source": "autotune",
                 "tuned_ms_per_time_step": tr.ms_per_step,
                 "table": {f"{k[0]}/{k[1]}": round(v, 5) for k, v in tr.table.items()}}
    eng = Gb300Engine(c, "float32", max_steps=max_steps)
    if tiles:
        eng.set_tuning(tiles["tile_z"], tiles["variant"])
    for _ in range(args.warmup):
        eng.step(CHUNK)
    sampler = ClockSampler(ranks.local)
    ranks.barrier()
    sampler.start()
    times = []
    for _ in range(args.steps):
        times.append(eng.step_timed(CHUNK))
    clocks = sampler.stop()
    ranks.barrier()
    total_ms = ranks.max(float(sum(times)))
    # Per-kernel times for the roofline: a separate pass with CUDA events around every kernel
    # class, captured inside the graph; profiling runs each class alone (no overlap of the sweep
    # and the slab kernel), so these are the kernels' own durations.
    eng.set_profiling(True)
    eng.step(CHUNK)  # capture the profiled graph
    ksum: dict[str, float] = {}
    for _ in range(prof_chunks):
        eng.step(CHUNK)
        for k, v in eng.kernel_times().items():  # per-step averages over this chunk
            ksum[k] = ksum.get(k, 0.0) + v
    ktimes = {k: v / prof_chunks for k, v in ksum.items()}
    eng.set_profiling(False)
    updates = float(cells) * c.batch * CHUNK * args.steps * ranks.world
    value = updates / (total_ms / 1e3) / 1e9
    all_bytes = eng.kernel_bytes()  # the engine's traffic model, per time step and kernel class
    kb = {k: v for k, v in all_bytes.items() if k != "step" and v > 0}
    dominant = max(kb, key=lambda k: ktimes.get(k, 0.0))
    eng.step(CHUNK)  # re-capture the graph of the timed region to count its kernels
    graph_kernels = eng.graph_kernels()
    peak, peak_kind = measured_peak()
    achieved = kb[dominant] / (ktimes[dominant] / 1e3) / 1e9
    step_bytes = all_bytes["step"]  # what the launch shape in use must move per time step
    model_bytes = eng.model_bytes()  # the separate sweeps' traffic model (72 + 6 / B B per cell-update)
    eng.close()

    # e2e through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        ranks.barrier()
        t0 = time.perf_counter()
        eng2 = Gb300Engine(c, "float32", max_steps=max_steps)
        t_create = time.perf_counter() - t0
        h2d = eng2.h2d_bytes
        for _ in range(args.steps):
            eng2.step(CHUNK)
            eng2.energy()
        res = eng2.results()
        eng2.close()
        e2e_s = ranks.max(time.perf_counter() - t0)
        d2h = args.steps * 6 * 8 + sum(v.nbytes for v in res.values())
        e2e = {
            "value": float(cells) * c.batch * CHUNK * args.steps * ranks.world / e2e_s / 1e9,
            "unit": "Gcell-updates/s",
            "h2d_bytes_per_step": h2d / args.steps,
            "d2h_bytes_per_step": d2h / args.steps,
            "seconds": e2e_s,
            "create_seconds": t_create,
        }

    cpu = None
    if ranks.rank == 0 and ranks.world == 1 and not args.no_cpu:
        cpu = cpu_sample(c, args.cpu_seconds)

    sweeps = None
    if args.sweep_instances > 0 and args.sweep_steps > 0:
        sweeps = sweep_measure(args.sweep_instances, args.sweep_steps)
        if args.surrogate_instances:
            sweeps["surrogate"] = surrogate_measure(args.surrogate_instances)

    board = None
    if args.board_chunks > 0 and ranks.world == 1 and args.workload == "via_transition":
        board = board_measure(args.board_chunks)

    if ranks.rank == 0:
        line = {
            "metric": "Gcell-updates/s",
            "value": value,
            "unit": "Gcell-updates/s",
            "n_gpus": ranks.world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(args, c, ranks.world),
            "time_steps_per_step": CHUNK,
            "tiles": tiles,
            "roofline": {
                "bound": "hbm",
                "kernel": dominant,
                "achieved": achieved,
                "peak": peak,
                "peak_source": peak_kind,
                "unit": "GB/s",
                "frac": achieved / peak,
                # the committed ncu traffic summaries are of the via-transition workload
                "traffic": profiled_traffic(dominant) if args.workload == "via_transition" else None,
                "kernel_ms": ktimes,
                "algorithmic_bytes_per_launch": kb,
                # the whole time step of the timed region: the traffic model of the separate
                # sweeps (Gcell-updates/s x bytes per cell-update) over the measured peak, and the
                # bytes the launch shape in use moves (less with the fused sweep)
                "step_frac": model_bytes / (total_ms / (args.steps * CHUNK) / 1e3) / 1e9 / peak,
                "step_moved_frac": step_bytes / (total_ms / (args.steps * CHUNK) / 1e3) / 1e9 / peak,
                "step_bytes_model": model_bytes,
                "step_bytes_moved": step_bytes,
            },
            "e2e": e2e,
            "gpu_launches": graph_kernels * args.steps,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "sweeps": sweeps,
            "large_board": board,
        }
        print(json.dumps(line), flush=True)


def run_reference(args: argparse.Namespace, ranks: Ranks) -> None:
    if ranks.rank != 0:
        return
    from oracle.numpy_engine import OracleEngine

    # the NumPy stages of the compiler: the reference arm maps no library of this package
    _, c = build_problem(args, native=False)
    nx, ny, nz = c.grid.n
    eng = OracleEngine(c, "float32")
    for _ in range(args.warmup):
        eng.step(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.step(1)
    dt = time.perf_counter() - t0
    value = nx * ny * nz * c.batch * args.steps / dt / 1e9
    sample = (
        f"one time step of the full {nx}x{ny}x{nz} grid (batch {c.batch}, float32) per bench step; "
        "the reference's NumPy engine restated (the reference is a Python package, not installable "
        "on the GPU host); NumPy elementwise runs on one thread"
    )
    print(
        json.dumps(
            {
                "impl": "reference",
                "metric": "Gcell-updates/s",
                "value": value,
                "unit": "Gcell-updates/s",
                "n_gpus": ranks.world,
                "steps": args.steps,
                "warmup": args.warmup,
                "ms_per_step": dt * 1e3 / args.steps,
                "higher_is_better": True,
                "scaling": "weak",
                "vs_baseline": None,
                "dtype": "f32",
                "data": "synthetic",
                "config": workload_config(args, c, ranks.world),
                "time_steps_per_step": 1,
                "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": 1, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
            }
        ),
        flush=True,
    )


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="via_transition", choices=["via_transition", "microstrip", "large_board"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--tile-z", type=int, default=0, help="planes per block")
    ap.add_argument("--variant", type=int, default=-1,
                    help="3 fused interior sweep, 2 TMA-staged, 1 cp.async-staged, 0 register marching")
    ap.add_argument("--cells", default="", help="via-transition grid 'nx,ny,nz' (smaller profiling cases)")
    ap.add_argument("--sweep-instances", type=int, default=64, help="batched-sweep instances (0: skip)")
    ap.add_argument("--sweep-steps", type=int, default=8000, help="time steps per sweep instance")
    ap.add_argument("--surrogate-instances", type=int, default=384, help="surrogate sweep instances (0: skip)")
    ap.add_argument("--board-chunks", type=int, default=3,
                    help="timed 64-step chunks of the large-board region after the sweeps (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    ranks = Ranks(args.gpus)
    try:
        if args.impl == "reference":
            run_reference(args, ranks)
        else:
            run_gb300(args, ranks)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
