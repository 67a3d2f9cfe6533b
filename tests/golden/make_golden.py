"""Generate the golden fixtures from the reference implementation itself.

Run in a checkout that has the reference's source tree at hand (not needed anywhere else):

    python tests/golden/make_golden.py <reference root> [part ...]

where the parts are any of ``cases debye touchstone tail runs jobs workloads compiled`` (all of
them by default; ``workloads`` runs the reference's NumPy engine on the full-size workloads of
``workloads.py`` and takes about an hour on one host thread; ``workloads:<name>`` runs one).

For every problem in ``cases.CASES`` it builds the model from the reference's own classes,
compiles it with the reference's ``compile_model`` and steps the reference's ``NumpyEngine`` in
float32 and float64. It stores fingerprints (digests of every compiled array and of the float32
fields, the probe DFTs, the energy) under ``tests/golden/<case>.npz``. The tests compare
``open_analysis_gb300.model.compile_model`` and the oracle in ``oracle/`` against them, and the
GPU tests compare the CUDA engine against the oracle and these fingerprints.
"""

from __future__ import annotations

import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


PARTS = ("cases", "debye", "touchstone", "tail", "runs", "jobs", "workloads", "compiled")


def main(reference_root: str, parts: tuple[str, ...] = PARTS) -> None:
    root = Path(reference_root)
    sys.path.insert(0, str(root / "packages" / "oa-fdtd" / "src"))
    sys.path.insert(0, str(root / "packages" / "oa-accel" / "src"))
    sys.path.insert(0, str(HERE))
    sys.path.insert(0, str(HERE.parent.parent))
    import numpy as np
    from cases import CASES, namespace  # type: ignore[import-not-found]
    from fingerprint import compiled_fingerprint, save, state_fingerprint  # type: ignore[import-not-found]
    from oa_fdtd.model import compile_model  # type: ignore[import-not-found]
    from oa_fdtd.reference import NumpyEngine  # type: ignore[import-not-found]

    ns = namespace("ref")
    if "cases" in parts:
        cases(np, ns, CASES, compile_model, NumpyEngine, compiled_fingerprint, state_fingerprint, save)
    if "debye" in parts:
        debye_fits(np)
    if "touchstone" in parts:
        touchstone_files(np)
    if "tail" in parts:
        tail_fits(np)
    if "runs" in parts:
        run_loops(np)
    if "jobs" in parts:
        job_parse(np)
    picked = tuple(p.split(":", 1)[1] for p in parts if p.startswith("workloads:"))
    if "workloads" in parts or picked:
        workload_fixtures(np, ns, picked)
    if "compiled" in parts:
        reference_compiled(np, ns)


def cases(np, ns, CASES, compile_model, NumpyEngine, compiled_fingerprint, state_fingerprint, save):  # type: ignore[no-untyped-def]
    """Every problem of ``cases.CASES``: compiled arrays, float32 and float64 engine states."""
    for name, (builder, steps) in CASES.items():
        model = builder(ns)
        c = compile_model(model, "float32")
        data = compiled_fingerprint(c)
        data["steps"] = steps
        for dtype in ("float32", "float64"):
            eng = NumpyEngine(c, dtype)
            eng.step(steps)
            for k, v in state_fingerprint(eng).items():
                data[f"{dtype}.{k}"] = v
        if hasattr(model, "plane_sets"):
            wave_fixture(np, model, c, NumpyEngine, steps, data)
        if name == "mixed_walls":
            eng = NumpyEngine(c, "float32")
            eng.step(steps)
            for comp, arr in zip(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"), (*eng.E, *eng.H), strict=True):
                data[f"full.{comp}"] = np.ascontiguousarray(arr)
        save(str(HERE / f"{name}.npz"), data)
        print(name, "steps", steps, "batch", c.batch, "keys", len(data))


SAMPLES = 4096  # float64 field values kept per component for the error against the FP64 oracle


def workload_fixtures(np, ns, only=()):  # type: ignore[no-untyped-def]
    """The benchmark workloads of ``workloads.py`` built from the reference's classes, compiled by
    its ``compile_model`` and stepped by its ``NumpyEngine`` in float32 and float64 (from the
    seeded fields where the workload has a seed). Stored per workload: the compiled arrays'
    fingerprint, the float32 state (field digests, DFTs, energy), the float64 DFTs and energy,
    each float32 field's rel-L2 distance from the float64 one, float64 values at seeded sample
    points, and for the port workload without a seed the S-parameters of the float32 engine
    (through the reference's ``sparams``) and of the reference's own ``run()`` in float64."""
    import time

    from fingerprint import compiled_fingerprint, save, state_fingerprint  # type: ignore[import-not-found]
    from oa_fdtd.model import compile_model  # type: ignore[import-not-found]
    from oa_fdtd.reference import NumpyEngine  # type: ignore[import-not-found]
    from oa_fdtd.run import RunResult, run, source_spectrum, sparams  # type: ignore[import-not-found]
    from workloads import NAMES, convert, sample_index, seeded_values, workloads  # type: ignore[import-not-found]

    for name, w in workloads().items():
        if only and name not in only:
            continue
        t0 = time.perf_counter()
        model = convert(w["model"](), ns)
        c = compile_model(model, "float32")
        data = compiled_fingerprint(c)
        steps, seed = w["steps"], w["seed"]
        data["steps"], data["seed"] = steps, -1 if seed is None else seed
        eng = {}
        for dtype in ("float32", "float64"):
            e = NumpyEngine(c, dtype)
            if seed is not None:
                for k, arr in enumerate(e.E + e.H):
                    arr[...] = seeded_values(arr.shape, seed, k)
            e.step(steps)
            eng[dtype] = e
            print(name, dtype, f"{time.perf_counter() - t0:.0f} s", flush=True)
        f32, f64 = eng["float32"], eng["float64"]
        for k, v in state_fingerprint(f32).items():
            data[f"float32.{k}"] = v
        data["float64.energy"] = np.float64(f64.energy())
        for pname, v in f64.results().items():
            data[f"float64.dft.{pname}"] = np.asarray(v, np.complex128)
        idx = sample_index(f32.E[0].size, SAMPLES, 99)
        data["sample.index"] = idx
        for k, (a32, a64) in enumerate(zip(f32.E + f32.H, f64.E + f64.H, strict=True)):
            diff = np.linalg.norm((a32.astype(np.float64) - a64).ravel())
            data[f"rel64.{NAMES[k]}"] = float(diff / max(np.linalg.norm(a64.ravel()), 1e-300))
            data[f"float64.sample.{NAMES[k]}"] = np.ascontiguousarray(a64.reshape(-1)[idx])
        if seed is None and model.ports:
            port_r = np.array([float(q["r_ohm"]) for q in c.ports])
            res = RunResult(probes=f32.results(), source_dft=source_spectrum(c, steps), steps=steps, dt=c.dt,
                            engine="numpy", dtype="float32", stopped_by="max_steps", energy_db=0.0, peak_bytes=0,
                            port_r=port_r)
            data["float32.s"] = sparams(model, res)
            r64 = run(model, engine="numpy", dtype="float64", end_db=None, max_steps=steps)
            data["float64.s"] = sparams(model, r64)
        save(str(HERE / f"workload_{name}.npz"), data)
        print(name, "done", f"{time.perf_counter() - t0:.0f} s", flush=True)


COMPILED_CASES = ("dispersive_copper", "mode_stripline")


def reference_compiled(np, ns):  # type: ignore[no-untyped-def]
    """The reference's own ``Compiled`` of two cases, stored with ``compiled_io.dump`` (the
    waveform sampled for the first 128 steps), so the GPU engine can be fed the reference's
    objects on a host without the reference."""
    from cases import CASES  # type: ignore[import-not-found]
    from compiled_io import dump  # type: ignore[import-not-found]
    from oa_fdtd.model import compile_model  # type: ignore[import-not-found]

    for name in COMPILED_CASES:
        c = compile_model(CASES[name][0](ns), "float32")
        np.savez_compressed(HERE / f"ref_compiled_{name}.npz", **dump(c, 128))
        print("reference compiled", name)


def wave_fixture(np, model, c, engine_cls, steps, data):  # type: ignore[no-untyped-def]
    """Mode-port case: the reference's port S-parameters and wave-plane S-parameters (with its
    propagation constants) from its float64 run, the probe parts summed as its run loop does."""
    from oa_fdtd.ports.deembed import wave_sparams  # type: ignore[import-not-found]
    from oa_fdtd.run import port_voltage_factor  # type: ignore[import-not-found]

    eng = engine_cls(c, "float64")
    eng.step(steps)
    probes = eng.results()
    sums = {f"V:{q['name']}": q["probe_parts"] for q in c.ports if q.get("probe_parts")}
    sums.update(c.probe_sums)
    for nm, parts in sums.items():
        probes[nm] = sum(probes.pop(q) for q in parts)
    fac = port_voltage_factor(c.dt, model.frequencies)
    probes = {k: v * fac for k, v in probes.items()}
    port_r = np.array([float(q["r_ohm"]) for q in c.ports])
    s_wave, gammas = wave_sparams(probes, model.plane_sets, port_r)
    data["wave.s"] = s_wave
    data["wave.gamma"] = np.stack(gammas)
    for ps_i, ps in enumerate(model.plane_sets):
        data[f"wave.planes{ps_i}"] = np.array([ps.spacing, ps.ref, ps.spacing_b if ps.spacing_b is not None else np.nan])


def tail_series(np):  # type: ignore[no-untyped-def]
    """Synthetic probe series for the matrix-pencil tail: (name, y, dt, t_first, f_band)."""
    dt = 1e-12
    n = 9000
    t = 1e-9 + np.arange(n) * dt
    two = 0.8 * np.exp(-t / 0.9e-9) * np.cos(2 * np.pi * 7.1e9 * t + 0.3) + 0.35 * np.exp(-t / 0.6e-9) * np.sin(
        2 * np.pi * 12.4e9 * t)
    grow = two + 1e-3 * np.exp(t / 3e-9) * np.cos(2 * np.pi * 45e9 * t)  # growing, out of the band
    quiet = 1e-14 * np.cos(2 * np.pi * 5e9 * t) + np.where(t < 1.2e-9, 1.0, 0.0)  # tail below noise
    return [("two_modes", two, dt, 1e-9, 20e9), ("growing_out_of_band", grow, dt, 1e-9, 20e9),
            ("below_noise", quiet, dt, 1e-9, 20e9)]


def tail_fits(np):  # type: ignore[no-untyped-def]
    """The reference's matrix-pencil tail fits and their DFT continuations on synthetic series."""
    from oa_fdtd.tail import extrapolate_dft, fit_tail  # type: ignore[import-not-found]

    out = {}
    freqs = np.linspace(1e9, 20e9, 12)
    for name, y, dt, t0, fb in tail_series(np):
        fit = fit_tail(y, dt, t0, f_band=fb)
        out[f"{name}.none"] = np.array(fit is None)
        if fit is None:
            continue
        out[f"{name}.s"] = fit.s
        out[f"{name}.c"] = fit.c
        out[f"{name}.meta"] = np.array([fit.t_ref, fit.n_dropped, fit.residual])
        out[f"{name}.dft"] = extrapolate_dft(fit, dt, t0 + y.size * dt, freqs)
    np.savez(HERE / "tail_fits.npz", **out)
    print("tail fits", len(out))


def job_parse(np):  # type: ignore[no-untyped-def]
    """The reference's CLI job parser and compiler on ``cases.job_dict()``: the compiled
    fingerprint."""
    from cases import job_dict  # type: ignore[import-not-found]
    from fingerprint import compiled_fingerprint, save  # type: ignore[import-not-found]
    from oa_fdtd.cli import model_from_job  # type: ignore[import-not-found]
    from oa_fdtd.model import compile_model  # type: ignore[import-not-found]

    c = compile_model(model_from_job(job_dict()), "float32")
    save(str(HERE / "job_parse.npz"), compiled_fingerprint(c))
    print("job parse", c.grid.n)


RUNS = {
    # case: run() keyword arguments (float64 NumPy engine)
    "microstrip": {"max_steps": 6000, "end_db": -40.0},
    "mode_stripline": {"max_steps": 1500, "end_db": -60.0, "tail": True},
}


def run_loops(np):  # type: ignore[no-untyped-def]
    """The reference's own run loop (engine "numpy", float64) on two cases: the step count, why it
    stopped, the energy level, the S-parameters, and the tail continuation where it applies."""
    from cases import CASES, namespace  # type: ignore[import-not-found]
    from oa_fdtd.ports.deembed import wave_sparams  # type: ignore[import-not-found]
    from oa_fdtd.run import port_voltage_factor, run, sparams  # type: ignore[import-not-found]

    out = {}
    for name, kw in RUNS.items():
        m = CASES[name][0](namespace("ref"))
        res = run(m, engine="numpy", dtype="float64", **kw)
        out[f"{name}.steps"] = np.array(res.steps)
        out[f"{name}.stopped_by"] = np.array(res.stopped_by)
        out[f"{name}.energy_db"] = np.array(res.energy_db)
        out[f"{name}.s"] = sparams(m, res)
        if hasattr(m, "plane_sets"):  # wave planes with the port S fallback and gamma smoothing
            fac = port_voltage_factor(res.dt, m.frequencies)
            probes = {k: v * fac for k, v in res.probes.items()}
            sw, gam = wave_sparams(probes, m.plane_sets, res.port_r, s_port=out[f"{name}.s"], freqs=m.frequencies)
            out[f"{name}.wave_s"] = sw
            out[f"{name}.wave_gamma"] = np.stack(gam)
        for k, v in sorted((res.tail or {}).items()):
            if isinstance(v, (int, float, bool)) or (isinstance(v, np.ndarray) and v.dtype.kind in "biufc"):
                out[f"{name}.tail.{k}"] = np.asarray(v)
    np.savez(HERE / "run_loops.npz", **out)
    print("run loops", sorted(out))


# Djordjevic-Sarkar materials fitted by the reference's multi-pole Debye fit:
# (dk, df, f_ref, f_lo, f_hi) [-, -, Hz, Hz, Hz]
DEBYE_CASES = (
    (4.3, 0.02, 1e9, 0.1e9, 12e9),   # the FR-4 of the reference's DS-line test
    (3.7, 0.008, 1e9, 0.05e9, 40e9),
    (3.0, 0.002, 10e9, 1e9, 60e9),
)


def touchstone_files(np):  # type: ignore[no-untyped-def]
    """Touchstone text written by the reference's writer for seeded S matrices: 1, 2 and 3 ports,
    one reference impedance (v1.1) and per-port ones (v2.0)."""
    import importlib.util

    import oa_fdtd  # type: ignore[import-not-found]

    # the module alone: the adapter package imports the framework, absent here
    path = Path(oa_fdtd.__file__).parent / "adapter" / "touchstone.py"
    spec = importlib.util.spec_from_file_location("reference_touchstone", path)
    mod = importlib.util.module_from_spec(spec)  # type: ignore[arg-type]
    spec.loader.exec_module(mod)  # type: ignore[union-attr]
    format_touchstone = mod.format_touchstone

    rng = np.random.default_rng(11)
    out = {}
    for n, z0 in ((1, [50.0]), (2, [50.0, 50.0]), (2, [49.2, 51.0]), (3, [50.0, 50.0, 50.0]), (3, [25.0, 50.0, 75.0])):
        freqs = np.linspace(1e9, 5e9, 4)
        s = rng.standard_normal((4, n, n)) + 1j * rng.standard_normal((4, n, n))
        names = [f"port{i + 1}" for i in range(n)]
        key = f"n{n}_" + "_".join(f"{z:g}" for z in z0)
        out[key + ".s"] = s
        out[key + ".freqs"] = freqs
        out[key + ".z0"] = np.array(z0)
        out[key + ".text"] = np.array(format_touchstone(freqs, s, z0, names, ["made by the reference"]))
    np.savez(HERE / "touchstone.npz", **out)
    print("touchstone", len(out) // 4)


def debye_fits(np):  # type: ignore[no-untyped-def]
    from oa_fdtd.materials import fit_djordjevic_sarkar  # type: ignore[import-not-found]

    out = {}
    for n, (dk, df, fr, lo, hi) in enumerate(DEBYE_CASES):
        fit = fit_djordjevic_sarkar(dk, df, fr, lo, hi)
        out[f"{n}.case"] = np.array([dk, df, fr, lo, hi])
        out[f"{n}.eps_inf"] = np.array([fit.eps_inf])
        out[f"{n}.delta"] = fit.delta
        out[f"{n}.tau"] = fit.tau
        out[f"{n}.err"] = np.array([fit.err_eps, fit.err_tand])
    np.savez(HERE / "debye_fits.npz", **out)
    print("debye fits", len(DEBYE_CASES))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py <reference root> [part ...]; parts: " + " ".join(PARTS))
    main(sys.argv[1], tuple(sys.argv[2:]) or PARTS)
