"""Known answers: the reference's analytic validation cases on the GPU engine (``-m gpu``) and,
where they are cheap, on the CPU oracle (which pins the oracle to the same answers).

The cases and their bars are the reference's (``tests/golden/fdtd/{cavity,cpml,tem_line}`` and
``tests/golden/fdtd_physics/{ds_line,sibc_line}`` of the reference project, and
``packages/oa-fdtd/tests/test_analytic.py`` / ``test_physics.py``): cavity resonances to 5e-4
after Richardson extrapolation with observed order 2, CPML reflection below -60 dB from 0.1 to
40 GHz, late-time energy decay below -80 dB, a matched TEM line with |S21| = 1 to 1e-4 and
S11 below -45 dB, a mismatched port with |S11| = 1/3, the Yee dispersion relation, leapfrog
energy conservation over 1e5 steps, a Djordjevic-Sarkar line within 0.02 dB / 1 degree and a
surface-impedance line within 2 % of its loss.
"""

from __future__ import annotations

import numpy as np
import pytest
from known_answers import (
    cavity_frequencies,
    cavity_mode_freq,
    copper_line_s,
    cpml_reflection,
    db,
    dielectric_line_s,
    graded_lines,
    line_model,
    plate_line,
    refine,
    tem_model,
)

from open_analysis_gb300.grid import C0, EPS0, MU0, Grid
from open_analysis_gb300.materials import fit_djordjevic_sarkar
from open_analysis_gb300.model import Model, Probe, SoftSource, Waveform, compile_model
from open_analysis_gb300.run import run, sparams
from open_analysis_gb300.sibc import slab_surface_impedance
from oracle.numpy_engine import OracleEngine

GPU = pytest.param("gb300", marks=pytest.mark.gpu)
CPU = pytest.param(OracleEngine, id="oracle")


def _dtype(engine: object) -> str:
    return "float32" if engine == "gb300" else "float64"


# ----------------------------------------------------------------------------------- cavity
A, B, D = 0.030, 0.025, 0.035
MODES = [(1, 0, 1), (0, 1, 1), (1, 1, 0)]  # TE101, TE011, TM110
TARGETS = [cavity_mode_freq(A, B, D, *m) for m in MODES]


def test_cavity_targets_match_the_golden_case() -> None:
    np.testing.assert_allclose(TARGETS, [6580833082.124073, 7368320675.20633, 7804846493.112532], rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("ratio", [1.0, 1.05], ids=["uniform", "graded"])
def test_cavity_richardson(ratio: float) -> None:
    """Three grids (10x8x12 cells and two bisections), float32: the extrapolated resonances
    within 5e-4 of the analytic ones, the observed order of convergence 2."""
    levels = [(graded_lines(A, 10, ratio), graded_lines(B, 8, ratio), graded_lines(D, 12, ratio))]
    for _ in range(2):
        levels.append(tuple(refine(v) for v in levels[-1]))  # type: ignore[arg-type]
    f1, f2, f3 = (np.array(cavity_frequencies(lv, TARGETS, "gb300", "float32", 30e-9)) for lv in levels)
    order = float(np.median(np.log2(np.abs(f1 - f2) / np.abs(f2 - f3))))
    extrapolated = f3 + (f3 - f2) / 3.0
    err = np.abs(extrapolated - np.array(TARGETS)) / np.array(TARGETS)
    assert err.max() < 5e-4, err
    assert 1.8 < order < 2.2, order


# ------------------------------------------------------------------------------------- CPML
@pytest.mark.parametrize(
    ("engine", "side"),
    [
        pytest.param("gb300", "hi", marks=pytest.mark.gpu),
        pytest.param("gb300", "lo", marks=pytest.mark.gpu),
        pytest.param(OracleEngine, "hi", id="oracle-hi"),  # one side on the CPU keeps the suite short
    ],
)
def test_cpml_reflection_below_60_db(engine: object, side: str) -> None:
    f = np.array([0.1e9, 0.5e9, 1e9, 5e9, 10e9, 20e9, 30e9, 40e9])
    r = cpml_reflection(f, engine, _dtype(engine), side)
    assert float(db(r.max())) < -60.0


@pytest.mark.parametrize("engine", [GPU, CPU])
def test_cpml_late_time_energy_decay(engine: object) -> None:
    d = C0 / 40e9 / 20.0
    m = line_model(80, d, np.array([1e9]), 20, 40, dc=False)
    res = run(m, engine=engine, dtype="float64", end_db=-80.0, max_steps=20000, min_steps=200)
    assert res.stopped_by == "end_criterion"
    assert res.energy_db <= -80.0


# -------------------------------------------------------------------------------- TEM lines
@pytest.mark.gpu
def test_parallel_plate_tem_line() -> None:
    """Port R = Z0 = eta0 h / w: a matched, lossless line (float32)."""
    m = tem_model(20e9)
    res = run(m, engine="gb300", dtype="float32", end_db=-70.0, max_steps=20000)
    s = sparams(m, res)
    assert np.abs(s[0, 0]).max() < 10 ** (-45 / 20)
    assert np.abs(np.abs(s[1, 0]) - 1.0).max() < 1e-4
    assert np.abs(s[1, 0] - s[0, 1]).max() < 1e-6  # reciprocity


@pytest.mark.parametrize("engine", [GPU, CPU])
def test_mismatched_port_reflection(engine: object) -> None:
    """A port R = 2 Z0 reflects |S11| = 1/3."""
    m = tem_model()
    m = tem_model(r_first=2 * m.ports[0].r_ohm)
    res = run(m, engine=engine, dtype=_dtype(engine), end_db=-70.0, max_steps=20000)
    s = sparams(m, res)
    assert np.abs(np.abs(s[0, 0]) - 1.0 / 3.0).max() < 1e-3


@pytest.mark.parametrize("engine", [GPU, CPU])
def test_yee_dispersion(engine: object) -> None:
    """The phase constant between two planes 20 cells apart equals the Yee dispersion relation's
    (and differs visibly from the continuum's)."""
    d = C0 / 40e9 / 20.0
    freqs = np.array([2e9, 5e9, 10e9, 20e9, 30e9])
    m = line_model(120, d, freqs, 60, 70)
    m.probes.clear()
    for name, yy in (("a", 75), ("b", 95)):
        m.probes.append(Probe(name, "E", 2, (0, yy * d, 0), (2 * d, yy * d, 2 * d), "mean"))
    dtype = _dtype(engine)
    res = run(m, engine=engine, dtype=dtype, end_db=None, max_steps=1200)
    ratio = res.probes["b"][0] / res.probes["a"][0]
    k_num = -np.unwrap(np.angle(ratio)) / (20 * d)
    k_yee = 2.0 / d * np.arcsin(d / (C0 * res.dt) * np.sin(np.pi * freqs * res.dt))
    assert np.abs(k_num / k_yee - 1.0).max() < (1e-3 if dtype == "float64" else 2e-3)
    assert np.abs(k_num / (2 * np.pi * freqs / C0) - 1.0).max() > 1e-4


# ------------------------------------------------------------------------- energy drift
def _leapfrog_energy(c, h_prev, fields) -> float:  # type: ignore[no-untyped-def]
    """E^n with H^{n-1/2} . H^{n+1/2}: the energy the leapfrog scheme conserves exactly."""
    g = c.grid

    def weights(kind: str, comp: int) -> np.ndarray:
        out = np.ones((1, 1, 1, 1))
        for a in range(3):
            node = (a != comp) if kind == "E" else (a == comp)
            w = g.node_weights(a) if node else g.cell_weights(a)
            shape = [1, 1, 1, 1]
            shape[3 - a] = w.size
            out = out * w.reshape(shape)
        return out

    total = 0.0
    for ci, (en, hn) in enumerate((("Ex", "Hx"), ("Ey", "Hy"), ("Ez", "Hz"))):
        eps = (c.eps_tab[c.idx[ci]] * EPS0)[None]
        total += 0.5 * float(np.sum(eps * weights("E", ci) * fields[en] ** 2))
        total += 0.5 * MU0 * float(np.sum(weights("H", ci) * h_prev[ci] * fields[hn]))
    return total


def _drift(dtype: str, steps: int) -> float:
    from open_analysis_gb300.engine import Gb300Engine

    lines = (graded_lines(0.02, 8, 1.1), graded_lines(0.017, 6, 1.0), graded_lines(0.024, 9, 0.9))
    m = Model(Grid(*lines), Waveform("gauss_mod", 8e9, 16e9), np.array([1e9]))
    m.sources.append(SoftSource("s", 2, (0.007, 0.006, 0.01), (0.007, 0.006, 0.01)))
    c = compile_model(m, dtype)
    eng = Gb300Engine(c, dtype, max_steps=steps + 1000, use_graph=True)

    def snap() -> tuple[list[np.ndarray], dict[str, np.ndarray]]:
        f = eng.get_fields()
        return [f["Hx"], f["Hy"], f["Hz"]], f

    eng.step(800)  # the source pulse has ended
    energies = []
    for more in (0, steps - 801):
        if more:
            eng.step(more)
        h_prev, f0 = snap()
        eng.step(1)
        _, f1 = snap()
        energies.append(_leapfrog_energy(c, h_prev, {**f0, "Hx": f1["Hx"], "Hy": f1["Hy"], "Hz": f1["Hz"]}))
    return abs(energies[1] - energies[0]) / energies[0]


@pytest.mark.gpu
def test_closed_box_energy_drift_float64_1e5_steps() -> None:
    assert _drift("float64", 100_000) < 1e-6


@pytest.mark.gpu
def test_closed_box_energy_drift_float32_reported() -> None:
    drift = _drift("float32", 100_000)
    print(f"float32 energy drift over 1e5 steps: {drift:.3e}")
    assert drift < 1e-2


# ------------------------------------------------------------------ dispersive and lossy lines
@pytest.mark.gpu
def test_debye_ds_line_matches_analytic() -> None:
    """FR-4 (Djordjevic-Sarkar 4.3 / 0.02 at 1 GHz, Debye fit over 0.1-12 GHz) filling a 12 mm
    line: S21 within 0.02 dB and 1 degree, S11 within 0.01 of the analytic line (float32)."""
    fit = fit_djordjevic_sarkar(4.3, 0.02, 1e9, 0.1e9, 12e9)
    freqs = np.linspace(1e9, 10e9, 10)
    length, dy = 0.012, 0.25e-3
    m = plate_line(length, dy, freqs, 12e9, poles=fit.poles, eps_inf=fit.eps_inf)
    res = run(m, engine="gb300", dtype="float32", end_db=-60.0, max_steps=40000)
    s = sparams(m, res)
    s11, s21 = dielectric_line_s(freqs, fit.eval(freqs), length, m.ports[0].r_ohm)
    assert np.abs(db(s[1, 0]) - db(s21)).max() < 0.02
    assert np.abs(np.angle(s[1, 0] / s21, deg=True)).max() < 1.0
    assert np.abs(s[0, 0] - s11).max() < 0.01
    assert abs(float(db(s21[-1])) - (-0.4420)) < 0.02  # the golden value at 10 GHz


@pytest.mark.gpu
def test_sibc_line_attenuation() -> None:
    """Plates of 2e5 S/m, 0.25 mm thick, 60 mm line: S21 within 2 % of the loss and 1 degree of
    the line with the slab surface impedance (float32)."""
    sigma, t = 2e5, 0.25e-3
    freqs = np.linspace(1e9, 10e9, 10)
    length, dy = 0.06, 0.25e-3
    m = plate_line(length, dy, freqs, 12e9, sigma_cu=sigma, t_cu=t)
    res = run(m, engine="gb300", dtype="float32", end_db=-60.0, max_steps=40000)
    s = sparams(m, res)
    _, s21 = copper_line_s(freqs, slab_surface_impedance(freqs, sigma, t), length, m.ports[0].r_ohm)
    loss = db(s21)
    assert loss.min() < -0.5
    assert np.abs(db(s[1, 0]) - loss).max() < 0.02 * np.abs(loss).max()
    assert np.abs(np.angle(s[1, 0] / s21, deg=True)).max() < 1.0
    assert abs(float(loss[-1]) - (-0.6112)) < 0.02 * 0.6112  # the golden value at 10 GHz
