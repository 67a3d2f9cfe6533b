"""Problem builders and analytic answers for the known-answer tests.

The problems are the reference's own analytic validation cases (its ADR-0010 section 9 cases,
``tests/golden/fdtd/*/case.toml`` and ``tests/golden/fdtd_physics/*/case.toml`` of the reference
project; problem set-up as in ``packages/oa-fdtd/tests/fdtd_helpers.py`` and
``fdtd_phys_helpers.py``): a PEC cavity, normal incidence on a CPML, parallel-plate TEM lines
with lumped ports, a Debye-dielectric line and a surface-impedance line, each with its closed-form
answer. ``engine`` is anything ``open_analysis_gb300.run.run`` accepts.
"""

from __future__ import annotations

from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.grid import C0, EPS0, ETA0, MU0, Grid
from open_analysis_gb300.model import (
    Conductor,
    LumpedPort,
    Model,
    Probe,
    Region,
    SoftSource,
    Waveform,
    compile_model,
)
from open_analysis_gb300.pml import CpmlSpec
from open_analysis_gb300.run import run
from open_analysis_gb300.tail import matrix_pencil

FloatArray = npt.NDArray[np.float64]
ComplexArray = npt.NDArray[np.complex128]

PLATE_W, PLATE_H = 0.008, 0.001  # parallel-plate line width and gap [m]


# ----------------------------------------------------------------------------------- grids
def graded_lines(length: float, n: int, ratio: float) -> FloatArray:
    """``n`` cells over ``length`` growing by ``ratio`` from cell to cell (1: uniform)."""
    if ratio == 1.0:
        return np.linspace(0.0, length, n + 1)
    widths = ratio ** np.arange(n)
    return np.concatenate([[0.0], np.cumsum(widths) / widths.sum() * length])


def refine(lines: FloatArray) -> FloatArray:
    """Every cell halved (the grading ratio per original cell is kept)."""
    out = np.empty(2 * lines.size - 1)
    out[0::2] = lines
    out[1::2] = 0.5 * (lines[1:] + lines[:-1])
    return out


# ---------------------------------------------------------------------------------- cavity
def cavity_mode_freq(a: float, b: float, d: float, m: int, n: int, p: int) -> float:
    """Resonance of mode (m, n, p) of an a x b x d PEC box [Hz]."""
    return 0.5 * C0 * float(np.sqrt((m / a) ** 2 + (n / b) ** 2 + (p / d) ** 2))


def cavity_frequencies(
    lines: tuple[FloatArray, FloatArray, FloatArray], targets: list[float], engine: Any, dtype: str, t_end: float
) -> list[float]:
    """Ring a PEC box with three point sources, record three E probes and return, per target,
    the nearest matrix-pencil frequency of their summed signal [Hz]."""
    from open_analysis_gb300.run import make_engine

    g = Grid(*lines)
    ext = [float(v[-1] - v[0]) for v in lines]
    wf = Waveform("gauss_mod", f0=0.5 * (min(targets) + max(targets)), bandwidth=2.0 * max(targets))
    model = Model(g, wf, np.array([1e9]))
    src = tuple(e * r for e, r in zip(ext, (0.31, 0.37, 0.43), strict=True))
    obs = tuple(e * r for e, r in zip(ext, (0.67, 0.29, 0.61), strict=True))
    for ax in range(3):
        model.sources.append(SoftSource(f"s{ax}", ax, src, src))
        model.probes.append(Probe(f"p{ax}", "E", ax, obs, obs))
    c = compile_model(model, dtype)
    steps = int(t_end / c.dt)
    eng, _ = make_engine(c, engine, dtype, True, steps + 64)
    eng.step(steps)
    series = eng.series()
    signal = sum(series[f"p{ax}"][0] for ax in range(3))
    freqs, _ = matrix_pencil(signal, c.dt, order=2 * len(targets) + 10, decimate=4)
    return [float(freqs[np.argmin(np.abs(freqs - t))]) for t in targets]


# ------------------------------------------------------------------------------ TEM lines
def line_model(ny: int, d: float, freqs: FloatArray, src_y: int, probe_y: int, cells: int = 10, dc: bool = True) -> Model:
    """A cubic-cell TEM line along y (PMC x walls, PEC z walls, CPML at both y ends) with an E_z
    plane source and an E_z plane probe."""
    across = np.arange(3) * d
    g = Grid(across, np.arange(ny + 1) * d, across)
    wf = Waveform("gauss", bandwidth=45e9) if dc else Waveform("gauss_mod", 20e9, 40e9)
    m = Model(g, wf, freqs, walls=("pmc", "pmc", "cpml", "cpml", "pec", "pec"), cpml=CpmlSpec(cells=cells))
    m.sources.append(SoftSource("s", 2, (0.0, src_y * d, 0.0), (2 * d, src_y * d, 2 * d)))
    m.probes.append(Probe("p", "E", 2, (0.0, probe_y * d, 0.0), (2 * d, probe_y * d, 2 * d), "mean"))
    return m


def cpml_reflection(freqs: FloatArray, engine: Any, dtype: str, side: str, cells: int = 10, steps: int = 3000) -> FloatArray:
    """|reflected / incident| of a wave at normal incidence on a ``cells``-cell CPML: the probe of a
    short line minus the same probe on a line 1400 cells longer (no reflection in the window)."""
    d = C0 / 40e9 / 20.0
    n, extra = 2 * cells + 60, 1400
    s0, p0 = cells + 10, cells + 30
    if side == "hi":
        short = line_model(n, d, freqs, s0, p0, cells)
        long_ = line_model(n + extra, d, freqs, s0, p0, cells)
    else:  # the wave runs towards the low-y CPML
        short = line_model(n, d, freqs, n - s0, n - p0, cells)
        long_ = line_model(n + extra, d, freqs, n - s0 + extra, n - p0 + extra, cells)
    a = run(short, engine=engine, dtype=dtype, end_db=None, max_steps=steps).probes["p"][0]
    b = run(long_, engine=engine, dtype=dtype, end_db=None, max_steps=steps).probes["p"][0]
    return np.asarray(np.abs(a - b) / np.abs(b))


def tem_model(f_max: float = 3e9, r_first: float | None = None) -> Model:
    """An 8 mm x 4 mm parallel-plate line, 60 mm long (0.5 mm cells), PMC sides, lumped ports of
    Z0 = eta0 h / w across the gap at both ends (``r_first`` overrides the first port's R)."""
    w, h = 0.008, 0.004
    z0 = ETA0 * h / w
    nx, nz, ny, dy = 4, 4, 120, 0.5e-3
    g = Grid(np.linspace(0, w, nx + 1), np.arange(ny + 1) * dy, np.linspace(0, h, nz + 1))
    ports = [
        LumpedPort("p1", 2, (0, 0.0, 0), (w, 0.0, h), z0 if r_first is None else r_first),
        LumpedPort("p2", 2, (0, ny * dy, 0), (w, ny * dy, h), z0),
    ]
    return Model(
        g,
        Waveform("gauss_mod", f_max / 2.0, f_max),
        np.linspace(0.5e9, f_max, 12),
        walls=("pmc", "pmc", "pmc", "pmc", "pec", "pec"),
        ports=ports,
    )


# ------------------------------------------------------------------- plate lines with loss
def plate_line(
    length: float,
    dy: float,
    freqs: FloatArray,
    f_max: float,
    *,
    poles: tuple[tuple[float, float], ...] = (),
    eps_inf: float = 1.0,
    sigma_cu: float | None = None,
    t_cu: float = 0.25e-3,
) -> Model:
    """A TEM line between two one-cell-thick plates (surface-impedance copper of ``sigma_cu``,
    else PEC), PMC side walls, lumped ports across the gap at both ends; the gap is filled with
    ``eps_inf`` and Debye ``poles`` when given."""
    nx, nz_gap = 4, 4
    dz = PLATE_H / nz_gap
    ny = round(length / dy)
    zl = [0.0, t_cu, *[t_cu + (i + 1) * dz for i in range(nz_gap)], 2 * t_cu + PLATE_H]
    g = Grid(np.linspace(0, PLATE_W, nx + 1), np.arange(ny + 1) * dy, np.array(zl))
    z0 = ETA0 * PLATE_H / PLATE_W / np.sqrt(eps_inf)
    ports = [
        LumpedPort("p1", 2, (0, 0, t_cu), (PLATE_W, 0, t_cu + PLATE_H), z0),
        LumpedPort("p2", 2, (0, ny * dy, t_cu), (PLATE_W, ny * dy, t_cu + PLATE_H), z0),
    ]
    regions = []
    if poles or eps_inf != 1.0:
        regions = [Region((0, 0, t_cu), (PLATE_W, length, t_cu + PLATE_H), eps_inf, poles=poles)]
    big = 1.0
    kind = "pec" if sigma_cu is None else "thick_sibc"
    sig = 5.8e7 if sigma_cu is None else sigma_cu
    conductors = [
        Conductor((-big, -big, -big), (PLATE_W + big, length + big, t_cu), sig, t_cu, model=kind),
        Conductor((-big, -big, t_cu + PLATE_H), (PLATE_W + big, length + big, 3 * t_cu + PLATE_H), sig, t_cu, model=kind),
    ]
    return Model(
        g,
        Waveform("gauss_mod", f_max / 2.0, f_max),
        freqs,
        regions=regions,
        conductors=conductors,
        walls=("pmc", "pmc", "pmc", "pmc", "pec", "pec"),
        ports=ports,
    )


def abcd_s(gamma: ComplexArray, zc: ComplexArray, length: float, r1: float, r2: float) -> tuple[ComplexArray, ComplexArray]:
    """``(S11, S21)`` of a uniform line section (propagation ``gamma``, impedance ``zc``) between
    resistive ports ``r1`` and ``r2``, from its ABCD matrix."""
    ch, sh = np.cosh(gamma * length), np.sinh(gamma * length)
    a, b, c, d = ch, zc * sh, sh / zc, ch
    den = a * r2 + b + c * r1 * r2 + d * r1
    return (a * r2 + b - c * r1 * r2 - d * r1) / den, 2.0 * np.sqrt(r1 * r2) / den


def dielectric_line_s(freqs: FloatArray, eps: ComplexArray, length: float, r_port: float) -> tuple[ComplexArray, ComplexArray]:
    """Analytic S of the plate line filled with relative permittivity ``eps(f)``."""
    root = np.sqrt(eps)
    gamma = 1j * 2 * np.pi * freqs * root / C0
    return abcd_s(gamma, ETA0 * PLATE_H / PLATE_W / root, length, r_port, r_port)


def copper_line_s(freqs: FloatArray, zs: ComplexArray, length: float, r_port: float) -> tuple[ComplexArray, ComplexArray]:
    """Analytic S of the vacuum plate line whose two plates have surface impedance ``zs``."""
    w = 2 * np.pi * freqs
    z_series = 1j * w * MU0 * PLATE_H / PLATE_W + 2.0 * zs / PLATE_W
    y_shunt = 1j * w * EPS0 * PLATE_W / PLATE_H
    return abcd_s(np.sqrt(z_series * y_shunt), np.sqrt(z_series / y_shunt), length, r_port, r_port)


def db(x: Any) -> FloatArray:
    return np.asarray(20 * np.log10(np.abs(x)))
