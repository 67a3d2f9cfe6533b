"""Small problems shared by the fixture generator and the parity tests.

Each builder takes a namespace ``ns`` holding the problem types (``Grid, Model, Region,
Conductor, LumpedPort, SoftSource, Probe, Waveform, CpmlSpec``), so the same problem can be built
from the reference's own classes (when generating fixtures) and from ``open_analysis_gb300``.
The problems cover every feature of the time step: graded grids, CPML on some walls, PMC and PEC
walls, lossy dielectrics, PEC regions, lumped ports, soft sources, E and H probes, batch > 1,
multi-pole Debye dielectrics and surface-impedance copper.
"""

from __future__ import annotations

from types import SimpleNamespace
from typing import Any

import numpy as np


def graded(length: float, n: int, ratio: float) -> np.ndarray:
    """``n`` cells over ``length`` with geometric growth ``ratio`` per cell."""
    if ratio == 1.0:
        return np.linspace(0.0, length, n + 1)
    w = ratio ** np.arange(n)
    return np.concatenate([[0.0], np.cumsum(w) / w.sum() * length])


def mixed_walls(ns: Any, batch: int = 2) -> Any:
    """Graded 24x20x22 box: CPML x, PMC y, PEC z; lossy slab, PEC patch, source, port, probes."""
    lines = (graded(0.024, 24, 1.03), graded(0.02, 20, 1.0), graded(0.022, 22, 0.97))
    m = ns.Model(
        ns.Grid(*lines),
        ns.Waveform("gauss_mod", 10e9, 20e9),
        np.array([2e9, 6e9, 10e9, 14e9]),
        walls=("cpml", "cpml", "pmc", "pmc", "pec", "pec"),
    )
    m.cpml = ns.CpmlSpec(cells=4)
    m.regions.append(ns.Region((0, 0, 0.004), (0.024, 0.02, 0.012), eps_r=4.4, sigma=0.02))
    m.regions.append(ns.Region((0.008, 0.006, 0.012), (0.016, 0.014, 0.0121), pec=True))
    m.sources.append(ns.SoftSource("s", 2, (0.012, 0.01, 0.006), (0.012, 0.01, 0.006)))
    m.ports.append(ns.LumpedPort("p", 2, (0.006, 0.01, 0.0), (0.006, 0.01, 0.004), 50.0))
    m.probes.append(ns.Probe("e", "E", 2, (0.016, 0.01, 0.002), (0.016, 0.01, 0.002)))
    m.probes.append(ns.Probe("h", "H", 1, (0.016, 0.01, 0.002), (0.016, 0.01, 0.002)))
    if batch > 1:
        m.drive = np.array([[1.0, 1.0], [0.0, -2.0]])[:batch]
    return m


def dispersive_copper(ns: Any) -> Any:
    """18x16x20 via-like stack: two-pole Debye dielectric, SIBC plane with a hole, SIBC barrel,
    two lumped ports (two batch members), CPML on x and z-high, PMC on y-low, PEC elsewhere."""
    h = 0.25e-3
    g = ns.Grid(
        np.arange(19) * h,
        graded(16 * h, 16, 1.02),
        np.arange(21) * h,
    )
    m = ns.Model(
        g,
        ns.Waveform("gauss_mod", 10e9, 18e9),
        np.linspace(1e9, 19e9, 7),
        walls=("cpml", "cpml", "pmc", "pec", "pec", "cpml"),
    )
    m.cpml = ns.CpmlSpec(cells=4, kappa_max=5.0)
    m.regions.append(
        ns.Region((0, 0, 2 * h), (18 * h, 16 * h, 14 * h), 3.8, 0.0, False, ((0.3, 8e-12), (0.15, 40e-12)))
    )
    cx, cy = 9 * h, 8 * h
    # plane at z = 8 h with a square antipad of 4 cells around the barrel
    for lo, hi in (
        ((-1, -1, 8 * h), (cx - 2 * h, 1, 9 * h)),
        ((cx + 2 * h, -1, 8 * h), (1, 1, 9 * h)),
        ((cx - 2 * h, -1, 8 * h), (cx + 2 * h, cy - 2 * h, 9 * h)),
        ((cx - 2 * h, cy + 2 * h, 8 * h), (cx + 2 * h, 1, 9 * h)),
    ):
        m.conductors.append(ns.Conductor(lo, hi, 5.8e7, 35e-6))
    m.conductors.append(ns.Conductor((cx - h, cy - h, 3 * h), (cx + h, cy + h, 13 * h), 5.8e7, 35e-6))
    m.ports.append(ns.LumpedPort("p1", 2, (cx, cy, 13 * h), (cx, cy, 15 * h), 50.0))
    m.ports.append(ns.LumpedPort("p2", 2, (cx, cy, h), (cx, cy, 3 * h), 50.0))
    m.probes.append(ns.Probe("hx", "H", 0, (4 * h, 5 * h, 6 * h), (5 * h, 6 * h, 6 * h), "line"))
    m.probes.append(ns.Probe("ez", "E", 2, (4 * h, 5 * h, 5 * h), (6 * h, 6 * h, 7 * h), "mean"))
    return m


def microstrip(ns: Any, nx: int = 40, ny: int = 24, nz: int = 16, cpml: int = 6) -> Any:
    """Microstrip at 50 um cells: FR-4 (4.3) slab 4 cells high, zero-thickness PEC strip of
    7 cells on top, PEC ground (z low), CPML elsewhere; lumped ports under both strip ends."""
    h = 50e-6
    g = ns.Grid(np.arange(nx + 1) * h, np.arange(ny + 1) * h, np.arange(nz + 1) * h)
    m = ns.Model(
        g,
        ns.Waveform("gauss_mod", 10e9, 20e9),
        np.linspace(0.5e9, 20e9, 16),
        walls=("cpml", "cpml", "cpml", "cpml", "pec", "cpml"),
        courant=0.99,
    )
    m.cpml = ns.CpmlSpec(cells=cpml, m=3.0, kappa_max=5.0)
    sub = 4 * h
    m.regions.append(ns.Region((-1, -1, 0.0), (1, 1, sub), 4.3))
    yc = (ny // 2) * h
    x0, x1 = (cpml + 2) * h, (nx - cpml - 2) * h
    m.regions.append(ns.Region((x0, yc - 3.5 * h, sub), (x1, yc + 3.5 * h, sub), pec=True))
    m.ports.append(ns.LumpedPort("p1", 2, (x0, yc, 0.0), (x0, yc, sub), 50.0))
    m.ports.append(ns.LumpedPort("p2", 2, (x1, yc, 0.0), (x1, yc, sub), 50.0))
    return m


def mode_stripline(ns: Any) -> Any:
    """60x22x14 stripline: single-pole Debye fill between PEC z walls, PEC y walls (graded y),
    CPML on x, a zero-thickness PEC strip, quasi-TEM mode ports at both strip ends (both driven,
    batch of two) and three wave planes behind each port (mode probes)."""
    h = 0.1e-3
    nx, ny, nz = 60, 22, 14
    g = ns.Grid(np.arange(nx + 1) * h, graded(ny * 0.1e-3, ny, 1.02), np.arange(nz + 1) * h)
    m = ns.Model(
        g,
        ns.Waveform("gauss_mod", 10e9, 18e9),
        np.linspace(1e9, 19e9, 7),
        walls=("cpml", "cpml", "pec", "pec", "pec", "pec"),
    )
    m.cpml = ns.CpmlSpec(cells=4)
    m.regions.append(ns.Region((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), eps_r=3.4, poles=((0.3, 8e-12),)))
    ys = g.lines[1]
    y0, y1, zc = float(ys[8]), float(ys[14]), 7 * h
    x0, x1 = 6 * h, (nx - 6) * h
    m.regions.append(ns.Region((x0, y0, zc), (x1, y1, zc), pec=True))
    rect = ((float(ys[0]), 0.0), (float(ys[-1]), nz * h))
    sig = (((y0, zc), (y1, zc)),)
    m.ports.append(ns.ModePort("p1", 0, x0, rect[0], rect[1], sig, direction=1))
    m.ports.append(ns.ModePort("p2", 0, x1, rect[0], rect[1], sig, direction=-1))
    m.plane_sets = [ns.add_wave_planes(m, "p1", 3 * h), ns.add_wave_planes(m, "p2", 3 * h)]
    return m


CASES = {
    "mixed_walls": (mixed_walls, 40),
    "dispersive_copper": (dispersive_copper, 40),
    "microstrip": (microstrip, 60),
    "mode_stripline": (mode_stripline, 60),
}


def job_dict() -> dict[str, Any]:
    """An engine-level job in the reference's CLI format using every key it reads: graded grid
    lines, walls with CPML and PMC, a CPML spec, the Courant number, a lossy dielectric and a PEC
    region, two lumped ports (one with a sign), a soft source, E and H probes with each weight."""
    x = graded(0.012, 18, 1.02).tolist()
    y = graded(0.010, 14, 1.0).tolist()
    z = graded(0.006, 12, 0.98).tolist()
    return {
        "grid": {"x": x, "y": y, "z": z},
        "waveform": {"kind": "gauss_mod", "f0": 8e9, "bandwidth": 12e9},
        "frequencies": np.linspace(2e9, 14e9, 5).tolist(),
        "walls": ["cpml", "cpml", "pmc", "pmc", "pec", "cpml"],
        "cpml": {"cells": 4, "m": 3.0, "kappa_max": 4.0},
        "courant": 0.9,
        "regions": [
            {"lo": [-1, -1, 0.0], "hi": [1, 1, 0.002], "eps_r": 3.7, "sigma": 0.01},
            {"lo": [0.004, 0.003, 0.002], "hi": [0.008, 0.007, 0.002], "pec": True},
        ],
        "ports": [
            {"name": "a", "axis": 2, "lo": [0.004, 0.005, 0.0], "hi": [0.004, 0.005, 0.002], "r_ohm": 50.0},
            {"name": "b", "axis": 2, "lo": [0.008, 0.005, 0.0], "hi": [0.008, 0.005, 0.002], "r_ohm": 35.0, "sign": -1.0},
        ],
        "sources": [{"name": "s", "axis": 1, "lo": [0.006, 0.005, 0.003], "hi": [0.006, 0.005, 0.003], "amplitude": 0.5}],
        "probes": [
            {"name": "e_line", "kind": "E", "axis": 2, "lo": [0.006, 0.005, 0.0], "hi": [0.006, 0.005, 0.002], "weight": "line"},
            {"name": "h_mean", "kind": "H", "axis": 0, "lo": [0.005, 0.004, 0.003], "hi": [0.007, 0.006, 0.003], "weight": "mean"},
            {"name": "e_sum", "kind": "E", "axis": 0, "lo": [0.006, 0.005, 0.004], "hi": [0.006, 0.005, 0.004]},
        ],
    }


def namespace(module_root: str) -> Any:
    """Problem types of ``open_analysis_gb300`` (``module_root="gb300"``) or of the reference
    package (``module_root="ref"``, importable only where the reference is present)."""
    if module_root == "gb300":
        from open_analysis_gb300 import deembed, grid, model, pml

        return SimpleNamespace(
            Grid=grid.Grid,
            Model=model.Model,
            Region=model.Region,
            Conductor=model.Conductor,
            LumpedPort=model.LumpedPort,
            ModePort=model.ModePort,
            SoftSource=model.SoftSource,
            Probe=model.Probe,
            Waveform=model.Waveform,
            CpmlSpec=pml.CpmlSpec,
            add_wave_planes=deembed.add_wave_planes,
        )
    from oa_fdtd import grid as rgrid  # type: ignore[import-not-found]
    from oa_fdtd import model as rmodel  # type: ignore[import-not-found]
    from oa_fdtd import pml as rpml  # type: ignore[import-not-found]
    from oa_fdtd.ports import deembed as rdeembed  # type: ignore[import-not-found]

    return SimpleNamespace(
        Grid=rgrid.Grid,
        Model=rmodel.Model,
        Region=rmodel.Region,
        Conductor=rmodel.Conductor,
        LumpedPort=rmodel.LumpedPort,
        ModePort=rmodel.ModePort,
        SoftSource=rmodel.SoftSource,
        Probe=rmodel.Probe,
        Waveform=rmodel.Waveform,
        CpmlSpec=rpml.CpmlSpec,
        add_wave_planes=rdeembed.add_wave_planes,
    )
