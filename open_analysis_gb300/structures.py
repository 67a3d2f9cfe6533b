"""Synthetic engine-level problems with the shapes of the benchmark workloads.

No board files or meshers are needed (the reference's EMProblem front end is not part of this
package): each builder returns a :class:`~open_analysis_gb300.model.Model` directly, with seeded
geometry where the workload calls for randomness.

* :func:`microstrip` — 50-ohm-class microstrip, 120 x 60 x 40 cells of 50 um, FR-4 (4.3)
  substrate 0.2 mm, zero-thickness PEC strip 0.36 mm wide, PEC ground, 8-cell CPML (m = 3,
  kappa_max = 5), Gaussian-derivative source 0-20 GHz, 0.99 Courant, two lumped ports, 64 DFT
  frequencies.
* :func:`via_transition` — 400 x 400 x 120 cells of 25 um: a four-layer stack with a single-pole
  Debye dielectric (eps_inf 4.0, delta_eps 0.35, tau 8 ps), three copper planes and two trace
  layers as surface-impedance copper (sigma 5.8e7 S/m), a via (0.3 mm drill as the 1.694 r
  square barrel, 0.5 mm pads, 0.8 mm antipads), 10-cell CPML, two lumped ports, 256 DFT
  frequencies 0.1-20 GHz.
* :func:`large_board` — 1600 x 1200 x 160 cells of 20 um (307 M cells): an eight-layer stack of
  single-pole Debye dielectrics (eps_inf 3.4-4.2 per layer, seeded), 12 routed traces and 40 vias
  of surface-impedance copper at seeded positions, a PEC ground under the stack, 12-cell CPML,
  eight lumped ports (trace ends to the ground) driven as a batch of eight, 512 DFT frequencies
  0.05-40 GHz.
* :func:`sweep_instances` — a seeded parameter sweep of microstrip and stripline instances with
  uneven grids (80-240 x 40-120 x 30-80 cells of 50 um), trace width 0.1-0.6 mm, substrate
  0.1-0.4 mm, single-pole Debye substrate (eps_inf 3.0-4.8, delta_eps 0.1-0.5, tau 2-20 ps),
  8-cell CPML, two lumped ports, 128 DFT frequencies.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.grid import Grid, uniform_lines
from open_analysis_gb300.model import Conductor, LumpedPort, Model, Region, Waveform
from open_analysis_gb300.pml import CpmlSpec

FloatArray = npt.NDArray[np.float64]


@dataclass(frozen=True)
class GaussDerivative:
    """First derivative of a Gaussian, normalised to a unit peak: no DC content, spectrum
    proportional to ``f exp(-(pi f tau)^2)``. ``tau = sqrt(ln 10) / (pi bandwidth)`` as for the
    reference's Gaussian, so the envelope factor is -20 dB at ``bandwidth``. Same interface as
    :class:`~open_analysis_gb300.model.Waveform` (``kind``, ``tau``, ``delay_tau``, call).
    """

    bandwidth: float
    delay_tau: float = 5.0
    kind: str = "gauss_deriv"
    f0: float = 0.0

    @property
    def tau(self) -> float:
        return math.sqrt(math.log(10.0)) / (math.pi * self.bandwidth)

    def __call__(self, t: FloatArray) -> FloatArray:
        tau = self.tau
        x = (t - self.delay_tau * tau) / tau
        return -math.sqrt(2.0 * math.e) * x * np.exp(-(x**2))  # type: ignore[no-any-return]


def microstrip(nx: int = 120, ny: int = 60, nz: int = 40, h: float = 50e-6, batch_both: bool = True) -> Model:
    """The plain 50-ohm microstrip workload (defaults: 120 x 60 x 40 cells of 50 um)."""
    g = Grid(uniform_lines(nx, h), uniform_lines(ny, h), uniform_lines(nz, h))
    freqs = np.linspace(20e9 / 64, 20e9, 64)
    m = Model(
        g,
        GaussDerivative(bandwidth=20e9),  # type: ignore[arg-type]
        freqs,
        walls=("cpml", "cpml", "cpml", "cpml", "pec", "cpml"),
        cpml=CpmlSpec(cells=8, m=3.0, kappa_max=5.0),
        courant=0.99,
    )
    sub = 0.2e-3
    m.regions.append(Region((-1.0, -1.0, 0.0), (1.0, 1.0, sub), 4.3))
    yc = (ny // 2) * h
    x0, x1 = 14 * h, (nx - 14) * h
    m.regions.append(Region((x0, yc - 0.18e-3, sub), (x1, yc + 0.18e-3, sub), pec=True))
    m.ports.append(LumpedPort("p1", 2, (x0, yc, 0.0), (x0, yc, sub), 50.0))
    m.ports.append(LumpedPort("p2", 2, (x1, yc, 0.0), (x1, yc, sub), 50.0))
    if not batch_both:
        m.excite = ("p1",)
    return m


def via_transition(
    nx: int = 400,
    ny: int = 400,
    nz: int = 120,
    h: float = 25e-6,
    n_freq: int = 256,
    cpml_cells: int = 10,
    drill: float = 0.3e-3,
    pad: float = 0.5e-3,
    antipad: float = 0.8e-3,
    eps_inf: float = 4.0,
    delta_eps: float = 0.35,
    tau: float = 8e-12,
) -> Model:
    """Top trace -> via -> bottom trace through three planes (four dielectric layers).

    Layer positions scale with ``nz``: the stack spans z cells ``[0.13 nz, 0.87 nz]``; the planes
    sit at the quarter points of the stack. Lateral features are given in metres and snapped by
    the compiler to the mesh.
    """
    g = Grid(uniform_lines(nx, h), uniform_lines(ny, h), uniform_lines(nz, h))
    freqs = np.linspace(0.1e9, 20e9, n_freq)
    m = Model(
        g,
        Waveform("gauss_mod", 10.05e9, 19.9e9),
        freqs,
        walls=("cpml",) * 6,
        cpml=CpmlSpec(cells=cpml_cells),
        courant=0.95,
    )
    kb = int(round(0.13 * nz))  # bottom trace layer (one cell of copper)
    kt = int(round(0.87 * nz))  # top trace layer
    span = kt - (kb + 1)
    planes = [kb + 1 + (span * q) // 4 for q in (1, 2, 3)]
    z = lambda k: k * h  # noqa: E731
    big = 1.0
    m.regions.append(Region((-big, -big, z(kb)), (big, big, z(kt + 1)), eps_inf, poles=((delta_eps, tau),)))
    cx, cy = (nx // 2) * h, (ny // 2) * h
    half_ap = 0.5 * antipad
    cu = dict(sigma=5.8e7, thickness=35e-6)
    for k in planes:
        lo_z, hi_z = z(k), z(k + 1)
        for lo, hi in (
            ((-big, -big, lo_z), (cx - half_ap, big, hi_z)),
            ((cx + half_ap, -big, lo_z), (big, big, hi_z)),
            ((cx - half_ap, -big, lo_z), (cx + half_ap, cy - half_ap, hi_z)),
            ((cx - half_ap, cy + half_ap, lo_z), (cx + half_ap, big, hi_z)),
        ):
            m.conductors.append(Conductor(lo, hi, **cu))
    side = 0.5 * drill / 0.5902  # square barrel with the conformal radius of the drill
    m.conductors.append(Conductor((cx - side / 2, cy - side / 2, z(kb)), (cx + side / 2, cy + side / 2, z(kt + 1)), **cu))
    for k in (kb, kt):
        m.conductors.append(Conductor((cx - pad / 2, cy - pad / 2, z(k)), (cx + pad / 2, cy + pad / 2, z(k + 1)), **cu))
    w = 0.4e-3
    x_p1, x_p2 = round(0.1 * nx) * h, round(0.9 * nx) * h
    m.conductors.append(Conductor((x_p1, cy - w / 2, z(kt)), (cx, cy + w / 2, z(kt + 1)), **cu))
    m.conductors.append(Conductor((cx, cy - w / 2, z(kb)), (x_p2, cy + w / 2, z(kb + 1)), **cu))
    # ports: top trace to the plane below it; bottom trace to the plane above it
    m.ports.append(LumpedPort("p1", 2, (x_p1, cy, z(planes[2] + 1)), (x_p1, cy, z(kt)), 50.0))
    m.ports.append(LumpedPort("p2", 2, (x_p2, cy, z(kb + 1)), (x_p2, cy, z(planes[0])), 50.0))
    return m


def large_board(nx: int = 1600, ny: int = 1200, nz: int = 160, h: float = 20e-6, seed: int = 2026,
                n_freq: int = 512, cpml_cells: int = 12) -> Model:
    """The large board region (defaults: 1600 x 1200 x 160 cells of 20 um). Eight dielectric
    layers of ``(nz - 2 (cpml + 4)) / 8`` cells fill the middle of the z extent over a PEC ground;
    traces run on the layer interfaces as two axis-aligned segments (an L) of 5 cells width, one
    cell thick; vias are square barrels of 0.2-0.3 mm spanning two to five layers; the first eight
    traces carry a lumped port (50 ohm) from their start down to the ground."""
    rng = np.random.default_rng(seed)
    g = Grid(uniform_lines(nx, h), uniform_lines(ny, h), uniform_lines(nz, h))
    m = Model(
        g,
        Waveform("gauss_mod", 20.025e9, 39.95e9),
        np.linspace(0.05e9, 40e9, n_freq),
        walls=("cpml",) * 6,
        cpml=CpmlSpec(cells=cpml_cells),
        courant=0.95,
    )
    k0 = cpml_cells + 4
    layer = (nz - 2 * k0) // 8
    at = lambda k: k * h  # noqa: E731  (cell index -> coordinate, every axis)
    big = 1.0
    for n in range(8):
        eps = float(rng.uniform(3.4, 4.2))
        m.regions.append(Region((-big, -big, at(k0 + n * layer)), (big, big, at(k0 + (n + 1) * layer)), eps,
                                poles=((0.3, 8e-12),)))
    m.regions.append(Region((-big, -big, at(k0)), (big, big, at(k0)), pec=True))  # ground under the stack
    cu = dict(sigma=5.8e7, thickness=18e-6)
    margin = cpml_cells + 20
    w = 5 * h
    for t in range(12):
        kz = k0 + layer * int(rng.integers(1, 8))  # on a layer interface
        xa, xb = sorted(int(v) for v in rng.integers(margin, nx - margin, 2))
        ya, yb = sorted(int(v) for v in rng.integers(margin, ny - margin, 2))
        # an L: along x at ya from xa to xb, then along y at xb from ya to yb
        m.conductors.append(Conductor((at(xa), at(ya), at(kz)), (at(xb), at(ya) + w, at(kz + 1)), **cu))
        m.conductors.append(Conductor((at(xb) - w, at(ya), at(kz)), (at(xb), at(yb), at(kz + 1)), **cu))
        if t < 8:
            m.ports.append(LumpedPort(f"p{t + 1}", 2, (at(xa), at(ya) + 2 * h, at(k0)), (at(xa), at(ya) + 2 * h, at(kz)), 50.0))
    for _ in range(40):
        side = float(rng.uniform(0.2e-3, 0.3e-3)) * 0.5 / 0.5902
        cx, cy = (int(v) * h for v in (rng.integers(margin, nx - margin), rng.integers(margin, ny - margin)))
        a = int(rng.integers(0, 6))
        b = min(8, a + int(rng.integers(2, 6)))
        m.conductors.append(Conductor((cx - side / 2, cy - side / 2, at(k0 + a * layer)),
                                      (cx + side / 2, cy + side / 2, at(k0 + b * layer)), **cu))
    return m


@dataclass(frozen=True)
class LineParams:
    """One sweep instance: grid cells, trace width and substrate height [m], the Debye substrate
    and whether a second ground plane makes it a stripline."""

    nx: int
    ny: int
    nz: int
    width: float
    height: float
    eps_inf: float
    delta_eps: float
    tau: float
    stripline: bool


def sweep_params(n: int, seed: int = 2026) -> list[LineParams]:
    """``n`` instances drawn uniformly from the sweep ranges (seeded); even instances are
    microstrips, odd ones striplines."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append(
            LineParams(
                nx=int(rng.integers(80, 241)),
                ny=int(rng.integers(40, 121)),
                nz=int(rng.integers(30, 81)),
                width=float(rng.uniform(0.1e-3, 0.6e-3)),
                height=float(rng.uniform(0.1e-3, 0.4e-3)),
                eps_inf=float(rng.uniform(3.0, 4.8)),
                delta_eps=float(rng.uniform(0.1, 0.5)),
                tau=float(rng.uniform(2e-12, 20e-12)),
                stripline=bool(i % 2),
            )
        )
    return out


def line_instance(p: LineParams, h: float = 50e-6, n_freq: int = 128) -> Model:
    """A microstrip (or stripline: a second PEC plane at twice the substrate height, the
    dielectric filling both sides) on a PEC ground with a Debye substrate, 8-cell CPML on the
    other walls, lumped ports at the two trace ends, DFT at ``n_freq`` frequencies 0.1-20 GHz."""
    g = Grid(uniform_lines(p.nx, h), uniform_lines(p.ny, h), uniform_lines(p.nz, h))
    m = Model(
        g,
        Waveform("gauss_mod", 10e9, 20e9),
        np.linspace(0.1e9, 20e9, n_freq),
        walls=("cpml", "cpml", "cpml", "cpml", "pec", "cpml"),
        cpml=CpmlSpec(cells=8, m=3.0, kappa_max=5.0),
    )
    sub = max(2, round(p.height / h)) * h  # the substrate on whole cells
    fill = 2 * sub if p.stripline else sub
    m.regions.append(Region((-1.0, -1.0, 0.0), (1.0, 1.0, fill), p.eps_inf, poles=((p.delta_eps, p.tau),)))
    if p.stripline:
        m.regions.append(Region((-1.0, -1.0, fill), (1.0, 1.0, fill), pec=True))
    yc = (p.ny // 2) * h
    x0, x1 = 12 * h, (p.nx - 12) * h
    half = max(h, round(p.width / (2 * h)) * h)
    m.regions.append(Region((x0, yc - half, sub), (x1, yc + half, sub), pec=True))
    m.ports.append(LumpedPort("p1", 2, (x0, yc, 0.0), (x0, yc, sub), 50.0))
    m.ports.append(LumpedPort("p2", 2, (x1, yc, 0.0), (x1, yc, sub), 50.0))
    return m


def sweep_instances(n: int = 64, seed: int = 2026, h: float = 50e-6, n_freq: int = 128) -> list[Model]:
    """The sweep's models (see :func:`sweep_params`)."""
    return [line_instance(p, h, n_freq) for p in sweep_params(n, seed)]


WORKLOADS = {
    "microstrip_120x60x40": microstrip,
    "via_transition_400x400x120": via_transition,
}
