"""CFS-CPML coefficients and the per-term correction boxes.

Mirrors ``packages/oa-fdtd/src/oa_fdtd/pml.py`` (``CpmlSpec :45-52``, ``Correction :56-70``,
``_profile :90-100``, ``build_pml :103-146``). The method is Roden and Gedney's convolutional PML
with complex-frequency-shifted stretching (Microwave Opt. Technol. Lett. 27(5), 2000): inside a
slab the derivative ``d`` along the slab axis becomes ``d / kappa + psi`` with
``psi <- b psi + c d``. The correction of one curl term is therefore
``F_c += sign * k * ((1/kappa - 1) d + psi)``, ``k = cb`` for E and ``dt / mu0`` for H, added
after the bulk update. The GB300 engine fuses it into its sweeps in exactly that order.

The tables below are the curl sign convention shared with the reference (``pml.py:26-41``); they
must stay identical because the compiled correction list is part of the engine input.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.grid import EPS0, ETA0, MU0, Grid

FloatArray = npt.NDArray[np.float64]
Box = tuple[tuple[int, int], tuple[int, int], tuple[int, int]]  # storage [lo, hi) per x, y, z

# (corrected component c, derivative axis a, source component b, sign):
#   E_c += sign * cb * d_a H_b        H_c += sign * (dt / mu0) * d_a E_b
E_TERMS = (
    (0, 1, 2, 1.0),
    (0, 2, 1, -1.0),
    (1, 2, 0, 1.0),
    (1, 0, 2, -1.0),
    (2, 0, 1, 1.0),
    (2, 1, 0, -1.0),
)
H_TERMS = tuple((c, a, b, -s) for c, a, b, s in E_TERMS)


@dataclass(frozen=True)
class CpmlSpec:
    """Layer parameters: thickness in cells, grading order, kappa_max, design reflection
    ``r0`` (sets sigma_max) and ``f_low`` (alpha_max = 2 pi f_low eps0)."""

    cells: int = 10
    m: float = 3.0
    kappa_max: float = 8.0
    r0: float = 1e-8
    f_low: float = 1e8


@dataclass(frozen=True)
class Correction:
    """One curl-term correction ``F_c += sign * k * (ek * d + psi)`` over ``box``."""

    kind: str  # "E" or "H"
    c: int
    a: int
    b: int
    sign: float
    box: Box

    @property
    def shape(self) -> tuple[int, int, int]:
        """psi shape ``(nz, ny, nx)`` of one batch member."""
        return (
            self.box[2][1] - self.box[2][0],
            self.box[1][1] - self.box[1][0],
            self.box[0][1] - self.box[0][0],
        )


@dataclass(frozen=True)
class AxisCoeffs:
    """1-D float64 coefficients over the storage index of one axis: ``eb, ec, ek`` on the node
    lattice (E terms), ``hb, hc, hk`` on the cell lattice (H terms); ``ek = 1/kappa - 1``."""

    eb: FloatArray
    ec: FloatArray
    ek: FloatArray
    hb: FloatArray
    hc: FloatArray
    hk: FloatArray


@dataclass(frozen=True)
class Pml:
    corrections: tuple[Correction, ...]
    coeffs: dict[int, AxisCoeffs]


def grading(
    depth: FloatArray, thick: float, spec: CpmlSpec, dt: float
) -> tuple[FloatArray, FloatArray, FloatArray]:
    """``(b, c, 1/kappa - 1)`` of the polynomially graded CFS profile at ``depth`` into the layer.

    sigma = sigma_max rho^m with sigma_max = -(m + 1) ln(r0) / (2 eta0 thick);
    kappa = 1 + (kappa_max - 1) rho^m; alpha = alpha_max (1 - rho) inside the layer;
    b = exp(-(sigma / kappa + alpha) dt / eps0); c = sigma (b - 1) / (kappa (sigma + kappa alpha)).
    """
    rho = np.clip(depth / thick, 0.0, 1.0)
    sigma_max = -(spec.m + 1.0) * math.log(spec.r0) / (2.0 * ETA0 * thick)
    sigma = sigma_max * rho**spec.m
    kappa = 1.0 + (spec.kappa_max - 1.0) * rho**spec.m
    alpha = 2.0 * math.pi * spec.f_low * EPS0 * (1.0 - rho) * (rho > 0)
    b = np.exp(-(sigma / kappa + alpha) * dt / EPS0)
    den = kappa * (sigma + kappa * alpha)
    positive = den > 0
    c = np.where(positive, sigma * (b - 1.0) / np.where(positive, den, 1.0), 0.0)
    b = np.where(rho > 0, b, 0.0)
    return b, c, 1.0 / kappa - 1.0


def _slab(grid: Grid, axis: int, side: int, cells: int) -> tuple[float, float, Box, Box]:
    """Inner-face coordinate, thickness and the E/H storage ranges of one CPML slab."""
    n = grid.n[axis]
    lines = grid.lines[axis]
    if side == 0:
        inner = float(lines[cells])
        thick = abs(inner - float(lines[0]))
        return inner, thick, (1, cells + 1), (1, cells + 1)  # type: ignore[return-value]
    inner = float(lines[n - cells])
    thick = abs(inner - float(lines[n]))
    return inner, thick, (n - cells + 2, n + 2), (n - cells + 1, n + 1)  # type: ignore[return-value]


def build_pml(grid: Grid, walls: tuple[str, ...], spec: CpmlSpec, dt: float) -> Pml:
    """Coefficient arrays and correction boxes for every wall flagged ``"cpml"``.

    Corrections are listed per axis (x, y, z), per side (low, high), E terms before H terms, each
    in term-table order; the engine applies them in this order.
    """
    corrections: list[Correction] = []
    coeffs: dict[int, AxisCoeffs] = {}
    for axis in range(3):
        sides = [s for s in (0, 1) if walls[2 * axis + s] == "cpml"]
        if not sides:
            continue
        n = grid.n[axis]
        if 2 * spec.cells >= n:
            raise ValueError(
                f"axis {'xyz'[axis]}: {n} cells cannot hold two {spec.cells}-cell CPML layers"
            )
        size = grid.length(axis)
        node_pos = np.full(size, np.nan)
        cell_pos = np.full(size, np.nan)
        node_pos[1 : n + 2] = grid.lines[axis]
        cell_pos[1 : n + 1] = grid.centers(axis)
        arr = {key: np.zeros(size) for key in ("eb", "ec", "ek", "hb", "hc", "hk")}
        for side in sides:
            inner, thick, e_rng, h_rng = _slab(grid, axis, side, spec.cells)
            if side == 0:
                depth_e, depth_h = inner - node_pos, inner - cell_pos
            else:
                depth_e, depth_h = node_pos - inner, cell_pos - inner
            for prefix, depth, rng in (("e", depth_e, e_rng), ("h", depth_h, h_rng)):
                b, c, k = grading(np.nan_to_num(depth, nan=0.0), thick, spec, dt)
                lo, hi = rng
                arr[prefix + "b"][lo:hi] = b[lo:hi]
                arr[prefix + "c"][lo:hi] = c[lo:hi]
                arr[prefix + "k"][lo:hi] = k[lo:hi]
            for kind, terms, rng in (("E", E_TERMS, e_rng), ("H", H_TERMS, h_rng)):
                for c_, a_, b_, sign in terms:
                    if a_ != axis:
                        continue
                    box = list(grid.valid(kind, c_))
                    box[axis] = rng
                    corrections.append(Correction(kind, c_, a_, b_, sign, tuple(box)))  # type: ignore[arg-type]
        coeffs[axis] = AxisCoeffs(**arr)
    return Pml(tuple(corrections), coeffs)


def mu_dt(dt: float) -> float:
    """``dt / mu0``."""
    return dt / MU0
