"""Yee lattice geometry and the storage layout the engine shares with its callers.

Mirrors ``packages/oa-fdtd/src/oa_fdtd/grid.py`` (the ``Grid`` type, ``grid.py:29-152``) so a
problem built for the reference engine builds here unchanged.

Storage layout (unchanged from the reference, because ``get_fields`` returns it and every flat
index in a compiled problem points into it): one array per field component, shape
``(B, nz + 2, ny + 2, pitch)``, C order, x fastest. ``pitch`` is ``nx + 2`` rounded up to 32
elements, so every x row starts on a 128-byte boundary for float32. Storage index ``I = i + 1``
along each axis; ``I = 0`` and ``I = n + 1`` are ghost planes (PMC mirrors). ``E_a`` is
cell-type along ``a`` and node-type along the other two axes; ``H_a`` is the dual.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import numpy.typing as npt

C0 = 299792458.0  # speed of light [m/s]
MU0 = 4e-7 * np.pi  # [H/m]
EPS0 = 1.0 / (MU0 * C0**2)  # [F/m]
ETA0 = MU0 * C0  # [ohm]
ROW_ALIGN = 32  # x-row padding [elements]

FloatArray = npt.NDArray[np.float64]
IntArray = npt.NDArray[np.intp]


def _padded(n: int) -> int:
    return ((n + ROW_ALIGN - 1) // ROW_ALIGN) * ROW_ALIGN


@dataclass(frozen=True)
class Grid:
    """Mesh lines ``x, y, z`` [m]: 1-D, strictly increasing, two or more lines each."""

    x: FloatArray
    y: FloatArray
    z: FloatArray

    def __post_init__(self) -> None:
        for axis_name in ("x", "y", "z"):
            lines = np.asarray(getattr(self, axis_name), dtype=np.float64)
            ok = lines.ndim == 1 and lines.size >= 2 and bool(np.all(np.diff(lines) > 0))
            if not ok:
                raise ValueError(
                    f"grid lines {axis_name} must be 1-D, increasing, with >= 2 entries"
                )
            object.__setattr__(self, axis_name, lines)

    # ---- sizes
    @property
    def lines(self) -> tuple[FloatArray, FloatArray, FloatArray]:
        return (self.x, self.y, self.z)

    @property
    def n(self) -> tuple[int, int, int]:
        """Cells per axis ``(nx, ny, nz)``."""
        return (self.x.size - 1, self.y.size - 1, self.z.size - 1)

    @property
    def cells(self) -> int:
        nx, ny, nz = self.n
        return nx * ny * nz

    @property
    def pitch(self) -> int:
        """Padded x extent of one storage row [elements]."""
        return _padded(self.n[0] + 2)

    @property
    def shape(self) -> tuple[int, int, int]:
        """Storage shape ``(nz + 2, ny + 2, pitch)`` of one component of one batch member."""
        return (self.n[2] + 2, self.n[1] + 2, self.pitch)

    def length(self, axis: int) -> int:
        """Storage extent along ``axis`` (0 = x, 1 = y, 2 = z)."""
        return self.pitch if axis == 0 else self.n[axis] + 2

    # ---- 1-D metrics, indexed by storage index
    def d(self, axis: int) -> FloatArray:
        """Primal cell lengths [m]."""
        return np.diff(self.lines[axis])

    def centers(self, axis: int) -> FloatArray:
        v = self.lines[axis]
        return 0.5 * (v[1:] + v[:-1])

    def coords(self, axis: int, node: bool) -> FloatArray:
        """Positions of the node-type (mesh lines) or cell-type (centres) lattice [m]."""
        return self.lines[axis] if node else self.centers(axis)

    def _on_storage(self, axis: int, values: FloatArray, start: int) -> FloatArray:
        out = np.zeros(self.length(axis))
        out[start : start + values.size] = values
        return out

    def inv_primal(self, axis: int) -> FloatArray:
        """``1 / d_i`` at storage index ``i + 1``; zero on ghosts and padding [1/m]."""
        return self._on_storage(axis, 1.0 / self.d(axis), 1)

    def inv_dual(self, axis: int) -> FloatArray:
        """``1 / ((d_{i-1} + d_i) / 2)`` at node storage index ``i + 1`` [1/m].

        A wall node mirrors its one neighbouring cell, so its dual length is that cell's length.
        """
        d = self.d(axis)
        mirrored = np.concatenate([d[:1], d, d[-1:]])
        return self._on_storage(axis, 2.0 / (mirrored[:-1] + mirrored[1:]), 1)

    def node_weights(self, axis: int) -> FloatArray:
        """Dual-cell length of each node, halved at the two walls [m]."""
        d = self.d(axis)
        padded = np.concatenate([[0.0], d, [0.0]])
        return self._on_storage(axis, 0.5 * (padded[:-1] + padded[1:]), 1)

    def cell_weights(self, axis: int) -> FloatArray:
        """Primal cell lengths on storage indices ``1 .. n`` [m]."""
        return self._on_storage(axis, self.d(axis), 1)

    def dt(self, courant: float = 0.95, c_max: float = C0) -> float:
        """Courant-limited time step of the non-uniform grid [s]."""
        inv_sq = sum(1.0 / float(np.min(self.d(a))) ** 2 for a in range(3))
        return float(courant / (c_max * inv_sq**0.5))

    # ---- lattice queries
    def is_node(self, kind: str, comp: int, axis: int) -> bool:
        """Whether component ``kind``/``comp`` sits on mesh lines (nodes) along ``axis``."""
        return (axis != comp) if kind == "E" else (axis == comp)

    def valid(self, kind: str, comp: int) -> tuple[tuple[int, int], ...]:
        """Per-axis storage ranges ``[lo, hi)`` (x, y, z) that hold real lattice points."""
        return tuple(
            (1, self.n[a] + 2) if self.is_node(kind, comp, a) else (1, self.n[a] + 1)
            for a in range(3)
        )

    def points(
        self, kind: str, comp: int, lo: tuple[float, float, float], hi: tuple[float, float, float]
    ) -> tuple[IntArray, tuple[int, int, int]]:
        """Flat storage indices of the points of one component inside the closed box.

        Ordered z, then y, then x. Returns ``(flat, (count_x, count_y, count_z))``. A degenerate
        (point-like) box along an axis snaps to the nearest point; a box that misses every point
        of an axis raises ``ValueError``.
        """
        picks: list[IntArray] = []
        for a in range(3):
            pos = self.coords(a, self.is_node(kind, comp, a))
            tol = 1e-6 * float(np.min(self.d(a)))
            inside = np.flatnonzero((pos >= lo[a] - tol) & (pos <= hi[a] + tol))
            if inside.size == 0 and hi[a] - lo[a] <= 2.0 * tol:
                inside = np.array([int(np.argmin(np.abs(pos - 0.5 * (lo[a] + hi[a]))))])
            if inside.size == 0:
                raise ValueError(f"box selects no {kind}{'xyz'[comp]} point along {'xyz'[a]}")
            picks.append((inside + 1).astype(np.intp))
        sz, sy = self.shape[1] * self.shape[2], self.shape[2]
        flat = (
            picks[2][:, None, None] * sz + picks[1][None, :, None] * sy + picks[0][None, None, :]
        ).ravel()
        return flat.astype(np.intp), (picks[0].size, picks[1].size, picks[2].size)


def uniform_lines(n: int, h: float, origin: float = 0.0) -> FloatArray:
    """``n + 1`` equally spaced mesh lines ``origin + i h``."""
    return origin + np.arange(n + 1, dtype=np.float64) * h


def courant_dt(grid: Grid, courant: float, eps_min: float = 1.0) -> float:
    """Time step used by the model compiler: the Courant limit at the fastest wave speed."""
    return grid.dt(courant, C0 / math.sqrt(eps_min))
