"""Surface-impedance boundary: finite-slab impedance, its passive ladder fit, and the face-edge
classification of copper boxes.

Mirrors ``packages/oa-fdtd/src/oa_fdtd/subcell/sibc.py`` (``slab_surface_impedance :29-40``,
``hammerstad_jensen :43-49``, ``SibcFit :52-74``, ``fit_surface_impedance :77-115``) and
``packages/oa-fdtd/src/oa_fdtd/subcell/edges.py`` (``classify_box :37-75``,
``outside_samples :83-112``). Setup-time only; its tables feed the engine's SIBC edge pass.

Model: ``Zs(w) = k / sigma * coth(k t)``, ``k = sqrt(j w mu sigma)``, times a roughness factor,
fitted by ``R0 + sum_p R_p j w tau_p / (1 + j w tau_p)`` with ``R_p >= 0`` (non-negative least
squares over a fixed log-spaced pole set, so every section is passive). Each section is
discretised bilinearly: ``v_p <- R_p c_p (J - J_prev) + g_p v_p`` with ``x = 2 tau / dt``,
``c_p = x / (1 + x)``, ``g_p = (x - 1) / (x + 1)``.

Face convention (shared with the E update): edge ``E_c`` at storage index ``p`` is circulated by
``H_b`` at ``p`` and ``p - s_a`` and by ``H_a`` at ``p`` and ``p - s_b`` with ``(c, a, b)``
cyclic; with the outward normal ``n`` the condition ``E_t = Zs n x H_t`` gives
``+a: E_c = +Zs H_b[p]``, ``-a: E_c = -Zs H_b[p - s_a]``, ``+b: E_c = -Zs H_a[p]``,
``-b: E_c = +Zs H_a[p - s_b]``; an edge on two faces averages the two samples.
"""

from __future__ import annotations

import math
from collections.abc import Callable
from dataclasses import dataclass

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.grid import Grid

FloatArray = npt.NDArray[np.float64]
ComplexArray = npt.NDArray[np.complex128]
IntArray = npt.NDArray[np.intp]
MU0 = 4e-7 * math.pi
TWO_PI = 2.0 * math.pi


def slab_surface_impedance(
    freqs: FloatArray, sigma: float, thickness: float, mu_r: float = 1.0
) -> ComplexArray:
    """``Zs`` [ohm/sq] of a slab of ``thickness`` with its far side shorted."""
    w = TWO_PI * np.maximum(np.asarray(freqs, dtype=np.float64), 1e-30)
    k = np.sqrt(1j * w * MU0 * mu_r * sigma)
    return np.asarray(k / sigma / np.tanh(k * thickness), dtype=np.complex128)


def hammerstad_jensen(freqs: FloatArray, sigma: float, rms: float, mu_r: float = 1.0) -> FloatArray:
    """Roughness factor ``1 + (2/pi) atan(1.4 (rms / delta)^2)``."""
    f = np.asarray(freqs, dtype=np.float64)
    if rms <= 0:
        return np.ones_like(f)
    w = TWO_PI * np.maximum(f, 1e-30)
    skin = np.sqrt(2.0 / (w * MU0 * mu_r * sigma))
    return np.asarray(1.0 + (2.0 / math.pi) * np.arctan(1.4 * (rms / skin) ** 2))


@dataclass(frozen=True)
class SibcFit:
    """Series resistance ``r0``, section resistances ``rp`` and time constants ``tau``."""

    r0: float
    rp: FloatArray
    tau: FloatArray
    f_lo: float
    f_hi: float
    err: float

    def eval(self, freqs: FloatArray) -> ComplexArray:
        w = TWO_PI * np.asarray(freqs, dtype=np.float64)
        z = np.full(w.shape, self.r0, dtype=np.complex128)
        for r, t in zip(self.rp, self.tau, strict=True):
            z = z + r * (1j * w * t) / (1.0 + 1j * w * t)
        return z

    def recursion(self, dt: float) -> tuple[FloatArray, FloatArray]:
        """Bilinear section coefficients ``(c_p, g_p)``."""
        x = 2.0 * self.tau / dt
        return x / (1.0 + x), (x - 1.0) / (x + 1.0)


def fit_surface_impedance(
    sigma: float,
    thickness: float,
    f_lo: float,
    f_hi: float,
    *,
    rms: float = 0.0,
    roughness: Callable[[FloatArray], FloatArray] | None = None,
    n_poles: int = 16,
    mu_r: float = 1.0,
) -> SibcFit:
    """Passive ladder fit of ``Zs(f) K(f)`` over ``[f_lo, f_hi]`` with ``n_poles`` sections.

    Samples: 240 log-spaced points from ``f_lo / 5`` to ``f_hi`` plus two pins at ``1e-3 f_lo``
    and ``1e-2 f_lo`` (the DC end); poles log-spaced from ``0.1 f_lo`` to ``5 f_hi``. Residuals
    are weighted by ``1 / |Z|``; the reactance rows carry a 0.2 weight so the loss leads.
    """
    from scipy.optimize import nnls

    if not 0 < f_lo < f_hi:
        raise ValueError("fit band needs 0 < f_lo < f_hi")
    f = np.concatenate([[f_lo * 1e-3, f_lo * 1e-2], np.geomspace(f_lo / 5.0, f_hi, 240)])
    factor = roughness(f) if roughness is not None else hammerstad_jensen(f, sigma, rms, mu_r)
    z = slab_surface_impedance(f, sigma, thickness, mu_r) * factor
    w = TWO_PI * f
    tau = 1.0 / (TWO_PI * np.geomspace(f_lo * 0.1, f_hi * 5.0, n_poles))
    wt = w[:, None] * tau[None, :]
    lor = 1.0 / (1.0 + wt**2)
    a_re = np.column_stack([np.ones_like(w), wt**2 * lor])
    a_im = np.column_stack([np.zeros_like(w), wt * lor])
    weight = 1.0 / np.abs(z)
    a = np.vstack([a_re * weight[:, None], 0.2 * a_im * weight[:, None]])
    rhs = np.concatenate([z.real * weight, 0.2 * z.imag * weight])
    x, _ = nnls(a, rhs, maxiter=100 * a.shape[1])
    fit = SibcFit(float(x[0]), x[1:].copy(), tau, f_lo, f_hi, 0.0)
    band = (f >= f_lo * (1 - 1e-9)) & (f <= f_hi * (1 + 1e-9))
    err = float(np.max(np.abs(fit.eval(f[band]).real - z[band].real) / z[band].real))
    return SibcFit(fit.r0, fit.rp, fit.tau, f_lo, f_hi, err)


# ---------------------------------------------------------------- copper box edge classes
@dataclass
class BoxEdges:
    """E edges of one copper box on the ``(nz + 1, ny + 1, nx + 1)`` edge lattice, per
    component: PEC interior, face (surface) edges, and the face flags (+1/-1/0) of the two
    transverse axes ``a = c + 1`` and ``b = c + 2`` (mod 3) of every face edge."""

    interior: list[tuple[IntArray, IntArray, IntArray]]
    surface: list[tuple[IntArray, IntArray, IntArray]]
    face_a: list[npt.NDArray[np.int8]]
    face_b: list[npt.NDArray[np.int8]]


def classify_box(grid: Grid, lo: tuple[float, ...], hi: tuple[float, ...]) -> BoxEdges:
    """Split the E edges inside the closed box into PEC interior and face edges."""
    empty = (np.zeros(0, np.intp), np.zeros(0, np.intp), np.zeros(0, np.intp))
    out = BoxEdges([], [], [], [])
    for c in range(3):
        a, b = (c + 1) % 3, (c + 2) % 3
        sel: list[IntArray] = []
        flags: list[npt.NDArray[np.int8]] = []
        for ax in range(3):
            node = ax != c
            pos = grid.coords(ax, node)
            tol = 1e-6 * float(np.min(grid.d(ax)))
            ids = np.flatnonzero((pos >= lo[ax] - tol) & (pos <= hi[ax] + tol))
            flag = np.zeros(ids.size, dtype=np.int8)
            if node:
                flag[np.abs(pos[ids] - hi[ax]) <= tol] = 1
                flag[np.abs(pos[ids] - lo[ax]) <= tol] = -1
            sel.append(ids)
            flags.append(flag)
        if min(s.size for s in sel) == 0:
            out.interior.append(empty)
            out.surface.append(empty)
            out.face_a.append(np.zeros(0, np.int8))
            out.face_b.append(np.zeros(0, np.int8))
            continue
        shape = (sel[2].size, sel[1].size, sel[0].size)
        kk = np.broadcast_to(sel[2][:, None, None], shape).ravel()
        jj = np.broadcast_to(sel[1][None, :, None], shape).ravel()
        ii = np.broadcast_to(sel[0][None, None, :], shape).ravel()
        flag_of = [
            np.broadcast_to(flags[0][None, None, :], shape).ravel(),
            np.broadcast_to(flags[1][None, :, None], shape).ravel(),
            np.broadcast_to(flags[2][:, None, None], shape).ravel(),
        ]
        fa, fb = flag_of[a], flag_of[b]
        on_face = (fa != 0) | (fb != 0)
        out.interior.append((kk[~on_face], jj[~on_face], ii[~on_face]))
        out.surface.append((kk[on_face], jj[on_face], ii[on_face]))
        out.face_a.append(fa[on_face].copy())
        out.face_b.append(fb[on_face].copy())
    return out


def outside_samples(
    grid: Grid,
    c: int,
    k: IntArray,
    j: IntArray,
    i: IntArray,
    fa: npt.NDArray[np.int8],
    fb: npt.NDArray[np.int8],
) -> tuple[npt.NDArray[np.int64], npt.NDArray[np.int32], npt.NDArray[np.int64], FloatArray]:
    """Flat edge index, and per edge two outside H samples: component, flat index and weight
    (sign / number of faces; 0 = unused). Slot 0 is the ``a`` face (``H_b``), slot 1 the ``b``
    face (``H_a``)."""
    a, b = (c + 1) % 3, (c + 2) % 3
    stride = (1, grid.shape[2], grid.shape[2] * grid.shape[1])
    p = ((k + 1) * stride[2] + (j + 1) * stride[1] + (i + 1)).astype(np.int64)
    n_faces = np.maximum((fa != 0).astype(np.float64) + (fb != 0).astype(np.float64), 1.0)
    hcomp = np.empty((p.size, 2), np.int32)
    hflat = np.empty((p.size, 2), np.int64)
    hsign = np.empty((p.size, 2), np.float64)
    hcomp[:, 0], hcomp[:, 1] = b, a
    hflat[:, 0] = np.where(fa > 0, p, p - stride[a])
    hflat[:, 1] = np.where(fb > 0, p, p - stride[b])
    hsign[:, 0] = np.where(fa != 0, np.where(fa > 0, 1.0, -1.0) / n_faces, 0.0)
    hsign[:, 1] = np.where(fb != 0, np.where(fb > 0, -1.0, 1.0) / n_faces, 0.0)
    return p, hcomp, hflat, hsign
