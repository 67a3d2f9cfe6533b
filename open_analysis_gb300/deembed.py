"""Wave-plane S-parameter extraction and reference-plane shifts for mode ports.

Restates the reference's de-embedding (``packages/oa-fdtd/src/oa_fdtd/ports/deembed.py``:
``gamma_from_planes :23-53``, ``smooth_gamma :56-84``, ``shift_reference :101-116``,
``uniform_length :138-178``, ``add_wave_planes :181-262``, ``wave_sparams :265-338``) in code of
its own. Host-side post-processing of the probe DFTs the engine returns; nothing here runs on
the GPU.

* Three modal voltage planes on a uniform line give the propagation constant without any
  assumption on the termination: ``V(z) = A e^{-g z} + B e^{g z}`` makes
  ``cosh(g d) = (V1 + V3) / (2 V2)`` for equal spacings (Newton iterations from there for unequal
  ones), branch ``Re g >= 0``, phase unwrapped along frequency.
* The forward and backward waves at the reference plane follow, and ``S = B A^-1`` over all the
  excitations (the ports' own terminations drop out); where the planes are too close in phase
  the ill-conditioned low band falls back to a smooth fit of gamma and, for the reflections, to the
  port S-parameters.
"""

from __future__ import annotations

from collections.abc import Callable, Sequence
from dataclasses import dataclass, replace
from typing import Any

import numpy as np
import numpy.typing as npt

FloatArray = npt.NDArray[np.float64]
ComplexArray = npt.NDArray[np.complex128]

DeembedHook = Callable[[ComplexArray, FloatArray], ComplexArray]


def _residual(g: ComplexArray, v1: ComplexArray, v2: ComplexArray, v3: ComplexArray, da: float, db: float) -> ComplexArray:
    """Zero where ``g`` fits three planes at distances ``da`` (1 to 2) and ``db`` (2 to 3)."""
    return np.asarray((v1 - v2 * np.cosh(g * da)) * np.sinh(g * db) + (v3 - v2 * np.cosh(g * db)) * np.sinh(g * da),
                      dtype=np.complex128)


def _newton(g: ComplexArray, v1: ComplexArray, v2: ComplexArray, v3: ComplexArray, da: float, db: float) -> ComplexArray:
    step = 1e-6 * np.maximum(np.abs(g), 1.0)
    r0 = _residual(g, v1, v2, v3, da, db)
    slope = (_residual(g + step, v1, v2, v3, da, db) - r0) / step
    ok = np.abs(slope) > 0
    return np.asarray(np.where(ok, g - r0 / np.where(ok, slope, 1.0), g), dtype=np.complex128)


def gamma_from_planes(v1: ComplexArray, v2: ComplexArray, v3: ComplexArray, spacing: float,
                      spacing_b: float | None = None) -> ComplexArray:
    """Propagation constant [1/m] from the modal voltages of three planes (``v2`` the middle one;
    ``spacing`` from plane 1 to 2, ``spacing_b`` from 2 to 3, default equal)."""
    db = spacing if spacing_b is None else spacing_b
    mean = 0.5 * (spacing + db)
    g = np.arccosh(((v1 + v3) / (2.0 * v2)).astype(np.complex128)) / mean
    g = np.asarray(np.where(g.real < 0, -g, g), dtype=np.complex128)
    if abs(db - spacing) > 1e-9 * spacing:
        for _ in range(8):
            g = _newton(g, v1, v2, v3, spacing, db)
    g = np.asarray(np.where(g.real < 0, -g, g), dtype=np.complex128)
    g = np.where(g.imag < 0, np.conj(g), g)
    beta = np.unwrap(g.imag * mean) / mean
    return np.asarray(g.real + 1j * beta, dtype=np.complex128)


def smooth_gamma(gamma: ComplexArray, freqs: FloatArray, spacing: float, min_phase: float,
                 fit_mask: npt.NDArray[np.bool_] | None = None) -> ComplexArray:
    """Below the band where the phase between planes reaches ``min_phase`` [rad], gamma from a
    least-squares fit of the conditioned points: ``alpha = a1 sqrt(f) + a2 f + a3 f^2`` (conductor
    and dielectric loss), ``beta = b1 f + b2 f^2 + b3 f^3`` (weak dispersion)."""
    good = np.abs(gamma.imag) * spacing >= min_phase
    use = good if fit_mask is None else good & fit_mask
    if use.sum() < 6 or good.all():
        return gamma
    fn = np.asarray(freqs, dtype=np.float64) / float(np.max(freqs))
    a_basis = np.column_stack([np.sqrt(fn), fn, fn**2])
    b_basis = np.column_stack([fn, fn**2, fn**3])
    ca = np.linalg.lstsq(a_basis[use], gamma.real[use], rcond=None)[0]
    cb = np.linalg.lstsq(b_basis[use], gamma.imag[use], rcond=None)[0]
    return np.asarray(np.where(good, gamma, a_basis @ ca + 1j * (b_basis @ cb)), dtype=np.complex128)


def shift_reference(s: ComplexArray, gamma: Sequence[ComplexArray] | ComplexArray, lengths: Sequence[float]) -> ComplexArray:
    """Move port ``i``'s reference plane inwards by ``lengths[i]`` [m]:
    ``S'_ij = S_ij e^{g_i L_i} e^{g_j L_j}`` (one gamma for all ports or one per port)."""
    n = s.shape[0]
    gam = [np.asarray(gamma)] * n if np.ndim(gamma[0]) == 0 else [np.asarray(x) for x in gamma]
    fac = [np.exp(gam[i] * lengths[i]) for i in range(n)]
    out = np.empty_like(s)
    for i in range(n):
        for j in range(n):
            out[i, j] = s[i, j] * fac[i] * fac[j]
    return out


def apply_hook(s: ComplexArray, freqs: FloatArray, hook: DeembedHook) -> ComplexArray:
    """A fixture de-embedder (for example a 2x-thru) on ``S[i, j, f]``."""
    return hook(s, freqs)


@dataclass(frozen=True)
class PlaneSet:
    """Three modal probe planes of one port, outer to inner: probe names, spacing [m] (and the
    inner spacing when unequal), and the signed distance [m] from the middle plane to the
    reference plane (positive inwards)."""

    port: str
    probes: tuple[str, str, str]
    spacing: float
    ref: float
    spacing_b: float | None = None


def uniform_length(model: Any, port: Any) -> float:
    """Length [m] of the uniform line behind a mode port: from the port plane to the first cell
    layer whose cross-section (regions and copper boxes cutting the port rectangle, with their
    in-plane extents) differs from the layer at the port."""
    n = port.axis
    ua, va = (a for a in range(3) if a != n)
    lo_r = {ua: port.lo[0], va: port.lo[1]}
    hi_r = {ua: port.hi[0], va: port.hi[1]}
    boxes = [(c.lo, c.hi, f"cu:{c.model}") for c in model.conductors]
    boxes += [(r.lo, r.hi, repr((r.eps_r, r.sigma, r.pec, r.poles))) for r in model.regions]

    def section(mid: float) -> tuple[Any, ...]:
        out = []
        for lo, hi, kind in boxes:
            if not lo[n] <= mid <= hi[n]:
                continue
            ext: list[float] = []
            for a in (ua, va):
                a0, a1 = max(lo[a], lo_r[a]), min(hi[a], hi_r[a])
                if a1 < a0:
                    break
                ext += [round(a0, 12), round(a1, 12)]
            else:
                out.append((kind, *ext))
        return tuple(sorted(out))

    lines = model.grid.lines[n]
    i = int(np.argmin(np.abs(lines - port.position)))
    step = port.direction
    first = None
    while 0 <= i + step < lines.size:
        here = section(0.5 * float(lines[i] + lines[i + step]))
        if first is None:
            first = here
        elif here != first:
            break
        i += step
    return abs(float(lines[i]) - port.position)


def add_wave_planes(model: Any, port: str, offset: float, spacing_cells: int = 16, max_phase: float = 2.2,
                    min_phase: float = 0.6, ref_position: float | None = None) -> PlaneSet:
    """Add three modal probe planes in the uniform line behind mode port ``port`` and describe them.

    The planes lie at least ``offset`` [m] from the port and from the end of the uniform line,
    within the half of the domain next to the port; the widest equal spacing of at most
    ``spacing_cells`` cells whose phase at the top frequency (largest permittivity) stays below
    ``max_phase`` [rad]. ``FDTD_UNEQUAL_PLANES`` when there is none or its phase is below
    ``min_phase``. ``ref_position`` [m] places the reference plane (default: the port plane)."""
    from open_analysis_gb300.model import ModelError, ModePort

    mp = next((p for p in model.ports if isinstance(p, ModePort) and p.name == port), None)
    if mp is None:
        raise ModelError("FDTD_BAD_PORT", f"no mode port named {port!r}")
    lines = model.grid.lines[mp.axis]
    i_port = int(np.argmin(np.abs(lines - mp.position)))
    step = mp.direction
    eps_max = max([1.0] + [r.eps_r + sum(d for d, _ in r.poles) for r in model.regions if not r.pec])
    f_top = float(np.max(model.frequencies))
    beta_top = 2.0 * np.pi * f_top * float(np.sqrt(eps_max)) / 299792458.0
    d_target = max_phase / beta_top
    uniform = uniform_length(model, mp)
    depth = min(0.45 * float(lines[-1] - lines[0]), uniform - offset)
    found = None
    for k in range(spacing_cells, 0, -1):
        for i_mid in range(i_port + step * 2, i_port + step * lines.size, step):
            if not 0 <= i_mid < lines.size:
                break
            idx = [i_mid - step * k, i_mid, i_mid + step * k]
            if min(idx) < 0 or max(idx) >= lines.size:
                continue
            if (float(lines[idx[0]]) - mp.position) * step < offset:
                continue
            if abs(float(lines[idx[2]]) - mp.position) > depth:
                break
            d1 = abs(float(lines[idx[1]] - lines[idx[0]]))
            d2 = abs(float(lines[idx[2]] - lines[idx[1]]))
            if d1 > d_target:
                break
            if abs(d1 - d2) <= 0.1 * d1:
                found = (idx, d1, d2)
                break
        if found:
            break
    if found is None:
        raise ModelError(
            "FDTD_UNEQUAL_PLANES",
            f"no three equally spaced planes behind {port} at least {offset:.3e} m from it and from the end "
            f"of its {uniform:.3e} m uniform line",
            "Lengthen the uniform line behind the port or use a uniform stretch of the mesh.",
        )
    idx, d1, d2 = found
    if beta_top * d1 < min_phase:
        raise ModelError(
            "FDTD_UNEQUAL_PLANES",
            f"the {uniform:.3e} m uniform line behind {port} holds planes only {d1:.3e} m apart "
            f"({beta_top * d1:.2f} rad at {f_top:.3e} Hz, below {min_phase} rad)",
            "Lengthen the uniform line behind the port; the port S is used meanwhile.",
        )
    pos = [float(lines[i]) for i in idx]
    names = tuple(f"W:{port}:{k}" for k in range(3))
    for nm, x in zip(names, pos, strict=True):
        model.mode_probes.append(replace(mp, name=nm, position=x))
    ref_x = float(lines[i_port]) if ref_position is None else float(ref_position)
    return PlaneSet(port, tuple(f"V:{nm}" for nm in names), d1, (ref_x - pos[1]) * step, d2)  # type: ignore[arg-type]


def wave_sparams(probes: dict[str, ComplexArray], planes: Sequence[PlaneSet], port_r: FloatArray,
                 s_port: ComplexArray | None = None, min_phase: float = 0.3, freqs: FloatArray | None = None,
                 floor_phase: float = 0.04, fit_mask: npt.NDArray[np.bool_] | None = None) -> tuple[ComplexArray, list[ComplexArray]]:
    """``(S[i, j, f], [gamma_i])`` from the modal waves on each port's three planes.

    Excitation ``j`` is batch member ``j``. Power waves at the reference plane, ``a = A / sqrt(R)``
    and ``b = B / sqrt(R)``, give ``S = B A^-1`` over the excitations (driven-wave normalisation
    ``b / a_jj`` where ``A`` is ill-conditioned). With ``freqs``, gamma is smoothed below
    ``min_phase`` (:func:`smooth_gamma`) and the reflections below ``floor_phase``, like any
    frequency where the plane S is not passive (max |S| > 1.02), come from ``s_port``; without
    ``freqs``, ``s_port`` replaces S wherever the phase is below ``min_phase``."""
    n = len(planes)
    nf = probes[planes[0].probes[0]].shape[1]
    s = np.zeros((n, n, nf), np.complex128)
    a = np.zeros((n, n, nf), np.complex128)
    b = np.zeros((n, n, nf), np.complex128)
    gammas: list[ComplexArray] = []
    for i, pl in enumerate(planes):
        db = pl.spacing if pl.spacing_b is None else pl.spacing_b
        for j in range(n):
            v1, v2, v3 = (probes[nm][j] for nm in pl.probes)
            g = gamma_from_planes(v1, v2, v3, pl.spacing, db)
            if freqs is not None:
                g = smooth_gamma(g, freqs, pl.spacing, min_phase, fit_mask)
            if j == 0:
                gammas.append(g)
            diff = (v1 - v2 * np.cosh(g * pl.spacing)) / np.sinh(g * pl.spacing)  # A - B at the middle plane
            a[i, j] = 0.5 * (v2 + diff) * np.exp(-g * pl.ref) / np.sqrt(port_r[i])
            b[i, j] = 0.5 * (v2 - diff) * np.exp(g * pl.ref) / np.sqrt(port_r[i])
    for k in range(nf):
        am, bm = a[:, :, k], b[:, :, k]
        diag = np.abs(np.diag(am))
        off = np.abs(am - np.diag(np.diag(am))).max() if n > 1 else 0.0
        if n == 1 or off > 0.3 * diag.min() or not np.all(np.isfinite(am)):
            s[:, :, k] = bm / np.diag(am)[None, :]
        else:
            s[:, :, k] = np.linalg.solve(am.T, bm.T).T
    if s_port is not None:
        thr = min_phase if freqs is None else floor_phase
        weak = np.zeros(nf, dtype=bool)
        for pl, g in zip(planes, gammas, strict=True):
            weak |= np.abs(g.imag) * pl.spacing < thr
        if freqs is None:
            s[:, :, weak] = s_port[:, :, weak]
        else:
            for i in range(n):
                s[i, i, weak] = s_port[i, i, weak]
            noisy = np.abs(s).max(axis=(0, 1)) > 1.02
            s[:, :, noisy] = s_port[:, :, noisy]
    return s, gammas
