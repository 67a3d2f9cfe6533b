"""Matrix-pencil tail extrapolation of truncated probe DFTs, and the matrix-pencil mode finder.

Mirrors ``packages/oa-fdtd/src/oa_fdtd/tail.py`` (``fit_tail :39-86``, ``extrapolate_dft :89-98``),
``packages/oa-fdtd/src/oa_fdtd/run.py:163-200`` (``_extend_tails``) and
``packages/oa-fdtd/src/oa_fdtd/analysis.py:14-37`` (``matrix_pencil``). Host-side post-processing
of the series the engine records on the device.

A run stopped at its step cap leaves a tail ``y_n, n >= S`` outside the running DFT. The last
``window`` samples are fitted by ``y_n = sum_m c_m z_m^n`` (matrix pencil on the decimated series,
amplitudes by least squares); the DFT of the continuation is added in closed form,
``sum_m c_m exp((s_m - j w)(t_S - t_0)) dt / (1 - exp((s_m - j w) dt))``. Non-decaying poles and
poles far above the band are dropped and counted.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np
import numpy.typing as npt

FloatArray = npt.NDArray[np.float64]
ComplexArray = npt.NDArray[np.complex128]


@dataclass(frozen=True)
class TailFit:
    s: ComplexArray  # poles [1/s]
    c: ComplexArray  # amplitudes at t_ref
    t_ref: float
    n_dropped: int
    residual: float


def _pencil_poles(seg: FloatArray, order: int | None, sv_tol: float, max_poles: int) -> ComplexArray:
    n = seg.size
    ell = n // 3
    hank = seg[np.arange(n - ell)[:, None] + np.arange(ell + 1)[None, :]]
    _, sv, vh = np.linalg.svd(hank, full_matrices=False)
    m = order if order is not None else min(max_poles, int(np.count_nonzero(sv > sv_tol * sv[0])))
    if m < 1:
        return np.zeros(0, np.complex128)
    v = vh[:m].conj().T
    return np.linalg.eigvals(np.linalg.pinv(v[:-1]) @ v[1:]).astype(np.complex128)


def fit_tail(
    y: FloatArray,
    dt: float,
    t_first: float,
    *,
    f_band: float,
    window: int = 6000,
    max_poles: int = 40,
    sv_tol: float = 1e-4,
    samples: int = 700,
) -> TailFit | None:
    """Fit the last ``window`` samples of ``y`` (sample ``n`` at ``t_first + n dt``); ``None``
    when the tail is below numerical noise or too short."""
    x = np.asarray(y, dtype=np.float64)
    w = min(window, x.size)
    seg = x[x.size - w :]
    scale = float(np.max(np.abs(x))) if x.size else 0.0
    if scale == 0.0 or float(np.max(np.abs(seg))) < 1e-9 * scale:
        return None
    d_max = max(int(1.0 / (6.0 * f_band * dt)), 1)
    d = int(np.clip(w // samples, 1, d_max))
    seg = seg[::-1][::d][::-1]  # decimate, keeping the last sample
    n = seg.size
    if n < 16:
        return None
    t0 = t_first + (x.size - 1 - d * (n - 1)) * dt
    h = d * dt
    z = _pencil_poles(seg, None, sv_tol, max_poles)
    if z.size == 0:
        return None
    s = np.log(z) / h
    keep = (s.real < -1e-3 / (n * h)) & (np.abs(s.imag) < 2.0 * np.pi * 2.0 * f_band)
    dropped = int(s.size - keep.sum())
    s = s[keep]
    if s.size == 0:
        return None
    vand = np.exp(np.outer(np.arange(n) * h, s))
    c, *_ = np.linalg.lstsq(vand, seg.astype(np.complex128), rcond=None)
    res = float(np.linalg.norm(vand @ c - seg) / max(np.linalg.norm(seg), 1e-300))
    return TailFit(s=s.astype(np.complex128), c=c.astype(np.complex128), t_ref=t0, n_dropped=dropped, residual=res)


def extrapolate_dft(fit: TailFit, dt: float, t_next: float, freqs: FloatArray) -> ComplexArray:
    """DFT ``sum_{n >= S} y_n exp(-j w t_n) dt`` of the fitted continuation; ``t_next`` is the
    stamp of the first sample not yet in the running DFT."""
    w = 2.0 * np.pi * np.asarray(freqs, dtype=np.float64)
    a = fit.s[None, :] - 1j * w[:, None]
    num = fit.c[None, :] * np.exp(a * (t_next - fit.t_ref)) * dt
    return np.asarray(np.sum(num / (1.0 - np.exp(a * dt)), axis=1), dtype=np.complex128)


def matrix_pencil(
    y: FloatArray, dt: float, order: int, decimate: int = 1, pencil: float = 0.4
) -> tuple[FloatArray, FloatArray]:
    """Non-negative frequencies [Hz] and damping rates [1/s] of ``order`` complex exponentials."""
    x = np.asarray(y[::decimate], dtype=np.float64)
    h = dt * decimate
    n = x.size
    ell = int(pencil * n)
    hank = x[np.arange(n - ell)[:, None] + np.arange(ell + 1)[None, :]]
    _, _, vh = np.linalg.svd(hank, full_matrices=False)
    v = vh[:order].conj().T
    z = np.linalg.eigvals(np.linalg.pinv(v[:-1]) @ v[1:])
    s = np.log(z.astype(np.complex128)) / h
    f = s.imag / (2.0 * np.pi)
    keep = f >= 0
    order_ix = np.argsort(f[keep])
    return f[keep][order_ix], (-s.real[keep])[order_ix]


def extend_tails(
    c: Any,
    probes: dict[str, ComplexArray],
    series: dict[str, FloatArray],
    sums: dict[str, list[str]],
    done: int,
) -> dict[str, Any]:
    """Add the continuation to every probe DFT in place. A summed probe (parts of one port) is
    fitted once and its correction added to its first part, which keeps ``sum(parts)`` right."""
    kind = {p["name"]: p["kind"] for p in c.probes}
    f_band = float(np.max(c.frequencies))
    in_sums = {q for parts in sums.values() for q in parts}
    groups: dict[str, list[str]] = {n: [n] for n in probes if n not in sums and n not in in_sums}
    groups.update({n: list(parts) for n, parts in sums.items()})
    n_fit = n_drop = 0
    worst = 0.0
    for parts in groups.values():
        if any(q not in series for q in parts):
            continue
        y = series[parts[0]].copy()
        for q in parts[1:]:
            y += series[q]
        off = 0.5 if kind.get(parts[0], "E") == "H" else 1.0
        for b in range(y.shape[0]):
            fit = fit_tail(y[b], c.dt, off * c.dt, f_band=f_band)
            if fit is None:
                continue
            probes[parts[0]][b] += extrapolate_dft(fit, c.dt, (done + off) * c.dt, c.frequencies)
            n_fit += 1
            n_drop += fit.n_dropped
            worst = max(worst, fit.residual)
    return {"applied": True, "fits": n_fit, "dropped_poles": n_drop, "worst_residual": worst}
