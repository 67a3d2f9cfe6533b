"""Dispersive dielectrics as multi-pole Debye models (model inputs for ``Region.poles``).

Restates ``packages/oa-fdtd/src/oa_fdtd/materials/debye.py`` (the reference's fit, its ADR-0010
section 5): the Djordjevic-Sarkar wideband permittivity (Djordjevic et al., IEEE Trans. EMC
43(4), 2001) and a non-negative least-squares fit of ``eps_inf + sum_k d_k / (1 + j w tau_k)`` on
a fixed log-spaced pole set, so every fit is causal and passive. Convention ``exp(+j w t)``:
``eps = eps' - j eps''``. The pole count grows until the permittivity error is below 0.2 % and
the loss-tangent error below 2 % over the band (the reference's limits), else the best fit up to
12 poles is returned. The pole placement, the weighting of the two error kinds and the stopping
rule follow the reference (``debye.py:77-128``), so the same material gives the same poles and
the engine sees the same coefficients.
"""

from __future__ import annotations

import math
from collections.abc import Callable
from dataclasses import dataclass

import numpy as np
import numpy.typing as npt
from scipy.optimize import nnls

FloatArray = npt.NDArray[np.float64]
ComplexArray = npt.NDArray[np.complex128]
TWO_PI = 2.0 * math.pi


@dataclass(frozen=True)
class DebyeFit:
    """``eps_inf`` [-], pole strengths ``delta`` [-], relaxation times ``tau`` [s], the fit band
    [Hz] and the worst relative errors of eps' and tan(delta) over it."""

    eps_inf: float
    delta: FloatArray
    tau: FloatArray
    f_lo: float
    f_hi: float
    err_eps: float
    err_tand: float

    @property
    def poles(self) -> tuple[tuple[float, float], ...]:
        """``(delta, tau)`` pairs for ``Region(poles=...)``."""
        return tuple((float(d), float(t)) for d, t in zip(self.delta, self.tau, strict=True))

    def eval(self, freqs: FloatArray) -> ComplexArray:
        """The fitted complex relative permittivity at ``freqs`` [Hz]."""
        w = TWO_PI * np.asarray(freqs, dtype=np.float64)
        out = np.full(w.shape, self.eps_inf, dtype=np.complex128)
        for d, t in zip(self.delta, self.tau, strict=True):
            out = out + d / (1.0 + 1j * w * t)
        return out


def djordjevic_sarkar_eps(
    freqs: FloatArray, dk: float, df: float, f_ref: float, f_low: float, f_high: float
) -> ComplexArray:
    """Djordjevic-Sarkar permittivity with dielectric constant ``dk`` and loss tangent ``df`` at
    ``f_ref`` [Hz]; the relaxation spectrum spans ``[f_low, f_high]`` [Hz]."""
    a1, a2, wr = TWO_PI * f_low, TWO_PI * f_high, TWO_PI * f_ref
    # the loss term at f_ref fixes the spectrum's strength c; eps_inf then fixes dk at f_ref
    c = dk * df / (math.atan(wr / a1) - math.atan(wr / a2))
    eps_inf = dk - c * 0.5 * math.log((a2**2 + wr**2) / (a1**2 + wr**2))
    w = TWO_PI * np.asarray(freqs, dtype=np.float64)
    real = eps_inf + c * 0.5 * np.log((a2**2 + w**2) / (a1**2 + w**2))
    imag = c * (np.arctan(w / a1) - np.arctan(w / a2))
    return np.asarray(real - 1j * imag, dtype=np.complex128)


def _design(w: FloatArray, tau: FloatArray) -> tuple[FloatArray, FloatArray]:
    """eps' and eps'' design matrices for the unknowns ``[eps_inf - 1, d_1 .. d_N]``."""
    wt = w[:, None] * tau[None, :]
    relax = 1.0 / (1.0 + wt**2)
    real = np.column_stack([np.ones_like(w), relax])
    imag = np.column_stack([np.zeros_like(w), wt * relax])
    return real, imag


def fit_debye(
    freqs: FloatArray,
    eps: ComplexArray,
    f_lo: float,
    f_hi: float,
    *,
    tol_eps: float = 2e-3,
    tol_tand: float = 2e-2,
    max_poles: int = 12,
    min_poles: int = 3,
    margin_decades: float = 1.0,
) -> DebyeFit:
    """The fewest log-spaced Debye poles (band widened by ``margin_decades`` each side) whose NNLS
    fit of ``eps`` meets both tolerances over ``[f_lo, f_hi]``; else the best of them."""
    f = np.asarray(freqs, dtype=np.float64)
    eps = np.asarray(eps, dtype=np.complex128)
    band = (f >= f_lo * (1 - 1e-9)) & (f <= f_hi * (1 + 1e-9))
    f, eps = f[band], eps[band]
    if f.size < 4 or not 0 < f_lo < f_hi:
        raise ValueError("fit needs 0 < f_lo < f_hi and at least four samples in the band")
    w = TWO_PI * f
    tand = -eps.imag / eps.real
    # both residuals in units of eps'; a tol_tand error of tan(delta) weighs like tol_eps of eps'
    w_real = 1.0 / eps.real
    w_imag = (tol_eps / tol_tand) / eps.real
    best: DebyeFit | None = None
    score = math.inf
    for n in range(min_poles, max_poles + 1):
        tau = 1.0 / (TWO_PI * np.geomspace(f_lo * 10**-margin_decades, f_hi * 10**margin_decades, n))
        real, imag = _design(w, tau)
        a = np.vstack([real * w_real[:, None], imag * w_imag[:, None]])
        rhs = np.concatenate([(eps.real - 1.0) * w_real, -eps.imag * w_imag])
        x, _ = nnls(a, rhs, maxiter=50 * a.shape[1])
        trial = DebyeFit(1.0 + float(x[0]), x[1:].copy(), tau, f_lo, f_hi, 0.0, 0.0)
        ev = trial.eval(f)
        err_eps = float(np.max(np.abs(ev.real - eps.real) / eps.real))
        err_tand = float(np.max(np.abs(-ev.imag / ev.real - tand) / np.maximum(tand, 1e-12)))
        trial = DebyeFit(trial.eps_inf, trial.delta, tau, f_lo, f_hi, err_eps, err_tand)
        s = err_eps / tol_eps + err_tand / tol_tand
        if best is None or s < score:
            best, score = trial, s
        if err_eps <= tol_eps and err_tand <= tol_tand:
            return trial
    assert best is not None
    return best


def fit_djordjevic_sarkar(
    dk: float,
    df: float,
    f_ref: float,
    f_lo: float,
    f_hi: float,
    f_low: float = 1e4 / TWO_PI,
    f_high: float = 1e12 / TWO_PI,
    n_samples: int = 400,
) -> DebyeFit:
    """Debye fit of a Djordjevic-Sarkar dielectric sampled log-uniformly over ``[f_lo, f_hi]``."""
    f = np.geomspace(f_lo, f_hi, n_samples)
    return fit_debye(f, djordjevic_sarkar_eps(f, dk, df, f_ref, f_low, f_high), f_lo, f_hi)


def fit_callable(
    fn: Callable[[FloatArray], ComplexArray], f_lo: float, f_hi: float, n_samples: int = 400
) -> DebyeFit:
    """Debye fit of any ``eps(f)`` callable (a table interpolant, say) over the band."""
    f = np.geomspace(f_lo, f_hi, n_samples)
    return fit_debye(f, fn(f), f_lo, f_hi)
