"""The matrix-pencil tail (``open_analysis_gb300/tail.py``) against the reference's own fits.

``tests/golden/tail_fits.npz`` holds the reference's ``fit_tail`` and ``extrapolate_dft`` results
on three synthetic probe series made by ``tests/golden/make_golden.py`` (``tail_series``): two
decaying modes; the same with a growing out-of-band term, which the fit must drop; and a tail
below numerical noise, which has no fit.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

from make_golden import tail_series  # noqa: E402

from open_analysis_gb300.tail import extrapolate_dft, fit_tail  # noqa: E402


def _sorted(s: np.ndarray, c: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    order = np.lexsort((s.real, s.imag))
    return s[order], c[order]


def test_tail_fits_match_the_reference() -> None:
    ref = np.load(GOLDEN / "tail_fits.npz")
    freqs = np.linspace(1e9, 20e9, 12)
    for name, y, dt, t0, fb in tail_series(np):
        fit = fit_tail(y, dt, t0, f_band=fb)
        assert (fit is None) == bool(ref[f"{name}.none"]), name
        if fit is None:
            continue
        t_ref, n_dropped, residual = ref[f"{name}.meta"]
        assert fit.t_ref == t_ref and fit.n_dropped == int(n_dropped), name
        assert abs(fit.residual - residual) <= 1e-9 + 1e-6 * abs(residual), name
        s, c = _sorted(fit.s, fit.c)
        rs, rc = _sorted(ref[f"{name}.s"], ref[f"{name}.c"])
        np.testing.assert_allclose(s, rs, rtol=1e-8, err_msg=name)
        np.testing.assert_allclose(c, rc, rtol=1e-7, atol=1e-12, err_msg=name)
        dft = extrapolate_dft(fit, dt, t0 + y.size * dt, freqs)
        np.testing.assert_allclose(dft, ref[f"{name}.dft"], rtol=1e-7, atol=1e-12 * np.abs(ref[f"{name}.dft"]).max())
