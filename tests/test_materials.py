"""The multi-pole Debye fit against fixtures made by the reference's own fit
(``tests/golden/make_golden.py``, ``debye_fits.npz``): the same poles bit for bit."""

from __future__ import annotations

from pathlib import Path

import numpy as np

from open_analysis_gb300.materials import djordjevic_sarkar_eps, fit_djordjevic_sarkar

GOLDEN = Path(__file__).resolve().parent / "golden" / "debye_fits.npz"


def test_debye_fits_match_the_reference() -> None:
    data = np.load(GOLDEN)
    n = len({k.split(".")[0] for k in data.files})
    assert n >= 3
    for i in range(n):
        dk, df, fr, lo, hi = data[f"{i}.case"]
        fit = fit_djordjevic_sarkar(dk, df, fr, lo, hi)
        assert fit.eps_inf == float(data[f"{i}.eps_inf"][0])
        assert np.array_equal(fit.delta, data[f"{i}.delta"])
        assert np.array_equal(fit.tau, data[f"{i}.tau"])
        assert np.array_equal(np.array([fit.err_eps, fit.err_tand]), data[f"{i}.err"])


def test_djordjevic_sarkar_matches_its_reference_values() -> None:
    """dk and df at f_ref by construction; passive (eps'' > 0) across the band."""
    f = np.geomspace(1e8, 1e11, 50)
    eps = djordjevic_sarkar_eps(np.array([1e9]), 4.3, 0.02, 1e9, 1e4 / (2 * np.pi), 1e12 / (2 * np.pi))
    assert abs(eps.real[0] - 4.3) < 1e-12
    assert abs(-eps.imag[0] / eps.real[0] - 0.02) < 1e-12
    assert (djordjevic_sarkar_eps(f, 4.3, 0.02, 1e9, 1e3, 1e12).imag < 0).all()
