"""Surrogate host logic and its CPU oracle (no GPU).

The network oracle (``oracle/mlp_oracle.py``) is pinned here by central finite differences of its
FP64 loss; the GPU kernels are checked against it in ``tests/test_surrogate_gpu.py``.
"""

from __future__ import annotations

import numpy as np
import pytest

from open_analysis_gb300.model import compile_model
from open_analysis_gb300.surrogate import (
    PARAM_RANGES,
    TOL_DB,
    TOL_LIN,
    ViaGrid,
    db_error,
    meshed,
    rows_to_s,
    s_to_rows,
    line_factor,
    scale_params,
    via_instance,
    via_params,
)
from oracle.mlp_oracle import AdamState, adam, bf16_round, forward, loss_and_grads

SMALL = ViaGrid(nx=64, ny=64, nz=60, h=50e-6, dz=100e-6, n_freq=32, cpml=6)


def _net(sizes: list[int], seed: int = 0) -> tuple[list[np.ndarray], list[np.ndarray]]:
    rng = np.random.default_rng(seed)
    w = [rng.standard_normal((a, b)) * np.sqrt(2.0 / a) for a, b in zip(sizes[:-1], sizes[1:], strict=True)]
    b = [rng.standard_normal(n) * 0.1 for n in sizes[1:]]
    return w, b


@pytest.mark.parametrize("act", ["relu", "tanh"])
def test_oracle_gradients_match_finite_differences(act: str) -> None:
    sizes = [7, 16, 16, 12]
    w, b = _net(sizes)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (9, 7))
    t = rng.standard_normal((9, 12))
    g = loss_and_grads(w, b, x, t, bf16=False, act=act)
    h = 1e-6
    for l in range(len(w)):
        for arr, grad in ((w[l], g.dw[l]), (b[l], g.db[l])):
            flat, gflat = arr.reshape(-1), grad.reshape(-1)
            for i in rng.choice(flat.size, size=min(6, flat.size), replace=False):
                keep = flat[i]
                flat[i] = keep + h
                up = loss_and_grads(w, b, x, t, bf16=False, act=act).loss
                flat[i] = keep - h
                dn = loss_and_grads(w, b, x, t, bf16=False, act=act).loss
                flat[i] = keep
                fd = (up - dn) / (2 * h)
                assert abs(fd - gflat[i]) <= 1e-7 + 1e-6 * abs(fd), (l, i, fd, gflat[i])


def test_bf16_rounding_is_nearest_even() -> None:
    one = 1.0
    ulp = 2.0**-7  # BF16 spacing at 1
    vals = np.array([one, one + ulp / 2, one + 1.5 * ulp, one + ulp / 2 + 2**-20, -3.0, 0.0, 2.0**-130])
    got = bf16_round(vals)
    assert got[0] == one
    assert got[1] == one  # tie -> even
    assert got[2] == one + 2 * ulp  # tie -> even (odd ulp rounds up)
    assert got[3] == one + ulp  # above the tie
    assert got[4] == -3.0 and got[5] == 0.0
    assert np.all(bf16_round(got) == got)


def test_bf16_forward_stays_close_to_fp64() -> None:
    w, b = _net([7, 64, 64, 8], seed=3)
    x = np.random.default_rng(4).uniform(-1, 1, (32, 7))
    y16, _ = forward(w, b, x, bf16=True)
    y64, _ = forward(w, b, x, bf16=False)
    rel = np.linalg.norm(y16 - y64) / np.linalg.norm(y64)
    assert 1e-5 < rel < 2e-2  # BF16 rounding is visible and small


def test_adam_oracle_first_step_moves_by_lr() -> None:
    p = [np.array([1.0, -2.0, 0.5])]
    g = [np.array([0.3, -0.1, 0.0])]
    st = AdamState([np.zeros(3)], [np.zeros(3)])
    adam(p, g, st, lr=0.01)
    # after one step m1/c1 = g and sqrt(m2/c2) = |g|: every weight with a gradient moves by lr
    np.testing.assert_allclose(p[0], [0.99, -1.99, 0.5], rtol=0, atol=1e-9)


def test_meshed_parameters_are_idempotent_and_in_range() -> None:
    p = via_params(200, seed=7)
    lo, hi = PARAM_RANGES[:, 0], PARAM_RANGES[:, 1]
    assert np.all(p >= lo) and np.all(p <= hi)
    q = meshed(p)
    np.testing.assert_array_equal(meshed(q), q)
    np.testing.assert_array_equal(q[:, 4:6], p[:, 4:6])
    g = ViaGrid()
    assert np.allclose(np.round(q[:, 1] / (2 * g.h)) * 2 * g.h, q[:, 1])
    assert np.allclose(np.round(q[:, 3] / g.dz) * g.dz, q[:, 3])
    s = scale_params(q)
    assert np.all(np.abs(s) <= 1.0 + 0.2)


def test_rows_round_trip_and_error_measure() -> None:
    rng = np.random.default_rng(0)
    s = rng.standard_normal((3, 2, 5)) + 1j * rng.standard_normal((3, 2, 5))
    np.testing.assert_array_equal(rows_to_s(s_to_rows(s)), s)
    assert abs(TOL_LIN - 5.7731e-3) < 1e-6
    assert abs(db_error(np.array([TOL_LIN]), np.array([0.0])) - TOL_DB) < 1e-12
    e = db_error(s, s + 1e-3, axis=(1, 2))
    assert e.shape == (3,) and np.allclose(e, 20 * np.log10(1.001))


def test_via_instance_compiles_with_every_part() -> None:
    p = via_params(2, seed=11)
    for q in p:
        c = compile_model(via_instance(q, SMALL), "float32")
        assert c.grid.shape == (SMALL.nz + 2, SMALL.ny + 2, 96)
        assert c.ade is not None and c.sibc is not None and c.sibc.flat.size > 1000
        assert c.batch == 1 and len(c.ports) == 2
    with pytest.raises(ValueError):
        via_instance(p[0], ViaGrid(nz=60))  # the tallest stack and stub do not fit


def test_line_factor_removes_the_tem_line() -> None:
    g = ViaGrid()
    p = meshed(via_params(5, seed=3), g)
    f = line_factor(p, g)
    assert f.shape == (5, 2, g.n_freq)
    assert np.all(np.abs(f) >= 1.0)  # exp(+alpha L): dividing it out can only shrink errors
    lossless = p.copy()
    lossless[:, 5] = 0.0  # no Debye term: a pure phase
    assert np.allclose(np.abs(line_factor(lossless, g)), 1.0, rtol=0, atol=1e-12)
    # the S21 factor's phase is the TEM delay over both traces and the via
    w = 2 * np.pi * np.linspace(0.1e9, 20e9, g.n_freq)
    length = (g.nx // 2 - g.cpml - 4) * g.h + (g.nx - g.cpml - 4 - g.nx // 2) * g.h + lossless[:, 3:4]
    want = w * np.sqrt(lossless[:, 4:5]) / 299792458.0 * length
    assert np.allclose(np.unwrap(np.angle(line_factor(lossless, g)[:, 1]), axis=1), want, atol=1e-9)
