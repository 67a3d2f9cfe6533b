"""Excitation batching: all ports as one batch, or a subset plus reciprocity, as the reference's
``packages/oa-fdtd/tests/test_batching.py:17-40`` checks it, on the oracle (CPU) and on the GPU
engine (``-m gpu``); an unknown excited port is ``FDTD_BAD_DRIVE``."""

from __future__ import annotations

import numpy as np
import pytest
from known_answers import plate_line

from open_analysis_gb300.model import ModelError
from open_analysis_gb300.run import run, sparams
from oracle.numpy_engine import OracleEngine

FREQS = np.linspace(1e9, 8e9, 4)


def _line(excite: tuple[str, ...] | None = None):  # type: ignore[no-untyped-def]
    m = plate_line(0.006, 0.25e-3, FREQS, 10e9)
    m.excite = excite
    return m


def _check_subset(engine: object) -> None:
    full = _line()
    res_full = run(full, engine=engine, dtype="float64", end_db=-60.0)
    s_full = sparams(full, res_full)
    assert res_full.probes["V:p1"].shape[0] == 2  # two excitations in one batch
    half = _line(("p1",))
    res_half = run(half, engine=engine, dtype="float64", end_db=-60.0)
    assert res_half.probes["V:p1"].shape[0] == 1  # one excitation
    s_half = sparams(half, res_half)
    assert np.all(np.isnan(s_half[:, 1]))  # the undriven column
    s_rec = sparams(half, res_half, reciprocal=True)
    assert np.isnan(s_rec[1, 1]).all()  # S22 needs port 2 driven
    known = ~np.isnan(s_rec)
    assert known[0, 1].all()  # S12 filled from S21
    assert np.abs(s_rec[known] - s_full[known]).max() < 1e-9
    assert np.abs(s_half[:, 0] - s_full[:, 0]).max() < 1e-12


def test_subset_excitation_matches_full_batch_on_the_oracle() -> None:
    _check_subset(OracleEngine)


@pytest.mark.gpu
def test_subset_excitation_matches_full_batch_on_the_gpu() -> None:
    _check_subset("gb300")


def test_unknown_excited_port_is_an_error() -> None:
    with pytest.raises(ModelError) as exc:
        run(_line(("nope",)), engine=OracleEngine, end_db=-40.0)
    assert exc.value.code == "FDTD_BAD_DRIVE"
