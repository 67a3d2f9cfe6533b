"""The model compiler and the oracle against fixtures generated by the reference itself."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
from cases import CASES, namespace
from fingerprint import compare_compiled, compiled_fingerprint, load, state_fingerprint

from open_analysis_gb300.model import compile_model
from oracle.numpy_engine import OracleEngine

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("native", [True, False], ids=["native", "numpy"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_compiler_matches_reference_arrays(case: str, native: bool) -> None:
    """Both compilers (the native volume stages and the NumPy ones) reproduce the reference's
    compiled arrays bit for bit; mode ports compile on the NumPy stages only."""
    from open_analysis_gb300.model import _native_library

    if native and (case == "mode_stripline" or _native_library() is None):
        pytest.skip("mode ports use the NumPy stages" if case == "mode_stripline" else "library not built")
    ref = load(str(GOLDEN / f"{case}.npz"))
    builder, _ = CASES[case]
    c = compile_model(builder(namespace("gb300")), "float32", native=native)
    mine = compiled_fingerprint(c)
    ref_c = {k: v for k, v in ref.items() if not k.startswith(("float32.", "float64.", "full.", "steps", "wave."))}
    assert compare_compiled(ref_c, mine) == []


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_oracle_matches_reference_engine(case: str, dtype: str) -> None:
    """float32 fields bit for bit; DFTs and energy to rounding of the float64 accumulators."""
    ref = load(str(GOLDEN / f"{case}.npz"))
    builder, steps = CASES[case]
    c = compile_model(builder(namespace("gb300")), "float32")
    eng = OracleEngine(c, dtype)
    eng.step(steps)
    got = state_fingerprint(eng)
    for comp in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        assert got[f"field.{comp}.sha"] == ref[f"{dtype}.field.{comp}.sha"], comp
    for k, v in ref.items():
        if k.startswith(f"{dtype}.dft."):
            w = got[k[len(dtype) + 1 :]]
            assert np.abs(w - v).max() <= 1e-13 * np.abs(v).max(), k
    e_ref = float(ref[f"{dtype}.energy"])
    assert abs(float(got["energy"]) - e_ref) <= 1e-12 * abs(e_ref)


def test_full_fields_fixture_consistent() -> None:
    ref = load(str(GOLDEN / "mixed_walls.npz"))
    from fingerprint import digest

    for comp in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
        assert digest(ref[f"full.{comp}"]) == ref[f"float32.field.{comp}.sha"]


@pytest.mark.parametrize("native", [True, False], ids=["native", "numpy"])
@pytest.mark.parametrize("name", ["microstrip_120x60x40", "via_transition_400x400x120", "large_board_200x150x80"])
def test_compiler_matches_reference_on_the_workloads(name: str, native: bool) -> None:
    """The benchmark workloads (the configured microstrip, the full-size via transition, the
    large-board structure on a reduced grid) compile to the reference's arrays bit for bit."""
    from workloads import workloads

    from open_analysis_gb300.model import _native_library

    if native and _native_library() is None:
        pytest.skip("library not built")
    ref = load(str(GOLDEN / f"workload_{name}.npz"))
    c = compile_model(workloads()[name]["model"](), "float32", native=native)
    skip = ("float32.", "float64.", "rel64.", "sample.", "steps", "seed")
    ref_c = {k: v for k, v in ref.items() if not k.startswith(skip)}
    assert compare_compiled(ref_c, compiled_fingerprint(c)) == []
