"""The benchmark workloads on the GPU against the reference's own NumPy engine.

The fixtures ``tests/golden/workload_<name>.npz`` come from the reference itself
(``tests/golden/make_golden.py``, part ``workloads``): its classes, its ``compile_model``, its
``NumpyEngine`` in float32 and float64, its ``run()`` and ``sparams``. The workloads
(``tests/golden/workloads.py``) are the configured microstrip at its stated size and step count,
the via transition at full size for 200 steps, and the large-board structure with its batch of
eight on a reduced grid; the last two start from seeded fields so that every CPML, Debye and
surface-impedance edge works from the first step.

Checked here, on the GPU engine in float32: every field bit for bit against the reference's
float32 engine (the parity gate of rel-L2 <= 1e-5 is then met with zero error), the probe DFTs to
1e-9 of their peak, the energy to 1e-10, the microstrip's S-parameters through ``run()`` +
``sparams()`` within 1e-3 of the reference's float64 ``run()`` (and to 1e-9 of its float32
engine). Each result's error against the FP64 oracle is computed and printed (``pytest -s``):
the fields' rel-L2 on seeded sample points, the DFTs' and S-parameters' largest deviation.
Also here: the engine's memory estimate against what it allocates on these problems.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
from fingerprint import digest, load
from workloads import NAMES, seeded_values, workloads

from open_analysis_gb300.model import compile_model

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
WORK = workloads()


def _rel(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _run(name: str):  # type: ignore[no-untyped-def]
    from open_analysis_gb300.engine import Gb300Engine

    ref = load(str(GOLDEN / f"workload_{name}.npz"))
    c = compile_model(WORK[name]["model"](), "float32")
    steps, seed = int(ref["steps"]), int(ref["seed"])
    eng = Gb300Engine(c, "float32", max_steps=steps)
    if seed >= 0:
        for k in range(6):
            eng.set_field(k, seeded_values(eng.shape, seed, k))
    eng.step(steps)
    return c, eng, ref


@pytest.mark.parametrize("name", sorted(WORK))
def test_workload_matches_the_reference_engine(name: str) -> None:
    c, eng, ref = _run(name)
    idx = ref["sample.index"]
    report = []
    for k, nm in enumerate(NAMES):
        got = eng.field(k)
        assert digest(got.astype(np.float32)) == ref[f"float32.field.{nm}.sha"], f"{nm} differs from the reference"
        sampled = _rel(got.reshape(-1)[idx], ref[f"float64.sample.{nm}"])
        full = float(ref[f"rel64.{nm}"])  # the reference's float32 against its float64, whole field
        # the same float32 field: its sampled error is the whole-field one, up to sampling
        assert sampled <= 10.0 * full + 1e-6, (nm, sampled, full)
        report.append(f"{nm} {full:.2e} (sampled {sampled:.2e})")
    res = eng.results()
    worst64 = 0.0
    for pname, v in res.items():
        want32, want64 = ref[f"float32.dft.{pname}"], ref[f"float64.dft.{pname}"]
        peak = max(np.abs(want64).max(), 1e-300)
        assert np.abs(v - want32).max() <= 1e-9 * max(np.abs(want32).max(), 1e-300), pname
        worst64 = max(worst64, float(np.abs(v - want64).max() / peak))
    e = eng.energy()
    assert abs(e - float(ref["float32.energy"])) <= 1e-10 * abs(float(ref["float32.energy"]))
    e64 = abs(e - float(ref["float64.energy"])) / abs(float(ref["float64.energy"]))
    print(f"\n{name}: {int(ref['steps'])} steps; error against the FP64 oracle: fields rel-L2 " + ", ".join(report)
          + f"; DFTs max {worst64:.2e} of peak; energy {e64:.2e}")
    eng.close()


def test_microstrip_sparams_match_the_reference_run() -> None:
    """The configured microstrip (120 x 60 x 40, 2000 steps): run() + sparams() on the GPU in
    float32 against the reference's run() in float64 (|dS| <= 1e-3) and its float32 engine."""
    from open_analysis_gb300.run import run, sparams

    name = "microstrip_120x60x40"
    ref = load(str(GOLDEN / f"workload_{name}.npz"))
    m = WORK[name]["model"]()
    res = run(m, engine="gb300", dtype="float32", end_db=None, max_steps=int(ref["steps"]))
    s = sparams(m, res)
    d64 = float(np.abs(s - ref["float64.s"]).max())
    d32 = float(np.abs(s - ref["float32.s"]).max())
    print(f"\n{name}: |S_gpu - S_ref(float64 run)| max {d64:.2e}; against the float32 reference engine {d32:.2e}")
    assert d64 <= 1e-3
    assert d32 <= 1e-9


@pytest.mark.parametrize("name", ["via_transition_400x400x120", "large_board_200x150x80"])
def test_memory_estimate_covers_the_allocations(name: str) -> None:
    from open_analysis_gb300.engine import Gb300Engine, estimate_bytes

    c = compile_model(WORK[name]["model"](), "float32")
    for steps, series in ((256, False), (256, True)):
        eng = Gb300Engine(c, "float32", max_steps=steps, record_series=series)
        peak = eng.peak_bytes()
        eng.close()
        est = estimate_bytes(c, 4, max_steps=steps, record_series=series)
        assert peak <= est <= 1.1 * peak, (name, series, peak, est)
