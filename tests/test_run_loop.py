"""``run()`` against the reference's own run loop (CPU, the oracle as engine).

``tests/golden/run_loops.npz`` (``make_golden.run_loops``) holds the reference's ``run(engine=
"numpy", dtype="float64")`` on two cases: the microstrip stopped by the end criterion, and the
mode-port stripline stopped at ``max_steps`` with the matrix-pencil tail continuation. Here the
same loop runs with the oracle in float64 (which equals the reference's engine bit for bit): the
same step count, stop reason and energy level, and the same S-parameters.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

from cases import CASES, namespace  # noqa: E402
from make_golden import RUNS  # noqa: E402

from open_analysis_gb300.run import run, sparams  # noqa: E402
from oracle.numpy_engine import OracleEngine  # noqa: E402


@pytest.mark.parametrize("case", sorted(RUNS))
def test_run_loop_matches_the_reference(case: str) -> None:
    ref = np.load(GOLDEN / "run_loops.npz")
    m = CASES[case][0](namespace("gb300"))
    res = run(m, engine=OracleEngine, dtype="float64", **RUNS[case])  # type: ignore[arg-type]
    assert res.steps == int(ref[f"{case}.steps"])
    assert res.stopped_by == str(ref[f"{case}.stopped_by"])
    assert abs(res.energy_db - float(ref[f"{case}.energy_db"])) <= 1e-9
    s, want = sparams(m, res), ref[f"{case}.s"]
    fin = np.isfinite(want)
    assert np.array_equal(np.isfinite(s), fin)
    assert np.abs(s[fin] - want[fin]).max() <= 1e-10 * max(1.0, np.abs(want[fin]).max())
    if f"{case}.wave_s" in ref.files:  # wave planes with the port S fallback and gamma smoothing
        from open_analysis_gb300.deembed import wave_sparams
        from open_analysis_gb300.run import port_voltage_factor

        fac = port_voltage_factor(res.dt, m.frequencies)
        probes = {k: v * fac for k, v in res.probes.items()}
        sw, gam = wave_sparams(probes, m.plane_sets, res.port_r, s_port=s, freqs=m.frequencies)
        np.testing.assert_allclose(np.stack(gam), ref[f"{case}.wave_gamma"], rtol=1e-8)
        np.testing.assert_allclose(sw, ref[f"{case}.wave_s"], rtol=1e-8, atol=1e-10)
    for key in [k for k in ref.files if k.startswith(f"{case}.tail.")]:
        got = (res.tail or {})[key.rsplit(".", 1)[1]]
        np.testing.assert_allclose(np.asarray(got, dtype=np.float64), ref[key].astype(np.float64), rtol=1e-6, err_msg=key)
