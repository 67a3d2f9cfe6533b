"""Mode ports and wave-plane extraction (CPU).

* The compiled mode-port arrays (modal impedance, loading, template, probe weights, channel
  amplitudes) equal the reference's bit for bit: ``tests/test_golden_compile.py`` runs the
  ``mode_stripline`` case of ``tests/golden/cases.py`` against fixtures made by the reference.
* Here: the wave-plane S-parameters and propagation constants from the oracle's float64 run equal
  the reference's (``wave.*`` in that fixture); the reference's own mode-solver checks (a
  homogeneous coupled pair: eps_eff exact, even and odd impedances apart; the parallel-plate
  impedance); gamma from unequal planes; reference-plane shifts; and a matched stripline between
  two mode ports run long enough to ring down: |S21| = 1 and S11 small, from the port voltages and
  from the wave planes.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

from cases import CASES, namespace  # noqa: E402
from fingerprint import load  # noqa: E402

from open_analysis_gb300.deembed import gamma_from_planes, shift_reference, wave_sparams  # noqa: E402
from open_analysis_gb300.grid import ETA0  # noqa: E402
from open_analysis_gb300.model import compile_model  # noqa: E402
from open_analysis_gb300.modes import solve_modes  # noqa: E402
from open_analysis_gb300.run import port_voltage_factor  # noqa: E402
from oracle.numpy_engine import OracleEngine  # noqa: E402


def _summed(c, eng) -> dict:  # type: ignore[no-untyped-def]
    probes = eng.results()
    sums = {f"V:{q['name']}": q["probe_parts"] for q in c.ports if q.get("probe_parts")}
    sums.update(c.probe_sums)
    for name, parts in sums.items():
        probes[name] = sum(probes.pop(q) for q in parts)
    return probes


def test_wave_sparams_match_the_reference() -> None:
    ref = load(str(GOLDEN / "mode_stripline.npz"))
    builder, steps = CASES["mode_stripline"]
    m = builder(namespace("gb300"))
    c = compile_model(m, "float32")
    for k, ps in enumerate(m.plane_sets):
        want = ref[f"wave.planes{k}"]
        assert ps.spacing == want[0] and ps.ref == want[1] and ps.spacing_b == want[2]
    eng = OracleEngine(c, "float64")
    eng.step(steps)
    fac = port_voltage_factor(c.dt, m.frequencies)
    probes = {k: v * fac for k, v in _summed(c, eng).items()}
    s, gammas = wave_sparams(probes, m.plane_sets, np.array([q["r_ohm"] for q in c.ports]))
    np.testing.assert_allclose(np.stack(gammas), ref["wave.gamma"], rtol=1e-9)
    np.testing.assert_allclose(s, ref["wave.s"], rtol=1e-7, atol=1e-12 * np.abs(ref["wave.s"]).max())


def test_homogeneous_coupled_pair() -> None:
    u, v = np.linspace(0, 6e-3, 61), np.linspace(0, 2e-3, 21)
    labels = -np.ones((61, 21), dtype=np.int64)
    labels[:, 0] = 0
    labels[:, -1] = 0
    labels[20:26, 10] = 1
    labels[35:41, 10] = 2
    ms = solve_modes(u, v, np.full((60, 20), 4.0), labels, 2)
    assert np.allclose(ms.eps_eff, 4.0, atol=1e-9)
    assert ms.z[0] > 0 and ms.z[1] > 0
    assert abs(ms.z[0] - ms.z[1]) / ms.z.max() > 0.003


def test_parallel_plate_impedance() -> None:
    # strip filling the width between PMC sides over a ground plane: Z = eta0 h / (w sqrt(eps))
    w, h = 4e-3, 1e-3
    u, v = np.linspace(0, w, 41), np.linspace(0, h, 11)
    labels = -np.ones((41, 11), dtype=np.int64)
    labels[:, 0] = 0
    labels[:, -1] = 1
    ms = solve_modes(u, v, np.full((40, 10), 2.25), labels, 1)
    assert abs(ms.eps_eff[0] - 2.25) < 1e-12
    assert abs(ms.z[0] - ETA0 * h / (w * 1.5)) / ms.z[0] < 2e-3


def test_gamma_from_unequal_planes_and_shift() -> None:
    f = np.linspace(1e9, 20e9, 40)
    g_true = 0.5 * np.sqrt(f / 1e9) + 1j * 2 * np.pi * f * 1.8 / 299792458.0
    a, b = 1.0, 0.3 * np.exp(0.4j)
    z = np.array([0.0, 1.1e-3, 2.5e-3])
    v = [a * np.exp(-g_true * zz) + b * np.exp(g_true * zz) for zz in z]
    g = gamma_from_planes(v[0], v[1], v[2], 1.1e-3, 1.4e-3)
    assert np.abs(g - g_true).max() < 1e-6 * np.abs(g_true).max()
    s = np.ones((2, 2, f.size), np.complex128)
    back = shift_reference(shift_reference(s, g_true, [1e-3, 2e-3]), g_true, [-1e-3, -2e-3])
    np.testing.assert_allclose(back, s, rtol=1e-12)


def test_debye_stripline_between_mode_ports() -> None:
    """The mode-port stripline (both ports driven) run until the energy is 60 dB down. Between the
    wave planes the line is uniform, so the plane-extracted transmission is the TEM line's own:
    ``|S21| = exp(-alpha L)`` with the Debye fill's ``k = (w / c) sqrt(eps(w))`` over the 4.8 mm
    between the port planes, and the reflection vanishes. The port-plane S keeps the sheets'
    discontinuity (S11 up to 0.16 here); the planes remove it. Below about 2 GHz the planes are
    too close in phase (0.04 rad at 1 GHz) and are not judged."""
    from open_analysis_gb300.run import run, sparams

    m = CASES["mode_stripline"][0](namespace("gb300"))
    res = run(m, engine=OracleEngine, dtype="float64", max_steps=4000, end_db=-60)  # type: ignore[arg-type]
    s = sparams(m, res)
    fac = port_voltage_factor(res.dt, m.frequencies)
    probes = {k: v * fac for k, v in res.probes.items()}
    sw, gam = wave_sparams(probes, m.plane_sets, res.port_r, s_port=s, freqs=m.frequencies)
    w = 2 * np.pi * np.asarray(m.frequencies)
    k = w * np.sqrt(3.4 + 0.3 / (1 + 1j * w * 8e-12)) / 299792458.0
    expect = np.exp(k.imag * 4.8e-3)
    band = m.frequencies >= 4e9
    high = m.frequencies >= 10e9
    assert np.abs(np.abs(sw[1, 0, band]) / expect[band] - 1).max() < 0.02
    assert np.abs(np.abs(sw[1, 0, high]) / expect[high] - 1).max() < 0.007
    assert np.abs(sw[0, 0, band]).max() < 0.02 and np.abs(sw[1, 1, band]).max() < 0.02
    assert np.abs(gam[0].imag[high] / k.real[high] - 1).max() < 0.01  # the line's phase constant
    assert np.abs(s[0, 0, band]).max() > 0.05  # the port-plane S still holds the sheets' reflection


@pytest.mark.gpu
def test_mode_ports_on_the_gpu_match_the_oracle() -> None:
    """The same stripline through ``run()`` on the GPU engine and on the oracle (float32, fixed
    step count): port and wave-plane S-parameters agree to the DFT's float64 rounding."""
    from open_analysis_gb300.run import run, sparams

    out = []
    for engine in ("gb300", OracleEngine):
        m = CASES["mode_stripline"][0](namespace("gb300"))
        res = run(m, engine=engine, dtype="float32", max_steps=2500, end_db=None)  # type: ignore[arg-type]
        s = sparams(m, res)
        fac = port_voltage_factor(res.dt, m.frequencies)
        probes = {k: v * fac for k, v in res.probes.items()}
        sw, _ = wave_sparams(probes, m.plane_sets, res.port_r, s_port=s, freqs=m.frequencies)
        out.append((s, sw))
    (s_g, w_g), (s_c, w_c) = out
    assert np.abs(s_g - s_c).max() < 1e-9
    assert np.abs(w_g - w_c).max() < 1e-7
