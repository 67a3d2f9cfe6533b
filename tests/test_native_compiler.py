"""The native model compiler (``oafdtd_materials_build``) against the NumPy stages it replaces.

Both must give the same compiled arrays bit for bit: the uint16 index arrays, the eps / sigma /
ca / cb tables and the Debye edge lists. The NumPy stages restate the reference's and are pinned
to it by ``tests/test_golden_compile.py`` (which runs the default, native, path as well). No GPU:
the native compiler is host code in the engine library.
"""

from __future__ import annotations

import numpy as np
import pytest

from open_analysis_gb300.grid import Grid, uniform_lines
from open_analysis_gb300.model import Conductor, LumpedPort, Model, Region, Waveform, _native_library, compile_model
from open_analysis_gb300.pml import CpmlSpec
from open_analysis_gb300.structures import microstrip, via_transition
from open_analysis_gb300.surrogate import HALF, via_instance, via_params

pytestmark = pytest.mark.skipif(_native_library() is None, reason="engine library not built")


def assert_same(a, b) -> None:  # type: ignore[no-untyped-def]
    for f in ("eps_tab", "sig_tab", "ca_tab", "cb_tab"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    for c in range(3):
        assert a.idx[c].dtype == b.idx[c].dtype == np.uint16
        assert np.array_equal(a.idx[c], b.idx[c]), ("idx", c)
    assert (a.ade is None) == (b.ade is None)
    if a.ade is not None:
        assert a.ade.comp == b.ade.comp
        assert np.array_equal(a.ade.kp, b.ade.kp) and np.array_equal(a.ade.tau, b.ade.tau)
        for x, y in zip(a.ade.flat, b.ade.flat, strict=True):
            assert x.dtype == y.dtype and np.array_equal(x, y)
        for x, y in zip(a.ade.beta, b.ade.beta, strict=True):
            assert np.array_equal(x, y)
        for x, y in zip(a.ade.cbe, b.ade.cbe, strict=True):
            assert np.array_equal(x, y)
    for p, q in zip(a.channels, b.channels, strict=True):
        assert np.array_equal(p["amps"], q["amps"])


def random_model(seed: int) -> Model:
    """Graded lines, overlapping dielectric regions with one to three Debye poles, a PEC region,
    surface-impedance copper, two lumped ports (their loading lands on the table), CPML and PMC."""
    rng = np.random.default_rng(seed)
    lines = []
    for n in (23, 19, 17):
        d = 50e-6 * rng.uniform(0.7, 1.4, n)
        lines.append(np.concatenate([[0.0], np.cumsum(d)]))
    g = Grid(*lines)
    ext = [float(v[-1]) for v in lines]
    m = Model(
        g,
        Waveform("gauss_mod", 10e9, 20e9),
        np.linspace(1e9, 20e9, 5),
        walls=("cpml", "pmc", "cpml", "cpml", "pec", "cpml"),
        cpml=CpmlSpec(cells=4),
    )
    taus = [4e-12, 9e-12, 2.5e-11]
    for _ in range(6):
        lo = [rng.uniform(-0.1, 0.6) * e for e in ext]
        hi = [lo[a] + rng.uniform(0.2, 0.9) * ext[a] for a in range(3)]
        poles = tuple((float(rng.uniform(0.05, 0.6)), taus[int(rng.integers(3))]) for _ in range(int(rng.integers(0, 3))))
        m.regions.append(Region(tuple(lo), tuple(hi), float(rng.uniform(1.5, 6.0)), sigma=float(rng.choice([0.0, 0.02, 0.3])),
                                poles=poles))
    m.regions.append(Region((0.3 * ext[0], 0.3 * ext[1], 0.5 * ext[2]), (0.6 * ext[0], 0.5 * ext[1], 0.5 * ext[2]), pec=True))
    m.conductors.append(Conductor((0.2 * ext[0], 0.6 * ext[1], 0.2 * ext[2]), (0.7 * ext[0], 0.8 * ext[1], 0.3 * ext[2]),
                                  sigma=5.8e7, thickness=35e-6))
    zt = float(lines[2][6])
    m.ports.append(LumpedPort("p1", 2, (float(lines[0][5]), float(lines[1][9]), 0.0), (float(lines[0][5]), float(lines[1][9]), zt), 50.0))
    m.ports.append(LumpedPort("p2", 2, (float(lines[0][15]), float(lines[1][9]), 0.0), (float(lines[0][15]), float(lines[1][12]), zt), 35.0))
    return m


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_random_models_equal_numpy(seed: int) -> None:
    m = random_model(seed)
    assert_same(compile_model(m, native=True), compile_model(m, native=False))


def test_benchmark_structures_equal_numpy() -> None:
    for m in (microstrip(), via_transition(nx=96, ny=80, nz=48), via_instance(via_params(1, seed=5)[0], HALF)):
        assert_same(compile_model(m, native=True), compile_model(m, native=False))


def test_vacuum_only_equals_numpy() -> None:
    g = Grid(uniform_lines(9, 1e-3), uniform_lines(7, 1e-3), uniform_lines(5, 1e-3))
    m = Model(g, Waveform("gauss", 0.0, 5e9), np.array([1e9]))
    assert_same(compile_model(m, native=True), compile_model(m, native=False))


def test_thread_counts_give_the_same_arrays(monkeypatch: pytest.MonkeyPatch) -> None:
    import open_analysis_gb300.model as model_mod

    m = random_model(7)
    base = compile_model(m, native=False)
    orig = model_mod._native_materials
    for threads in (1, 3, 16):
        monkeypatch.setattr(model_mod, "_native_materials", lambda *a, t=threads, **k: orig(*a, threads=t))
        assert_same(compile_model(m, native=True), base)
