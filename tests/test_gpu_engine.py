"""GPU engine against the CPU oracle: bit-exact fields, DFTs, energy, S-parameters.

The oracle (``oracle/numpy_engine.py``) is pinned against the reference itself by
``test_golden_compile.py``; here the CUDA engine runs the same compiled problems through the
C ABI. The library is built without FMA contraction and keeps the reference's operations in the
reference's order, so its fields equal the oracle's bit for bit. The one exception is the Debye
pole sum of multi-pole runs, which NumPy's einsum may reorder on some hosts: there the engine
equals the oracle with the poles summed in index order (``pole_sum="loop"``) and the einsum
oracle within float32 rounding noise.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
from cases import CASES, namespace
from fingerprint import digest, load

from open_analysis_gb300.model import compile_model
from oracle.numpy_engine import OracleEngine

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _engine(c, dtype="float32", **kw):  # type: ignore[no-untyped-def]
    from open_analysis_gb300.engine import Gb300Engine

    return Gb300Engine(c, dtype, max_steps=kw.pop("max_steps", 2000), **kw)


def test_report_numpy_pole_sum_order() -> None:
    """Not a check: records whether this host's NumPy sums Debye poles in the kernel's order
    (it decides whether multi-pole cases compare bit for bit or by rel-L2)."""
    print("einsum sequential:", _einsum_is_sequential())


def _ade_in_cpml(c) -> bool:  # type: ignore[no-untyped-def]
    """Whether a Debye edge lies inside an E CPML box: there the engine applies the correction
    after the Debye update (adding beta t to the currents), the same result up to rounding."""
    if c.ade is None:
        return False
    Y, X = c.grid.shape[1], c.grid.shape[2]
    for comp, flat in zip(c.ade.comp, c.ade.flat, strict=True):
        k, rem = np.divmod(np.asarray(flat), Y * X)
        j, i = np.divmod(rem, X)
        for corr in c.pml.corrections:
            if corr.kind != "E" or corr.c != comp:
                continue
            (x0, x1), (y0, y1), (z0, z1) = corr.box
            if np.any((i >= x0) & (i < x1) & (j >= y0) & (j < y1) & (k >= z0) & (k < z1)):
                return True
    return False


def _einsum_is_sequential() -> bool:
    """Whether this host's NumPy sums Debye poles as a plain float32 loop (the kernel's order)."""
    rng = np.random.default_rng(0)
    a = rng.random(3).astype(np.float32)
    j = rng.standard_normal((3, 4, 257)).astype(np.float32)
    seq = np.zeros((4, 257), np.float32)
    for p in range(3):
        seq = seq + a[p] * j[p]
    return bool(np.array_equal(np.einsum("p,pbe->be", a, j), seq))


def _rel(got, want) -> float:  # type: ignore[no-untyped-def]
    return float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))


def _fields(e) -> list:  # type: ignore[no-untyped-def]
    return [f.astype(np.float64) for f in (e.E + e.H)]


def _reference_tolerance(c, steps: int, dtype: str, ref_fields: list) -> list[float]:  # type: ignore[no-untyped-def]
    """Per component: 1e-5 (float32) or 1e-12 (float64) rel-L2, or twice the distance of the
    float32 oracle from the float64 oracle where the case itself is worse conditioned than that
    (a thin field component that float32 rounding alone moves by more than 1e-5)."""
    base = 1e-5 if dtype == "float32" else 1e-12
    if dtype != "float32":
        return [base] * 6
    r64 = OracleEngine(c, "float64")
    r64.step(steps)
    return [max(base, 2.0 * _rel(ref_fields[k], f)) for k, f in enumerate(_fields(r64))]


def check_against_oracles(c, gpu, steps: int, dtype: str = "float32", results: bool = True) -> None:  # type: ignore[no-untyped-def]
    """The engine's fields equal the oracle's (poles summed in index order) bit for bit, its DFTs
    and energy agree to float64 summation order, and its fields equal the einsum oracle's, or
    are within its rounding noise where einsum reorders the pole sum."""
    eng = OracleEngine(c, dtype, pole_sum="loop")
    eng.step(steps)
    for k, want in enumerate(_fields(eng)):
        got = gpu.field(k)
        assert np.array_equal(got, want), f"{NAMES[k]}: max |d| = {np.abs(got - want).max()}"
    if results:
        r_gpu, r_eng = gpu.results(), eng.results()
        assert set(r_gpu) == set(r_eng)
        for name, v in r_eng.items():
            assert r_gpu[name].shape == v.shape
            assert np.abs(r_gpu[name] - v).max() <= 1e-9 * max(np.abs(v).max(), 1e-300), name
        e_gpu, e_eng = gpu.energy(), eng.energy()
        assert abs(e_gpu - e_eng) <= 1e-10 * abs(e_eng)
    ref = OracleEngine(c, dtype)
    ref.step(steps)
    ref_fields = _fields(ref)
    if all(np.array_equal(a, b) for a, b in zip(ref_fields, _fields(eng), strict=True)):
        return
    tol = _reference_tolerance(c, steps, dtype, ref_fields)
    for k, want in enumerate(ref_fields):
        rel = _rel(gpu.field(k), want)
        assert rel <= tol[k], f"{NAMES[k]}: rel-L2 {rel} against the einsum oracle (bound {tol[k]})"


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_fields_match_oracle(case: str, dtype: str) -> None:
    builder, steps = CASES[case]
    c = compile_model(builder(namespace("gb300")), "float32")
    gpu = _engine(c, dtype)
    gpu.step(steps)
    check_against_oracles(c, gpu, steps, dtype)


@pytest.mark.parametrize("case", ["mixed_walls", "microstrip", "mode_stripline"])
def test_fields_match_reference_fixture(case: str) -> None:
    """The float32 fields' digests equal those of the reference's own NumPy engine."""
    ref = load(str(GOLDEN / f"{case}.npz"))
    builder, steps = CASES[case]
    c = compile_model(builder(namespace("gb300")), "float32")
    gpu = _engine(c)
    gpu.step(steps)
    for k, name in enumerate(NAMES):
        assert digest(gpu.field(k).astype(np.float32)) == ref[f"float32.field.{name}.sha"], name


def test_graph_equals_eager_and_runs_repeat() -> None:
    c = compile_model(CASES["mixed_walls"][0](namespace("gb300")), "float32")
    a = _engine(c, use_graph=True, max_steps=700)
    b = _engine(c, use_graph=False, max_steps=700)
    a.step(256)
    b.step(100)
    b.step(156)
    for k, v in a.results().items():
        assert np.array_equal(v, b.results()[k])
    for k in range(6):
        assert np.array_equal(a.field(k), b.field(k))
    d = _engine(c, use_graph=True, max_steps=700)
    d.step(256)
    assert np.array_equal(a.energy(), d.energy())


def test_step_past_max_steps_raises() -> None:
    c = compile_model(CASES["microstrip"][0](namespace("gb300")), "float32")
    eng = _engine(c, max_steps=10)
    eng.step(10)
    with pytest.raises(ValueError):
        eng.step(1)


def test_series_recording_matches_oracle() -> None:
    c = compile_model(CASES["mixed_walls"][0](namespace("gb300")), "float32")
    gpu = _engine(c, record_series=True, max_steps=200)
    ref = OracleEngine(c, "float32", record_series=True)
    gpu.step(70)
    ref.step(70)
    sg, sr = gpu.series(), ref.series()
    assert set(sg) == set(sr)
    for k, v in sr.items():
        assert sg[k].shape == v.shape
        assert np.abs(sg[k] - v).max() <= 1e-12 * max(np.abs(v).max(), 1e-300)


def test_run_sparams_match_oracle() -> None:
    """run() + sparams() through the engine against the same driver over the oracle."""
    from open_analysis_gb300.run import run, sparams

    m = CASES["microstrip"][0](namespace("gb300"))
    gpu = run(m, engine="gb300", dtype="float32", end_db=None, max_steps=300)
    ref = run(m, engine=OracleEngine, dtype="float32", end_db=None, max_steps=300)
    s_gpu, s_ref = sparams(m, gpu), sparams(m, ref)
    assert np.abs(s_gpu - s_ref).max() <= 1e-3
    assert np.abs(s_gpu - s_ref).max() <= 1e-9  # same float32 fields: only DFT rounding differs
    assert gpu.engine == "gb300" and gpu.peak_bytes > 0 and gpu.report["backend"] == "cuda"


def test_energy_end_criterion_runs() -> None:
    from open_analysis_gb300.run import run

    m = CASES["microstrip"][0](namespace("gb300"))
    res = run(m, engine="gb300", end_db=-30.0, max_steps=20000)
    assert res.stopped_by == "end_criterion" and res.energy_db <= -30.0


def test_kernel_profile_and_model_bytes() -> None:
    c = compile_model(CASES["dispersive_copper"][0](namespace("gb300")), "float32")
    eng = _engine(c)
    eng.set_profiling(True)
    eng.step(64)
    t = eng.kernel_times()
    assert t["step"] > 0 and t["h_sweep"] > 0 and t["e_sweep"] > 0 and t["e_slab"] > 0
    assert t["step"] >= t["h_sweep"] + t["e_sweep"]
    # one replay: the same kernels for each of the 64 time steps, then the step-counter bump
    n = eng.graph_kernels()
    assert n >= 64 * 2 + 1 and (n - 1) % 64 == 0, n
    assert eng.model_bytes() > 0


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("tile_z", [3, 32])
def test_launch_shapes_match_oracle(variant: int, tile_z: int) -> None:
    """Every sweep variant and z tiling gives the oracle's float32 fields bit for bit."""
    c = compile_model(CASES["microstrip"][0](namespace("gb300")), "float32")
    gpu = _engine(c)
    gpu.set_tuning(tile_z, variant)
    gpu.step(70)
    check_against_oracles(c, gpu, 70, results=False)


@pytest.mark.parametrize("cpml_cells", [6, 10])
def test_variants_agree_across_x_tiles(cpml_cells: int) -> None:
    """A grid two tiles wide in x (the second one past the grid's edge, where TMA boxes are
    zero-filled) with the benchmark's Debye stack, copper SIBC and CPML: the three sweep variants
    give identical fields, equal to the oracle's. With 10 CPML cells the interior starts after
    x = 10, as in the benchmark (its first quad is rounded up to an even one)."""
    from open_analysis_gb300.structures import via_transition

    c = compile_model(via_transition(nx=150, ny=24, nz=24, n_freq=8, cpml_cells=cpml_cells), "float32")
    assert c.grid.shape[2] > 128 and _ade_in_cpml(c)
    fields = {}
    for variant in (0, 1, 2, 3):
        gpu = _engine(c)
        gpu.set_tuning(5, variant)
        gpu.step(40)
        fields[variant] = [gpu.field(k) for k in range(6)]
        if variant == 2:
            check_against_oracles(c, gpu, 40)
        gpu.close()
    for k in range(6):
        assert np.array_equal(fields[2][k], fields[1][k]), NAMES[k]
        assert np.array_equal(fields[2][k], fields[0][k]), NAMES[k]
        assert np.array_equal(fields[2][k], fields[3][k]), NAMES[k]


def test_fused_variant_switches_mid_run_bit_for_bit() -> None:
    """The fused sweep (two buffers per field) against the oracle across variant switches and odd
    step counts: 70 steps fused (one graph chunk, six eager steps), 51 in place, 64 fused again,
    then 3 eager steps; the benchmark structure at 150 x 48 x 40 with 10-cell CPML."""
    from open_analysis_gb300.structures import via_transition

    c = compile_model(via_transition(nx=150, ny=48, nz=40, n_freq=8), "float32")
    gpu = _engine(c)
    gpu.set_tuning(8, 3)
    gpu.step(70)
    gpu.set_tuning(8, 2)
    gpu.step(51)
    gpu.set_tuning(16, 3)
    gpu.step(64)
    gpu.step(3)
    check_against_oracles(c, gpu, 188)


def test_via_transition_small_matches_oracle() -> None:
    """The benchmark structure (Debye stack, SIBC copper, via, CPML on all walls) at 48x40x32."""
    from open_analysis_gb300.structures import via_transition

    c = compile_model(via_transition(nx=48, ny=40, nz=32, n_freq=16, cpml_cells=6), "float32")
    assert _ade_in_cpml(c)  # the Debye stack reaches into the x and y slabs
    gpu = _engine(c)
    gpu.step(50)
    check_against_oracles(c, gpu, 50)


def test_benchmark_size_from_random_fields_matches_oracle() -> None:
    """The benchmark problem at full size (400x400x120 cells, batch 2: Debye stack, SIBC copper,
    10-cell CPML, lumped ports) started from seeded random fields, so every CPML slab, Debye
    edge and surface-impedance edge is active from the first step: three steps bit for bit."""
    from open_analysis_gb300.structures import via_transition

    c = compile_model(via_transition(), "float32")
    gpu = _engine(c, max_steps=64)
    ref = OracleEngine(c, "float32", pole_sum="loop")
    rng = np.random.default_rng(2026)
    for k, arr in enumerate(ref.E + ref.H):
        arr[...] = rng.standard_normal(arr.shape, dtype=np.float32)
        gpu.set_field(k, arr)
    gpu.step(3)
    ref.step(3)
    for k, want in enumerate(ref.E + ref.H):
        got = gpu.field(k)
        assert np.array_equal(got, want.astype(np.float64)), f"{NAMES[k]}: max |d| = {np.abs(got - want).max()}"


def test_snapshot_restore_resumes_bit_for_bit() -> None:
    """A snapshot after 70 steps (mid-chunk), 50 more steps; restoring it (into the same engine
    and into a fresh one) and stepping 50 again gives the same fields, DFTs and energy."""
    c = compile_model(CASES["dispersive_copper"][0](namespace("gb300")), "float32")
    a = _engine(c, max_steps=400)
    a.step(70)
    state = a.snapshot()
    a.step(50)
    want = [a.field(k) for k in range(6)]
    want_res, want_e = a.results(), a.energy()
    for eng in (a, _engine(c, max_steps=400)):
        eng.restore(state)
        assert eng.step_count == 70
        eng.step(50)
        for k in range(6):
            assert np.array_equal(eng.field(k), want[k]), NAMES[k]
        for name, v in want_res.items():
            assert np.array_equal(eng.results()[name], v), name
        assert eng.energy() == want_e
    other = _engine(compile_model(CASES["mixed_walls"][0](namespace("gb300")), "float32"))
    with pytest.raises(Exception):
        other.restore(state)


def test_run_report_carries_rate_and_traffic() -> None:
    from open_analysis_gb300.run import run

    res = run(CASES["microstrip"][0](namespace("gb300")), engine="gb300", end_db=None, max_steps=128)
    assert res.report["gcell_updates_per_s"] > 0 and res.report["bytes_per_step"] > 0
