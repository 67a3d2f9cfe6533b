"""Engine-level jobs and the worker's files: the reference's job format in, its npz / run.json /
Touchstone out. Touchstone text is pinned to the reference's own writer
(``tests/golden/touchstone.npz`` from ``tests/golden/make_golden.py``)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from open_analysis_gb300.grid import ETA0
from open_analysis_gb300.jobs import main, model_from_job, run_job
from open_analysis_gb300.model import ModelError
from open_analysis_gb300.touchstone import format_touchstone
from oracle.numpy_engine import OracleEngine

GOLDEN = Path(__file__).resolve().parent / "golden" / "touchstone.npz"


def test_touchstone_text_matches_the_reference_writer() -> None:
    data = np.load(GOLDEN)
    keys = sorted({k.rsplit(".", 1)[0] for k in data.files})
    assert len(keys) == 5
    for key in keys:
        s = data[key + ".s"]
        n = s.shape[1]
        names = [f"port{i + 1}" for i in range(n)]
        text = format_touchstone(data[key + ".freqs"], s, list(data[key + ".z0"]), names, ["made by the reference"])
        assert text == str(data[key + ".text"]), key


def _tem_job(tmp: Path, wire: bool = True) -> Path:
    """The reference's parallel-plate TEM line as a job: matched 50-ohm-free ports (R = Z0)."""
    w, h, dy, ny = 0.008, 0.004, 0.5e-3, 40
    z0 = ETA0 * h / w
    job = {
        "grid": {"x": np.linspace(0, w, 5).tolist(), "y": (np.arange(ny + 1) * dy).tolist(), "z": np.linspace(0, h, 5).tolist()},
        "waveform": {"kind": "gauss_mod", "f0": 1.5e9, "bandwidth": 3e9},
        "frequencies": np.linspace(0.5e9, 3e9, 6).tolist(),
        "walls": ["pmc", "pmc", "pmc", "pmc", "pec", "pec"],
        "ports": [
            {"name": "p1", "axis": 2, "lo": [0, 0, 0], "hi": [w, 0, h], "r_ohm": z0},
            {"name": "p2", "axis": 2, "lo": [0, ny * dy, 0], "hi": [w, ny * dy, h], "r_ohm": z0},
        ],
        "probes": [{"name": "mid", "kind": "E", "axis": 2, "lo": [0, ny * dy / 2, 0], "hi": [w, ny * dy / 2, h], "weight": "line"}],
        "run": {"dtype": "float32", "max_steps": 4000, "end_db": -50},
        "output": "tem.npz",
        "wire": wire,
    }
    path = tmp / "job.json"
    path.write_text(json.dumps(job))
    return path


def test_malformed_job_is_a_model_error(tmp_path: Path, capsys: pytest.CaptureFixture[str]) -> None:
    with pytest.raises(ModelError):
        model_from_job({"grid": {"x": [0, 1]}})
    bad = tmp_path / "bad.json"
    bad.write_text(json.dumps({"waveform": {}}))
    assert main(["run", str(bad)]) == 2
    err = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert err["code"] == "FDTD_BAD_JOB" and set(err) == {"code", "message", "path", "hint"}


def test_job_outputs_on_the_oracle(tmp_path: Path) -> None:
    path = _tem_job(tmp_path)
    summary = run_job(path, engine=OracleEngine)
    out = np.load(summary["output"])
    assert out["s"].shape == (2, 2, 6) and "probe_mid" in out
    wire = np.load(summary["wire"])
    assert wire["s"].shape == (6, 2, 2) and list(wire["names"]) == ["p1", "p2"]
    assert np.array_equal(wire["s"], np.moveaxis(out["s"], -1, 0))
    meta = json.loads(Path(summary["run_json"]).read_text())
    assert meta["port_names"] == ["p1", "p2"] and meta["steps"] == summary["steps"]
    text = Path(summary["touchstone"]).read_text()
    assert summary["touchstone"].endswith(".s2p") and "# HZ S RI R" in text
    assert np.abs(np.abs(out["s"][1, 0]) - 1.0).max() < 2e-2  # a matched line: |S21| ~ 1


@pytest.mark.gpu
def test_job_on_the_gpu_matches_the_oracle(tmp_path: Path) -> None:
    (tmp_path / "gpu").mkdir()
    (tmp_path / "cpu").mkdir()
    gpu = run_job(_tem_job(tmp_path / "gpu"), engine="gb300")
    cpu = run_job(_tem_job(tmp_path / "cpu"), engine=OracleEngine)
    assert gpu["engine"] == "gb300" and gpu["steps"] == cpu["steps"]
    s_gpu, s_cpu = np.load(gpu["output"])["s"], np.load(cpu["output"])["s"]
    assert np.abs(s_gpu - s_cpu).max() < 1e-9  # the same float32 fields; DFT rounding only


def test_wire_files_carry_the_modal_impedance(tmp_path: Path) -> None:
    """Mode ports: the worker's z0 is the modal impedance of each port (the run's port_r)."""
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    from cases import CASES, namespace

    from open_analysis_gb300.jobs import write_wire
    from open_analysis_gb300.run import run, sparams

    m = CASES["mode_stripline"][0](namespace("gb300"))
    res = run(m, engine=OracleEngine, dtype="float32", max_steps=64, end_db=None)
    paths = write_wire(tmp_path, "modes", m, sparams(m, res), res, 0.0, 0.0)
    wire = np.load(paths["wire"])
    assert np.array_equal(wire["z0"], res.port_r) and abs(wire["z0"][0] - 55.77) < 0.01
    assert "R 55.77" in Path(paths["touchstone"]).read_text() or "55.77" in Path(paths["touchstone"]).read_text()


def test_job_parser_matches_the_reference_cli() -> None:
    """``model_from_job`` on a job using every key of the reference's format compiles to the
    reference's arrays bit for bit (fixture from the reference's ``oa_fdtd.cli.model_from_job``)."""
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    from cases import job_dict
    from fingerprint import compare_compiled, compiled_fingerprint, load

    from open_analysis_gb300.model import compile_model

    ref = load(str(GOLDEN.parent / "job_parse.npz"))
    mine = compiled_fingerprint(compile_model(model_from_job(job_dict()), "float32"))
    assert compare_compiled(ref, mine) == []
