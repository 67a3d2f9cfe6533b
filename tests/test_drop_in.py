"""The drop-in boundary fed with the reference's own compiled objects.

``tests/golden/ref_compiled_<case>.npz`` holds the ``Compiled`` that the reference's
``compile_model`` built (``tests/golden/make_golden.py``, part ``compiled``), with the reference
grid's metrics and its waveform samples; ``compiled_io.load`` gives it back with the attributes of
the reference's class. The engine's descriptor (``engine.describe``, what ``oafdtd_create``
receives) built from it must equal, byte for byte, the one built from this package's
``compile_model``, and (``-m gpu``) the engine fed the reference's object must reproduce the
reference's own float32 fields and DFTs (``Fs/run.py:46-75`` builds the engine the same way).
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest
from cases import CASES, namespace
from compiled_io import load
from fingerprint import digest
from fingerprint import load as load_fixture

from open_analysis_gb300.engine import describe
from open_analysis_gb300.model import compile_model

GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
STORED = ("dispersive_copper", "mode_stripline")
MAX_STEPS = 128  # the stored waveform covers these steps


def _descriptor(c) -> tuple[dict, list]:  # type: ignore[no-untyped-def]
    """The descriptor's plain fields (pointers left out) and the host buffers it points into."""
    p, keep = describe(c, "float32", MAX_STEPS)
    fields = {}
    for name, _ in p._fields_:
        v = getattr(p, name)
        if isinstance(v, C.Array):
            if issubclass(v._type_, (C._Pointer, C.Array)):
                continue
            v = list(v)
        elif isinstance(v, C._Pointer):
            continue
        fields[name] = v
    return fields, keep


@pytest.mark.parametrize("case", STORED)
def test_reference_compiled_gives_the_same_descriptor(case: str) -> None:
    ref = load(str(GOLDEN / f"ref_compiled_{case}.npz"))
    mine = compile_model(CASES[case][0](namespace("gb300")), "float32")
    f_ref, k_ref = _descriptor(ref)
    f_mine, k_mine = _descriptor(mine)
    assert f_ref == f_mine
    assert len(k_ref) == len(k_mine)
    for n, (a, b) in enumerate(zip(k_ref, k_mine, strict=True)):
        if isinstance(a, np.ndarray):
            assert a.dtype == b.dtype and a.shape == b.shape, n
            assert a.tobytes() == b.tobytes(), f"buffer {n} ({a.dtype}, {a.shape}) differs"
        else:
            assert bytes(a) == bytes(b), f"buffer {n} differs"


@pytest.mark.gpu
@pytest.mark.parametrize("case", STORED)
def test_reference_compiled_on_the_gpu_reproduces_the_reference(case: str) -> None:
    from open_analysis_gb300.engine import Gb300Engine

    c = load(str(GOLDEN / f"ref_compiled_{case}.npz"))
    want = load_fixture(str(GOLDEN / f"{case}.npz"))
    steps = int(want["steps"])
    eng = Gb300Engine(c, "float32", max_steps=MAX_STEPS)
    eng.step(steps)
    for k, name in enumerate(NAMES):
        assert digest(eng.field(k).astype(np.float32)) == want[f"float32.field.{name}.sha"], name
    for name, v in eng.results().items():
        ref = want[f"float32.dft.{name}"]
        assert np.abs(v - ref).max() <= 1e-9 * max(np.abs(ref).max(), 1e-300), name
    eng.close()
