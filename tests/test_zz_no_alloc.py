"""The field energy without device allocation, through the C ABI, against the engine's own
energy entry point and the CPU oracle.

``oafdtd_energy_noalloc`` serves callers that cannot allocate device memory (a plugin whose host
application owns every device allocation, a service that reserves its device memory at start-up
and may not grow it): it takes fields already on the device and keeps its partial sums in a fixed
device array compiled into the library. This file runs last so that a failure here leaves every
other test's result in place.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest


@pytest.mark.gpu
def test_energy_noalloc_matches_engine_energy_on_two_calls() -> None:
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch sees no CUDA device")
    from cases import CASES, namespace

    from open_analysis_gb300 import native
    from open_analysis_gb300.engine import Gb300Engine
    from open_analysis_gb300.model import compile_model

    lib = native.load()
    c = compile_model(CASES["dispersive_copper"][0](namespace("gb300")), "float32")
    g = c.grid
    eng = Gb300Engine(c, "float32", max_steps=256)
    dev = torch.device("cuda:0")
    keep = []

    def on_device(a: np.ndarray) -> int:
        t = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        keep.append(t)
        return int(t.data_ptr())

    view = native.EnergyView()
    view.real_bytes = 4
    view.nx, view.ny, view.nz = g.n
    view.pitch = g.pitch
    view.batch = c.batch
    for a in range(3):
        view.idx[a] = on_device(np.asarray(c.idx[a]).view(np.int16))
        view.node_w[a] = on_device(g.node_weights(a))
        view.cell_w[a] = on_device(g.cell_weights(a))
    view.eps_tab = on_device(np.asarray(c.eps_tab, dtype=np.float64))
    view.stream = None
    from oracle.numpy_engine import OracleEngine

    oracle = OracleEngine(c, "float32", pole_sum="loop")
    free = []
    for steps in (30, 45):  # two calls in a row, on different fields
        eng.step(steps)
        oracle.step(steps)
        for k in range(6):
            view.field[k] = on_device(eng.field(k).astype(np.float32))
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info()[0]
        out = C.c_double()
        rc = lib.oafdtd_energy_noalloc(C.byref(view), C.byref(out))
        assert rc == native.OK, lib.oafdtd_last_error().decode()
        free.append((before, torch.cuda.mem_get_info()[0]))
        want = eng.energy()
        assert want > 0
        assert abs(out.value - want) <= 1e-12 * want, (out.value, want)
        want_cpu = oracle.energy()
        assert abs(out.value - want_cpu) <= 1e-10 * want_cpu, (out.value, want_cpu)
    # the second call (its device's set-up done by the first) leaves free device memory as it was
    assert free[1][0] == free[1][1], free
    # on a stream that is being captured the synchronous call is refused, and the capture survives
    s = torch.cuda.Stream()
    view.stream = s.cuda_stream
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        rc = lib.oafdtd_energy_noalloc(C.byref(view), C.byref(C.c_double()))
        y = keep[-1] * 2.0
    assert rc == native.E_INVALID and b"captured" in lib.oafdtd_last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, keep[-1] * 2.0)


def test_energy_noalloc_rejects_oversized_problems() -> None:
    from open_analysis_gb300 import native

    lib = native.load()
    view = native.EnergyView()
    view.real_bytes = 4
    view.nx, view.ny, view.nz, view.pitch, view.batch = 8, 8, 20000, 32, 1
    for k in range(6):
        view.field[k] = 16  # never dereferenced: the size check comes first
    for a in range(3):
        view.idx[a] = view.node_w[a] = view.cell_w[a] = 16
    view.eps_tab = 16
    out = C.c_double()
    assert lib.oafdtd_energy_noalloc(C.byref(view), C.byref(out)) == native.E_INVALID
    assert b"static scratch" in lib.oafdtd_last_error()
