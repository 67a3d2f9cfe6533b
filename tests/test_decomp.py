"""z-slab decomposition: the slabs together reproduce the single-domain run.

Fields are compared bit for bit (each plane is updated by exactly one slab, with the same
operands); probe DFTs and energies are sums of per-slab partial sums, so they agree to the
summation order (1e-12 of their peak). On the CPU the oracle is the per-slab engine, in one
process and as two ``gloo`` ranks; on the GPU (``-m gpu``) the CUDA engine is, as sub-engines on
one device launched one after the other.
"""

from __future__ import annotations

import socket

import numpy as np
import pytest
from cases import CASES, namespace

from open_analysis_gb300.decomp import LocalSlabs, plan_z, split_z
from open_analysis_gb300.model import ModelError, compile_model
from oracle.numpy_engine import OracleEngine

NAMES = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def _via(cpml: int = 6):  # type: ignore[no-untyped-def]
    from open_analysis_gb300.structures import via_transition

    return compile_model(via_transition(nx=40, ny=36, nz=30, n_freq=8, cpml_cells=cpml), "float32")


def _random_fields(eng, seed: int = 5) -> list[np.ndarray]:  # type: ignore[no-untyped-def]
    rng = np.random.default_rng(seed)
    out = []
    for arr in eng.E + eng.H:
        arr[...] = rng.standard_normal(arr.shape, dtype=np.float32)
        out.append(arr.astype(np.float64))
    return out


def _scatter(slabs, engines, fields) -> None:  # type: ignore[no-untyped-def]
    """Load global fields into every slab's storage, halo planes included."""
    for s, e in zip(slabs, engines, strict=True):
        z = e.shape[1] if hasattr(e, "shape") else e.E[0].shape[1]
        for comp, f in enumerate(fields):
            for kk in range(z):
                e.set_plane(comp, kk, f[:, s.z0 + kk])


def _check(local: LocalSlabs, ref, steps_done: int) -> None:  # type: ignore[no-untyped-def]
    for k, want in enumerate(ref.E + ref.H):
        got = local.field(k)
        assert np.array_equal(got, want.astype(np.float64)), f"{NAMES[k]}: max |d| = {np.abs(got - want).max()}"
    res, want_res = local.results(), ref.results()
    assert set(res) == set(want_res)
    for name, v in want_res.items():
        assert np.abs(res[name] - v).max() <= 1e-12 * max(np.abs(v).max(), 1e-300), name
    assert abs(local.energy() - ref.energy()) <= 1e-12 * abs(ref.energy())


def test_plan_covers_every_plane_once() -> None:
    for nz, parts in ((30, 2), (30, 3), (119, 4), (7, 4)):
        b = plan_z(nz, parts)
        assert b[0][0] == 1 and b[-1][1] == nz + 2
        assert all(b[i][1] == b[i + 1][0] for i in range(parts - 1))
        assert all(hi - lo >= 2 for lo, hi in b)
    with pytest.raises(ModelError):
        plan_z(4, 4)


def test_split_keeps_every_list_entry_once() -> None:
    c = _via()
    slabs = split_z(c, 3)
    assert sum(s.c.sibc.flat.size for s in slabs) == c.sibc.flat.size
    for ci in range(len(c.ade.comp)):
        assert sum(s.c.ade.flat[ci].size for s in slabs) == c.ade.flat[ci].size
    for pi, p in enumerate(c.probes):
        assert sum(np.asarray(s.c.probes[pi]["flat"]).size for s in slabs) == np.asarray(p["flat"]).size
    n_corr_cells = sum(int(np.prod(k.shape)) for k in c.pml.corrections)
    assert sum(int(np.prod(k.shape)) for s in slabs for k in s.c.pml.corrections) == n_corr_cells


@pytest.mark.parametrize("parts", [2, 3])
def test_oracle_slabs_equal_single_domain(parts: int) -> None:
    """The benchmark structure (Debye stack, SIBC copper, CPML on all walls) from random fields."""
    c = _via()
    ref = OracleEngine(c, "float32")
    fields = _random_fields(ref)
    local = LocalSlabs(c, parts, lambda sub: OracleEngine(sub, "float32"))
    _scatter(local.slabs, local.engines, fields)
    ref.step(6)
    local.step(6)
    _check(local, ref, 6)


def test_oracle_slabs_with_pmc_and_sources() -> None:
    """Mixed walls (PMC ghosts on z), a soft source and a port, from zero fields."""
    c = compile_model(CASES["mixed_walls"][0](namespace("gb300")), "float32")
    ref = OracleEngine(c, "float32")
    local = LocalSlabs(c, 3, lambda sub: OracleEngine(sub, "float32"))
    ref.step(40)
    local.step(40)
    _check(local, ref, 40)


# ------------------------------------------------------------------ two gloo ranks on the CPU
def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return int(s.getsockname()[1])


class _PointerPlanes(OracleEngine):
    """The oracle with the device-plane entry points of ``Gb300Engine`` over host memory: the
    plane is written to / read from the buffer at an address, in the engine's precision."""

    def __init__(self, c, dtype):  # type: ignore[no-untyped-def]
        super().__init__(c, dtype)
        self.B = self.E[0].shape[0]
        self.shape = self.E[0].shape

    def _view(self, addr: int):  # type: ignore[no-untyped-def]
        import ctypes

        n = self.B * self.shape[2] * self.shape[3]
        ctype = ctypes.c_float if np.dtype(self.dtype) == np.float32 else ctypes.c_double
        return np.ctypeslib.as_array((ctype * n).from_address(addr)).reshape(self.B, self.shape[2], self.shape[3])

    def plane_to_device(self, comp: int, k: int, dst: int) -> None:
        self._view(dst)[...] = (self.E + self.H)[comp][:, k]

    def plane_from_device(self, comp: int, k: int, src: int) -> None:
        (self.E + self.H)[comp][:, k] = self._view(src)


def _rank_main(rank: int, world: int, port: int, out, device: bool = False) -> None:  # type: ignore[no-untyped-def]
    import torch.distributed as dist

    from open_analysis_gb300.decomp import DistSlabs

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        c = _via()
        if device:  # the device-buffer exchange (NCCL's form) with host buffers under gloo
            run = DistSlabs(c, lambda sub: _PointerPlanes(sub, "float32"), device=True, buffer_device="cpu")
        else:
            run = DistSlabs(c, lambda sub: OracleEngine(sub, "float32"))
        ref = OracleEngine(c, "float32")
        fields = _random_fields(ref)
        s, e = run.slab, run.engine
        for comp, f in enumerate(fields):
            for kk in range(e.E[0].shape[1]):
                e.set_plane(comp, kk, f[:, s.z0 + kk])
        run.step(5)
        ref.step(5)
        ok = True
        for k, want in enumerate(ref.E + ref.H):  # this rank's owned planes
            lo = 0 if rank == 0 else s.a
            hi = want.shape[1] if rank == world - 1 else s.b
            for kk in range(lo, hi):
                ok &= bool(np.array_equal(e.plane(k, kk - s.z0), want[:, kk].astype(np.float64)))
        res, want_res = run.results(), ref.results()
        for name, v in want_res.items():
            ok &= bool(np.abs(res[name] - v).max() <= 1e-12 * max(np.abs(v).max(), 1e-300))
        ok &= abs(run.energy() - ref.energy()) <= 1e-12 * abs(ref.energy())
        out.put((rank, ok))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("device", [False, True], ids=["host", "device-buffers"])
def test_two_gloo_ranks_equal_single_domain(device: bool) -> None:
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out, device)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert got == {0: True, 1: True}


# ------------------------------------------------------------------------------- GPU slabs
@pytest.mark.gpu
@pytest.mark.parametrize("device", [False, True], ids=["host", "device"])
@pytest.mark.parametrize("parts", [2, 3])
def test_gpu_slabs_equal_single_engine(parts: int, device: bool) -> None:
    """Sub-engines on one GPU, planes exchanged through host float64 or device to device."""
    from open_analysis_gb300.engine import Gb300Engine

    c = _via(cpml=6)
    ref = OracleEngine(c, "float32", pole_sum="loop")
    fields = _random_fields(ref)
    one = Gb300Engine(c, "float32", max_steps=256)
    for k, f in enumerate(fields):
        one.set_field(k, f)
    local = LocalSlabs(c, parts, lambda sub: Gb300Engine(sub, "float32", max_steps=256), device=device)
    _scatter(local.slabs, local.engines, fields)
    one.step(20)
    local.step(20)
    ref.step(20)
    for k in range(6):
        want = one.field(k)
        assert np.array_equal(local.field(k), want), NAMES[k]
        assert np.array_equal(want, (ref.E + ref.H)[k].astype(np.float64)), NAMES[k]
    for name, v in one.results().items():
        assert np.abs(local.results()[name] - v).max() <= 1e-12 * max(np.abs(v).max(), 1e-300), name
