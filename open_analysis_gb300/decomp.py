"""z-slab domain decomposition of one compiled problem over several engines (one GPU each).

The reference runs one grid on one device. A grid larger than one GPU, or a run spread for
speed, splits along z: rank r owns the E/H planes ``[a_r, b_r)`` of the storage (planes 1 ..
nz+1 in total) and holds one halo plane on each side. The leapfrog step couples neighbouring
slabs through one plane per half step:

* after the H half, rank r sends Hx and Hy of its last plane ``b_r - 1`` to rank r + 1, whose
  E update of plane ``a_{r+1} = b_r`` takes their z derivatives (and whose surface-impedance edges
  may sample them);
* after the E half, rank r + 1 sends Ex and Ey of its first plane ``a_{r+1}`` to rank r, whose
  H update of plane ``b_r - 1`` takes their z derivatives.

Everything else is local: CPML psi, Debye currents and surface-impedance state live with the
edges of the owned planes, lists are split by plane and re-indexed, the 1-D metrics and CPML
coefficients are the global ones sliced (a slab edge is not a wall), probe sums, DFTs and
energies are per rank and add up. The halo planes get zero energy weight. A rank's engine also
updates the E values of its upper halo (the plane is in its storage); they are overwritten by the
exchange before anything reads them.

Transports: ``LocalSlabs`` holds every rank's engine in one process and copies the planes (tests;
several sub-engines on one GPU, launched one after the other, no kernel waiting on another);
``DistSlabs`` runs one rank per process and exchanges the planes with ``torch.distributed``
point-to-point messages through host memory (gloo), summing results with ``all_reduce``.
"""

from __future__ import annotations

import dataclasses
from collections.abc import Callable, Sequence
from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.model import AdeData, Compiled, ModelError, SibcData
from open_analysis_gb300.pml import AxisCoeffs, Correction, Pml

FloatArray = npt.NDArray[np.float64]

EX, EY, HX, HY = 0, 1, 3, 4


def plan_z(nz: int, parts: int) -> list[tuple[int, int]]:
    """Owned plane ranges ``[a, b)`` covering storage planes 1 .. nz+1, as even as possible."""
    planes = nz + 1
    if parts < 1 or parts > planes // 2:
        raise ModelError("FDTD_BAD_DECOMPOSITION", f"{parts} slabs cannot split {planes} planes (two or more each)")
    edges = [1 + (planes * r) // parts for r in range(parts + 1)]
    return [(edges[r], edges[r + 1]) for r in range(parts)]


class SlabGrid:
    """The grid as one slab sees it: x and y as the global grid, z the slab's storage planes
    ``z0 .. z0 + Z - 1`` with the global metrics (the slab faces are not walls) and zero energy
    weight on its halo planes."""

    def __init__(self, g: Any, z0: int, nz_local: int, halo_lo: bool, halo_hi: bool) -> None:
        self.g = g
        self.z0 = z0
        self._n = (g.n[0], g.n[1], nz_local)
        self.halo = (halo_lo, halo_hi)

    @property
    def n(self) -> tuple[int, int, int]:
        return self._n

    @property
    def cells(self) -> int:
        return int(np.prod(self._n))

    @property
    def pitch(self) -> int:
        return int(self.g.pitch)

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self._n[2] + 2, self._n[1] + 2, self.pitch)

    def length(self, axis: int) -> int:
        return self.pitch if axis == 0 else self._n[axis] + 2

    def _z(self, values: FloatArray, weights: bool) -> FloatArray:
        out = np.array(values[self.z0 : self.z0 + self.length(2)], dtype=np.float64)
        if weights:
            if self.halo[0]:
                out[0] = 0.0
            if self.halo[1]:
                out[-1] = 0.0
        return out

    def inv_primal(self, axis: int) -> FloatArray:
        return self.g.inv_primal(axis) if axis < 2 else self._z(self.g.inv_primal(2), False)

    def inv_dual(self, axis: int) -> FloatArray:
        return self.g.inv_dual(axis) if axis < 2 else self._z(self.g.inv_dual(2), False)

    def node_weights(self, axis: int) -> FloatArray:
        return self.g.node_weights(axis) if axis < 2 else self._z(self.g.node_weights(2), True)

    def cell_weights(self, axis: int) -> FloatArray:
        return self.g.cell_weights(axis) if axis < 2 else self._z(self.g.cell_weights(2), True)

    def is_node(self, kind: str, comp: int, axis: int) -> bool:
        return (axis != comp) if kind == "E" else (axis == comp)

    def valid(self, kind: str, comp: int) -> tuple[tuple[int, int], ...]:
        return tuple((1, self._n[a] + 2) if self.is_node(kind, comp, a) else (1, self._n[a] + 1) for a in range(3))


@dataclasses.dataclass(frozen=True)
class Slab:
    """One rank's share: owned planes ``[a, b)`` (global storage indices), the global storage
    plane ``z0`` of its local plane 0, and its problem."""

    a: int
    b: int
    z0: int
    c: Compiled

    @property
    def last_local(self) -> int:
        """Local index of the last owned plane."""
        return self.b - 1 - self.z0


def _plane_of(flat: npt.NDArray[np.int64], plane: int) -> npt.NDArray[np.int64]:
    return np.asarray(flat, dtype=np.int64) // plane


def split_z(c: Compiled, parts: int) -> list[Slab]:
    """The problem of every rank of a ``parts``-slab decomposition along z."""
    g = c.grid
    nx, ny, nz = g.n
    Y, X = g.shape[1], g.shape[2]
    plane = X * Y
    slabs = []
    bounds = plan_z(nz, parts)
    for r, (a, b) in enumerate(bounds):
        last = r == parts - 1
        z0 = a - 1
        z1 = nz + 1 if last else b  # last storage plane held
        sg = SlabGrid(g, z0, z1 - z0 - 1, r > 0, not last)
        shift = z0 * plane

        def own(flat: Any, lo: int = a, hi: int = b) -> npt.NDArray[np.bool_]:
            k = _plane_of(flat, plane)
            return (k >= lo) & (k < hi)

        walls = list(c.walls)
        if r > 0:
            walls[4] = "halo"
        if not last:
            walls[5] = "halo"
        corrections = []
        for k in c.pml.corrections:
            (x0, x1), (y0, y1), (zl, zh) = k.box
            lo, hi = max(zl, a), min(zh, b)
            if lo < hi:
                box = ((x0, x1), (y0, y1), (lo - z0, hi - z0))
                corrections.append(Correction(k.kind, k.c, k.a, k.b, k.sign, box))
        coeffs = {}
        for ax, co in c.pml.coeffs.items():
            if ax < 2:
                coeffs[ax] = co
            else:
                coeffs[ax] = AxisCoeffs(
                    *(np.array(getattr(co, f)[z0 : z1 + 1]) for f in ("eb", "ec", "ek", "hb", "hc", "hk"))
                )
        channels = []
        for ch in c.channels:
            flat = np.asarray(ch["flat"], dtype=np.int64)
            comps = np.broadcast_to(np.asarray(ch["comp"]), flat.shape)
            sel = own(flat)
            channels.append(
                {**ch, "flat": flat[sel] - shift, "comp": np.asarray(comps[sel]), "amps": np.asarray(ch["amps"])[sel]}
            )
        probes = []
        for p in c.probes:
            flat = np.asarray(p["flat"], dtype=np.int64)
            sel = own(flat)
            probes.append({**p, "flat": flat[sel] - shift, "weights": np.asarray(p["weights"])[sel]})
        ade = None
        if c.ade is not None:
            comp, flats, betas, cbes = [], [], [], []
            for cc, fl, be, cb in zip(c.ade.comp, c.ade.flat, c.ade.beta, c.ade.cbe, strict=True):
                sel = own(fl)
                comp.append(cc)
                flats.append(np.asarray(fl, dtype=np.int64)[sel] - shift)
                betas.append(np.asarray(be)[:, sel])
                cbes.append(np.asarray(cb)[sel])
            ade = AdeData(c.ade.kp, c.ade.tau, comp, flats, betas, cbes)
        sibc = None
        if c.sibc is not None:
            s = c.sibc
            sel = own(s.flat)
            hflat = np.asarray(s.hflat, dtype=np.int64)[sel]
            used = np.asarray(s.hsign)[sel] != 0
            hk = _plane_of(hflat, plane)
            if np.any(used & ((hk < z0) | (hk >= b))):
                raise ModelError("FDTD_BAD_DECOMPOSITION", "a surface-impedance edge samples H beyond its slab's halo")
            at_halo = used & (hk == z0) & (r > 0)
            if np.any(at_halo & ~np.isin(np.asarray(s.hcomp)[sel], (0, 1))):
                raise ModelError("FDTD_BAD_DECOMPOSITION", "a surface-impedance edge samples Hz on a slab halo")
            sibc = SibcData(
                comp=np.asarray(s.comp)[sel],
                flat=np.asarray(s.flat, dtype=np.int64)[sel] - shift,
                hcomp=np.asarray(s.hcomp)[sel],
                hflat=np.where(used, hflat - shift, 0),
                hsign=np.asarray(s.hsign)[sel],
                mat=np.asarray(s.mat)[sel],
                r0=s.r0,
                rp=s.rp,
                cp=s.cp,
                gp=s.gp,
            )
        sub = dataclasses.replace(
            c,
            grid=sg,  # type: ignore[arg-type]
            idx=[np.ascontiguousarray(i[z0 : z1 + 1]) for i in c.idx],
            walls=tuple(walls),
            pml=Pml(tuple(corrections), coeffs),
            channels=channels,
            probes=probes,
            ade=ade,
            sibc=sibc,
        )
        slabs.append(Slab(a, b, z0, sub))
    return slabs


def _sum_dicts(parts: Sequence[dict[str, Any]]) -> dict[str, Any]:
    out = {k: np.array(v, copy=True) for k, v in parts[0].items()}
    for d in parts[1:]:
        for k, v in d.items():
            out[k] = out[k] + v
    return out


def _plane_buffers(engine: Any, comps: Sequence[int], device: str = "cuda") -> dict[int, Any]:
    """One buffer per component for a plane of ``engine`` (its precision and shape), on
    ``device`` (the GPU; ``"cpu"`` only for the host tests of the exchange logic)."""
    import torch

    dtype = torch.float32 if engine.dtype == "float32" else torch.float64
    shape = (engine.B, engine.shape[2], engine.shape[3])
    return {comp: torch.empty(shape, dtype=dtype, device=device) for comp in comps}


class LocalSlabs:
    """Every rank's engine in this process; boundary planes copied between them. ``factory``
    builds an engine from a ``Compiled`` (for example ``lambda c: Gb300Engine(c, "float32")``);
    engines need ``half_h``, ``half_e``, ``plane``, ``set_plane`` and the engine protocol.
    ``device=True`` moves the planes device to device in the engines' own precision
    (``plane_to_device`` / ``plane_from_device``) instead of through host float64."""

    def __init__(self, c: Compiled, parts: int, factory: Callable[[Compiled], Any], device: bool = False) -> None:
        self.c = c
        self.slabs = split_z(c, parts)
        self.engines = [factory(s.c) for s in self.slabs]
        self.device = device
        self._buf = _plane_buffers(self.engines[0], (HX, HY, EX, EY)) if device else {}

    def _copy(self, comp: int, src: Any, k_src: int, dst: Any, k_dst: int) -> None:
        if self.device:
            buf = self._buf[comp]
            src.plane_to_device(comp, k_src, buf.data_ptr())
            dst.plane_from_device(comp, k_dst, buf.data_ptr())
        else:
            dst.set_plane(comp, k_dst, src.plane(comp, k_src))

    def step(self, n: int = 1) -> None:
        for _ in range(n):
            for e in self.engines:
                e.half_h()
            for r in range(len(self.slabs) - 1):  # H of the last owned plane up to the next slab
                s, e, nxt = self.slabs[r], self.engines[r], self.engines[r + 1]
                for comp in (HX, HY):
                    self._copy(comp, e, s.last_local, nxt, 0)
            for e in self.engines:
                e.half_e()
            for r in range(1, len(self.slabs)):  # E of the first owned plane down to the previous
                prev_s, prev, e = self.slabs[r - 1], self.engines[r - 1], self.engines[r]
                for comp in (EX, EY):
                    self._copy(comp, e, 1, prev, prev_s.b - prev_s.z0)

    def results(self) -> dict[str, Any]:
        return _sum_dicts([e.results() for e in self.engines])

    def series(self) -> dict[str, Any]:
        return _sum_dicts([e.series() for e in self.engines])

    def energy(self) -> float:
        return float(sum(e.energy() for e in self.engines))

    def field(self, comp: int) -> FloatArray:
        """One global component assembled from the owned planes (global ghost planes from the
        first and last slabs)."""
        g = self.c.grid
        out = np.zeros((self.c.batch, *g.shape))
        for r, (s, e) in enumerate(zip(self.slabs, self.engines, strict=True)):
            lo = 0 if r == 0 else s.a
            hi = g.shape[0] if r == len(self.slabs) - 1 else s.b
            for k in range(lo, hi):
                out[:, k] = e.plane(comp, k - s.z0)
        return out


class DistSlabs:
    """This process's rank of the decomposition; planes go to the neighbours through
    ``torch.distributed`` point-to-point messages, results are summed with ``all_reduce``.

    ``device=False``: host float64 tensors (any backend, ``gloo`` in the CPU tests).
    ``device=True``: device tensors in the engine's precision, copied device to device out of and
    into the engine (``plane_to_device`` / ``plane_from_device``), for the ``nccl`` backend with one
    GPU per rank (``torch.cuda.set_device`` and ``native.set_device`` to the local rank before the
    engine is built). The device mode needs two GPUs and is not run here."""

    def __init__(self, c: Compiled, factory: Callable[[Compiled], Any], device: bool = False,
                 buffer_device: str = "cuda") -> None:
        import torch.distributed as dist

        self.dist = dist
        self.rank, self.world = dist.get_rank(), dist.get_world_size()
        self.c = c
        self.slabs = split_z(c, self.world)
        self.slab = self.slabs[self.rank]
        self.engine = factory(self.slab.c)
        self.device = device
        self._on_gpu = buffer_device.startswith("cuda")
        if device:
            self._send = _plane_buffers(self.engine, (HX, HY, EX, EY), buffer_device)
            self._recv = _plane_buffers(self.engine, (HX, HY, EX, EY), buffer_device)

    def _swap_device(self, send_to: int | None, send: list[tuple[int, int]], recv_from: int | None,
                     recv: list[tuple[int, int]]) -> None:
        """Planes ``(comp, k)`` of this engine to ``send_to``; planes from ``recv_from`` into
        ``(comp, k)``: device buffers, one NCCL message each."""
        import torch

        e, ops = self.engine, []
        if send_to is not None:
            for comp, k in send:
                e.plane_to_device(comp, k, self._send[comp].data_ptr())  # finished on return
                ops.append(self.dist.P2POp(self.dist.isend, self._send[comp], send_to))
        if recv_from is not None:
            for comp, _ in recv:
                ops.append(self.dist.P2POp(self.dist.irecv, self._recv[comp], recv_from))
        if ops:
            for req in self.dist.batch_isend_irecv(ops):
                req.wait()
        if self._on_gpu:
            torch.cuda.synchronize()  # the received planes are complete before the engine reads them
        if recv_from is not None:
            for comp, k in recv:
                e.plane_from_device(comp, k, self._recv[comp].data_ptr())

    def _swap(self, send_to: int | None, send: list[FloatArray], recv_from: int | None, n_recv: int) -> list[FloatArray]:
        import torch

        shape = (self.c.batch, self.c.grid.shape[1], self.c.grid.shape[2])
        ops, bufs = [], []
        if send_to is not None:
            for a in send:
                ops.append(self.dist.P2POp(self.dist.isend, torch.from_numpy(np.ascontiguousarray(a)), send_to))
        if recv_from is not None:
            for _ in range(n_recv):
                t = torch.empty(shape, dtype=torch.float64)
                bufs.append(t)
                ops.append(self.dist.P2POp(self.dist.irecv, t, recv_from))
        if ops:
            for req in self.dist.batch_isend_irecv(ops):
                req.wait()
        return [t.numpy() for t in bufs]

    def step(self, n: int = 1) -> None:
        r, w, s, e = self.rank, self.world, self.slab, self.engine
        up = r + 1 if r + 1 < w else None
        down = r - 1 if r > 0 else None
        if self.device:
            for _ in range(n):
                e.half_h()
                self._swap_device(up, [(HX, s.last_local), (HY, s.last_local)], down, [(HX, 0), (HY, 0)])
                e.half_e()
                self._swap_device(down, [(EX, 1), (EY, 1)], up, [(EX, s.b - s.z0), (EY, s.b - s.z0)])
            return
        for _ in range(n):
            e.half_h()
            got = self._swap(up, [e.plane(HX, s.last_local), e.plane(HY, s.last_local)], down, 2)
            for comp, a in zip((HX, HY), got, strict=False):
                e.set_plane(comp, 0, a)
            e.half_e()
            got = self._swap(down, [e.plane(EX, 1), e.plane(EY, 1)], up, 2)
            for comp, a in zip((EX, EY), got, strict=False):
                e.set_plane(comp, s.b - s.z0, a)

    def _reduce(self, d: dict[str, Any]) -> dict[str, Any]:
        import torch

        out = {}
        for k in sorted(d):
            v = np.asarray(d[k])
            if np.iscomplexobj(v):
                t = torch.from_numpy(np.ascontiguousarray(np.stack([v.real, v.imag])))
                self.dist.all_reduce(t)
                out[k] = t[0].numpy() + 1j * t[1].numpy()
            else:
                t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64))
                self.dist.all_reduce(t)
                out[k] = t.numpy()
        return out

    def results(self) -> dict[str, Any]:
        return self._reduce(self.engine.results())

    def energy(self) -> float:
        import torch

        t = torch.tensor([float(self.engine.energy())], dtype=torch.float64)
        self.dist.all_reduce(t)
        return float(t.item())
