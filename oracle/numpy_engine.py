"""CPU oracle: the reference's NumPy leapfrog engine, restated.

TEST INFRASTRUCTURE ONLY. Nothing in the product (``open_analysis_gb300``) imports this module;
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` use it, as
the checker and as the timed CPU baseline. It is never a fallback for the GPU engine.

It follows ``packages/oa-fdtd/src/oa_fdtd/reference.py`` (``NumpyEngine :41-331``) operation by
operation, in the same floating-point order, so that a float32 run reproduces the reference's
float32 fields bit for bit and a float64 run is the FP64 error yardstick:

* step order ``reference.py:251-266``: H update, CPML-H, PMC ghosts, record H at (n+1/2) dt,
  ADE save, E update, CPML-E, SIBC, injection at (n+1/2) dt, ADE update, record E at (n+1) dt;
* H update ``:152-165``; E update ``:167-180``; CPML ``:182-207``; ghosts ``:209-221``;
* injection ``:223-234``; probes and running DFT ``:236-249``;
* ADE ``:115-127``; SIBC ``:129-150``; energy ``:269-280``; results/series ``:312-328``.

Its agreement with the reference itself is pinned by ``tests/golden`` (fixtures generated by
importing the reference; see ``tests/golden/make_golden.py``).

``pole_sum="loop"`` sums the Debye poles in a plain loop in index order, the order the GPU engine
uses; the reference's ``np.einsum`` (the default here) may reorder or fuse that sum on some hosts,
which changes the rounding of multi-pole runs only.
"""

from __future__ import annotations

from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.grid import EPS0, MU0
from open_analysis_gb300.pml import E_TERMS, H_TERMS

FloatArray = npt.NDArray[np.float64]
Rng = tuple[tuple[int, int], ...]


def _window(f: Any, rng: Rng, axis: int = -1, shift: int = 0) -> Any:
    """View of a ``(B, z, y, x)`` array over per-axis ranges ``rng`` (x, y, z), shifted by
    ``shift`` along ``axis``."""
    parts = [slice(None)]
    for a in (2, 1, 0):
        lo, hi = rng[a]
        s = shift if a == axis else 0
        parts.append(slice(lo + s, hi + s))
    return f[tuple(parts)]


def _coef(arr: FloatArray, axis: int, rng: Rng) -> FloatArray:
    lo, hi = rng[axis]
    shape = [1, 1, 1, 1]
    shape[3 - axis] = hi - lo
    return arr[lo:hi].reshape(shape)


class OracleEngine:
    """Engine protocol (``step/energy/results/series/peak_bytes/get_fields``) on the CPU."""

    name = "oracle"

    def __init__(
        self, c: Any, dtype: str = "float64", record_series: bool = False, pole_sum: str = "einsum", **_: Any
    ) -> None:
        if pole_sum not in ("einsum", "loop"):
            raise ValueError(f"pole_sum must be 'einsum' or 'loop', not {pole_sum!r}")
        self.pole_sum = pole_sum
        self.c = c
        self.record_series = record_series
        self.dtype = np.dtype(dtype)
        real = self.dtype
        g = c.grid
        batch = c.batch
        shape = (batch, *g.shape)
        self.E = [np.zeros(shape, real) for _ in range(3)]
        self.H = [np.zeros(shape, real) for _ in range(3)]
        self.ca = [c.ca_tab[m][None].astype(real) for m in c.idx]
        self.cb = [c.cb_tab[m][None].astype(real) for m in c.idx]
        self.dtmu = real.type(c.dt / MU0)
        self.ip = [g.inv_primal(a).astype(real) for a in range(3)]
        self.idd = [g.inv_dual(a).astype(real) for a in range(3)]
        self.full: Rng = tuple((1, g.n[a] + 2) for a in range(3))
        self.psi = [np.zeros((batch, *corr.shape), real) for corr in c.pml.corrections]
        self.pmc = [(a, s) for a in range(3) for s in (0, 1) if c.walls[2 * a + s] == "pmc"]
        self.step_count = 0
        self.probes_e = [p for p in c.probes if p["kind"] == "E"]
        self.probes_h = [p for p in c.probes if p["kind"] == "H"]
        nf = c.frequencies.size
        self.acc = {
            "E": np.zeros((nf, batch, len(self.probes_e)), np.complex128),
            "H": np.zeros((nf, batch, len(self.probes_h)), np.complex128),
        }
        self._series: dict[str, list[FloatArray]] = {"E": [], "H": []}
        self.omega = 2.0 * np.pi * c.frequencies
        self._setup_ade()
        self._setup_sibc()

    # ------------------------------------------------------------------ physics state
    def _flat(self, comp: int) -> Any:
        return self.E[comp].reshape(self.c.batch, -1)

    def _setup_ade(self) -> None:
        c, real, batch = self.c, self.dtype, self.c.batch
        self._ade: list[dict[str, Any]] = []
        if c.ade is None:
            return
        a = c.ade
        for comp, flat, beta, cbe in zip(a.comp, a.flat, a.beta, a.cbe, strict=True):
            self._ade.append(
                {
                    "c": comp,
                    "flat": flat,
                    "beta": beta.astype(real),
                    "cbe": cbe.astype(real),
                    "J": np.zeros((a.tau.size, batch, flat.size), real),
                    "eold": np.zeros((batch, flat.size), real),
                }
            )
        self._kp = a.kp.astype(real)

    def _setup_sibc(self) -> None:
        c, real, batch = self.c, self.dtype, self.c.batch
        self._sb = c.sibc
        if self._sb is None:
            return
        sb = self._sb
        ne = sb.flat.size
        self._sb_j = np.zeros((batch, ne), real)
        self._sb_v = np.zeros((sb.cp.size, batch, ne), real)
        self._sb_h = [
            [(hc, np.flatnonzero((sb.hcomp[:, s] == hc) & (sb.hsign[:, s] != 0))) for hc in range(3)]
            for s in range(2)
        ]
        self._sb_e = [np.flatnonzero(sb.comp == comp) for comp in range(3)]
        self._sb_alpha = (sb.rp[sb.mat] * sb.cp[None, :]).astype(real)  # (ne, P)

    def _ade_save(self) -> None:
        for st in self._ade:
            st["eold"][...] = self._flat(st["c"])[:, st["flat"]]

    def _ade_update(self) -> None:
        for st in self._ade:
            ef = self._flat(st["c"])
            e = ef[:, st["flat"]]
            if self.pole_sum == "loop":
                onekp = (1.0 + self._kp).astype(self.dtype)
                acc = np.zeros_like(e)
                for p in range(st["J"].shape[0]):
                    acc = acc + onekp[p] * st["J"][p]
                jt = 0.5 * acc
            else:
                jt = 0.5 * np.einsum("p,pbe->be", 1.0 + self._kp, st["J"])
            en = e - st["cbe"][None, :] * jt
            de = en - st["eold"]
            st["J"][...] = self._kp[:, None, None] * st["J"] + st["beta"][:, None, :] * de[None]
            ef[:, st["flat"]] = en

    def _sibc(self) -> None:
        sb = self._sb
        if sb is None:
            return
        batch = self.c.batch
        j = np.zeros((batch, sb.flat.size), self.dtype)
        for s in range(2):
            for hc, ids in self._sb_h[s]:
                if ids.size:
                    hf = self.H[hc].reshape(batch, -1)
                    sg = sb.hsign[ids, s].astype(self.dtype)[None, :]
                    j[:, ids] += sg * hf[:, sb.hflat[ids, s]]
        dj = j - self._sb_j
        gp = sb.gp.astype(self.dtype)[:, None, None]
        self._sb_v[...] = self._sb_alpha.T[:, None, :] * dj[None] + gp * self._sb_v
        out = sb.r0[sb.mat].astype(self.dtype)[None, :] * j + self._sb_v.sum(axis=0)
        self._sb_j = j
        for comp in range(3):
            ids = self._sb_e[comp]
            if ids.size:
                self._flat(comp)[:, sb.flat[ids]] = out[:, ids]

    # ------------------------------------------------------------------ Yee updates
    def _h_update(self) -> None:
        g = self.c.grid
        for comp in range(3):
            rng = g.valid("H", comp)
            acc = None
            for c_, a, b_, sign in H_TERMS:
                if c_ != comp:
                    continue
                d = (_window(self.E[b_], rng, a, 1) - _window(self.E[b_], rng)) * _coef(
                    self.ip[a], a, rng
                )
                term = d if sign > 0 else -d
                acc = term if acc is None else acc + term
            _window(self.H[comp], rng)[...] += self.dtmu * acc

    def _e_update(self) -> None:
        rng = self.full
        for comp in range(3):
            acc = None
            for c_, a, b_, sign in E_TERMS:
                if c_ != comp:
                    continue
                d = (_window(self.H[b_], rng) - _window(self.H[b_], rng, a, -1)) * _coef(
                    self.idd[a], a, rng
                )
                term = d if sign > 0 else -d
                acc = term if acc is None else acc + term
            e = _window(self.E[comp], rng)
            e[...] = _window(self.ca[comp], rng) * e + _window(self.cb[comp], rng) * acc

    def _pml(self, kind: str) -> None:
        c = self.c
        real = self.dtype
        for corr, psi in zip(c.pml.corrections, self.psi, strict=True):
            if corr.kind != kind:
                continue
            co = c.pml.coeffs[corr.a]
            rng = corr.box
            a = corr.a
            if kind == "E":
                d = (_window(self.H[corr.b], rng) - _window(self.H[corr.b], rng, a, -1)) * _coef(
                    self.idd[a], a, rng
                )
                cb_, cc_, ck_ = co.eb, co.ec, co.ek
            else:
                d = (_window(self.E[corr.b], rng, a, 1) - _window(self.E[corr.b], rng)) * _coef(
                    self.ip[a], a, rng
                )
                cb_, cc_, ck_ = co.hb, co.hc, co.hk
            psi *= _coef(cb_.astype(real), a, rng)
            psi += _coef(cc_.astype(real), a, rng) * d
            upd = _coef(ck_.astype(real), a, rng) * d + psi
            if kind == "E":
                _window(self.E[corr.c], rng)[...] += corr.sign * _window(self.cb[corr.c], rng) * upd
            else:
                _window(self.H[corr.c], rng)[...] += corr.sign * self.dtmu * upd

    def _ghosts(self) -> None:
        g = self.c.grid
        for a, s in self.pmc:
            dst, src = (0, 1) if s == 0 else (g.n[a] + 1, g.n[a])
            for comp in range(3):
                if comp == a:
                    continue
                h = self.H[comp]
                d_sel: list[Any] = [slice(None)] * 4
                s_sel: list[Any] = [slice(None)] * 4
                d_sel[3 - a], s_sel[3 - a] = dst, src
                h[tuple(d_sel)] = -h[tuple(s_sel)]

    def _inject(self, step: int) -> None:
        c = self.c
        for ci, ch in enumerate(c.channels):
            w = float(ch["waveform"](np.array([(step + 0.5) * c.dt]))[0])
            comps = np.broadcast_to(np.asarray(ch["comp"]), ch["flat"].shape)
            for cc in np.unique(comps):
                sel = comps == cc
                f = self.E[int(cc)].reshape(c.batch, -1)
                amps = ch["amps"][sel]
                f[:, ch["flat"][sel]] += ((c.drive[:, ci : ci + 1] * w) * amps[None, :]).astype(
                    self.dtype
                )

    def _record(self, kind: str, t: float) -> None:
        probes = self.probes_e if kind == "E" else self.probes_h
        if not probes:
            return
        arrs = self.E if kind == "E" else self.H
        batch = self.c.batch
        vals = np.empty((batch, len(probes)))
        for pi, p in enumerate(probes):
            f = arrs[p["comp"]].reshape(batch, -1)
            vals[:, pi] = (f[:, p["flat"]].astype(np.float64) * p["weights"][None, :]).sum(axis=1)
        if self.record_series:
            self._series[kind].append(vals)
        ph = np.exp(-1j * self.omega * t) * self.c.dt
        self.acc[kind] += ph[:, None, None] * vals[None, :, :]

    def step(self, n: int = 1) -> None:
        for _ in range(n):
            self.half_h()
            self.half_e()

    def half_h(self) -> None:
        """First half of a step: H update, CPML-H, PMC ghosts, H probes at (n + 1/2) dt."""
        k = self.step_count
        self._h_update()
        self._pml("H")
        self._ghosts()
        self._record("H", (k + 0.5) * self.c.dt)

    def half_e(self) -> None:
        """Second half: ADE save, E update, CPML-E, SIBC, injection at (n + 1/2) dt, ADE update,
        E probes at (n + 1) dt."""
        k = self.step_count
        self._ade_save()
        self._e_update()
        self._pml("E")
        self._sibc()
        self._inject(k)
        self._ade_update()
        self._record("E", (k + 1) * self.c.dt)
        self.step_count += 1

    def plane(self, comp: int, k: int) -> FloatArray:
        """Component ``comp`` (0..5 = Ex..Hz) at storage plane ``k``, shape (B, y, x)."""
        return (self.E + self.H)[comp][:, k].astype(np.float64)

    def set_plane(self, comp: int, k: int, values: FloatArray) -> None:
        (self.E + self.H)[comp][:, k] = values

    # ------------------------------------------------------------------ observables
    def _weights(self, kind: str, comp: int) -> FloatArray:
        g = self.c.grid
        out = np.ones((1, 1, 1, 1))
        for a in range(3):
            node = (a != comp) if kind == "E" else (a == comp)
            w = g.node_weights(a) if node else g.cell_weights(a)
            shape = [1, 1, 1, 1]
            shape[3 - a] = w.size
            out = out * w.reshape(shape)
        return out

    def energy(self) -> float:
        """``1/2 sum eps E^2 V + 1/2 mu0 sum H^2 V`` [J] in float64."""
        c = self.c
        total = 0.0
        for comp in range(3):
            eps = (c.eps_tab[c.idx[comp]] * EPS0)[None]
            total += 0.5 * float(
                np.sum(eps * self._weights("E", comp) * self.E[comp].astype(np.float64) ** 2)
            )
            total += 0.5 * MU0 * float(
                np.sum(self._weights("H", comp) * self.H[comp].astype(np.float64) ** 2)
            )
        return total

    def get_fields(self) -> dict[str, FloatArray]:
        names = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
        return {n: a.astype(np.float64) for n, a in zip(names, (*self.E, *self.H), strict=True)}

    def results(self) -> dict[str, FloatArray]:
        out: dict[str, FloatArray] = {}
        for kind, probes in (("E", self.probes_e), ("H", self.probes_h)):
            for pi, p in enumerate(probes):
                out[p["name"]] = self.acc[kind][:, :, pi].T.copy()
        return out

    def series(self) -> dict[str, FloatArray]:
        out: dict[str, FloatArray] = {}
        for kind, probes in (("E", self.probes_e), ("H", self.probes_h)):
            if probes and self._series[kind]:
                arr = np.stack(self._series[kind], axis=-1)
                for pi, p in enumerate(probes):
                    out[p["name"]] = arr[:, pi, :]
        return out

    def peak_bytes(self) -> int:
        return 0
