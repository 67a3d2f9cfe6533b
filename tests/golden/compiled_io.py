"""A compiled problem (the reference's ``Compiled``, ``oa_fdtd/model.py:246-269``) saved as plain
arrays and loaded back as an object with the same attributes, so that a problem compiled by the
reference can be fed to ``Gb300Engine`` on a host without the reference.

Everything the engine reads is stored as the reference computed it: the grid's lines and its
one-dimensional metrics (``inv_primal``, ``inv_dual``, ``node_weights``, ``cell_weights``, from the
reference's ``Grid``), the material index arrays and tables, walls, CPML corrections and
coefficients, channels with their waveform sampled at ``(n + 1/2) dt`` for the first ``steps``
steps, drive, probes, frequencies, the Debye and surface-impedance data. The loaded waveform
answers exactly those sample times.
"""

from __future__ import annotations

import json
from types import SimpleNamespace
from typing import Any

import numpy as np

AXES = range(3)
PML = ("eb", "ec", "ek", "hb", "hc", "hk")
SIBC = ("comp", "flat", "hcomp", "hflat", "hsign", "mat", "r0", "rp", "cp", "gp")


def dump(c: Any, steps: int) -> dict[str, Any]:
    """Arrays (and a JSON ``__meta__``) of a compiled problem."""
    g = c.grid
    out: dict[str, Any] = {}
    meta: dict[str, Any] = {"batch": int(c.batch), "walls": list(c.walls), "steps": int(steps)}
    out["dt"] = np.float64(c.dt)
    for a in AXES:
        out[f"grid.lines{a}"] = np.asarray(g.lines[a], np.float64)
        for f in ("inv_primal", "inv_dual", "node_weights", "cell_weights"):
            out[f"grid.{f}{a}"] = np.asarray(getattr(g, f)(a), np.float64)
    for ci in AXES:
        out[f"idx{ci}"] = np.asarray(c.idx[ci])
    for name in ("eps_tab", "sig_tab", "ca_tab", "cb_tab", "drive", "frequencies"):
        out[name] = np.asarray(getattr(c, name))
    meta["corrections"] = [[k.kind, int(k.c), int(k.a), int(k.b), float(k.sign), [list(map(int, r)) for r in k.box]]
                           for k in c.pml.corrections]
    meta["pml_axes"] = sorted(int(a) for a in c.pml.coeffs)
    for a, co in c.pml.coeffs.items():
        for name in PML:
            out[f"pml{a}.{name}"] = np.asarray(getattr(co, name), np.float64)
    t = (np.arange(steps) + 0.5) * c.dt
    meta["channels"] = len(c.channels)
    for i, ch in enumerate(c.channels):
        out[f"ch{i}.comp"] = np.asarray(ch["comp"])
        out[f"ch{i}.flat"] = np.asarray(ch["flat"], np.int64)
        out[f"ch{i}.amps"] = np.asarray(ch["amps"], np.float64)
        out[f"ch{i}.wave"] = np.array([float(ch["waveform"](np.array([tn]))[0]) for tn in t])
    meta["probes"] = [[q["name"], q["kind"], int(q["comp"])] for q in c.probes]
    for i, q in enumerate(c.probes):
        out[f"probe{i}.flat"] = np.asarray(q["flat"], np.int64)
        out[f"probe{i}.weights"] = np.asarray(q["weights"], np.float64)
    meta["ade"] = c.ade is not None
    if c.ade is not None:
        a = c.ade
        out["ade.tau"], out["ade.kp"] = np.asarray(a.tau), np.asarray(a.kp)
        meta["ade_comp"] = [int(v) for v in a.comp]
        for n, (fl, be, cbe) in enumerate(zip(a.flat, a.beta, a.cbe, strict=True)):
            out[f"ade{n}.flat"], out[f"ade{n}.beta"], out[f"ade{n}.cbe"] = np.asarray(fl), np.asarray(be), np.asarray(cbe)
    meta["sibc"] = c.sibc is not None
    if c.sibc is not None:
        for name in SIBC:
            out[f"sibc.{name}"] = np.asarray(getattr(c.sibc, name))
    out["__meta__"] = np.array(json.dumps(meta))
    return out


class StoredGrid:
    """The reference grid's shape and metrics as stored."""

    def __init__(self, z: Any) -> None:
        self.lines = tuple(z[f"grid.lines{a}"] for a in AXES)
        self.n = tuple(int(v.size - 1) for v in self.lines)
        self._m = {f: [z[f"grid.{f}{a}"] for a in AXES] for f in ("inv_primal", "inv_dual", "node_weights", "cell_weights")}
        self.pitch = int(self._m["inv_primal"][0].size)
        self.shape = (self.n[2] + 2, self.n[1] + 2, self.pitch)
        self.cells = self.n[0] * self.n[1] * self.n[2]

    def inv_primal(self, a: int) -> np.ndarray:
        return self._m["inv_primal"][a]

    def inv_dual(self, a: int) -> np.ndarray:
        return self._m["inv_dual"][a]

    def node_weights(self, a: int) -> np.ndarray:
        return self._m["node_weights"][a]

    def cell_weights(self, a: int) -> np.ndarray:
        return self._m["cell_weights"][a]


class SampledWave:
    """A waveform known at the times ``(n + 1/2) dt``, n < len(table)."""

    def __init__(self, table: np.ndarray, dt: float) -> None:
        self.table, self.dt = table, dt

    def __call__(self, t: Any) -> np.ndarray:
        n = np.rint(np.asarray(t, np.float64) / self.dt - 0.5).astype(np.int64)
        if n.size and (n.min() < 0 or n.max() >= self.table.size):
            raise ValueError("the stored waveform covers the first %d steps only" % self.table.size)
        return self.table[n]


def load(path: str) -> SimpleNamespace:
    """The stored problem with the attributes ``Gb300Engine`` reads from a ``Compiled``."""
    with np.load(path, allow_pickle=False) as f:
        z = {k: f[k] for k in f.files}
    meta = json.loads(str(z["__meta__"]))
    dt = float(z["dt"])
    corr = [SimpleNamespace(kind=k[0], c=k[1], a=k[2], b=k[3], sign=k[4], box=tuple(tuple(r) for r in k[5]))
            for k in meta["corrections"]]
    coeffs = {a: SimpleNamespace(**{n: z[f"pml{a}.{n}"] for n in PML}) for a in meta["pml_axes"]}
    chans = [{"comp": z[f"ch{i}.comp"], "flat": z[f"ch{i}.flat"], "amps": z[f"ch{i}.amps"],
              "waveform": SampledWave(z[f"ch{i}.wave"], dt)} for i in range(meta["channels"])]
    probes = [{"name": p[0], "kind": p[1], "comp": p[2], "flat": z[f"probe{i}.flat"], "weights": z[f"probe{i}.weights"]}
              for i, p in enumerate(meta["probes"])]
    ade = None
    if meta["ade"]:
        comp = meta["ade_comp"]
        ade = SimpleNamespace(tau=z["ade.tau"], kp=z["ade.kp"], comp=comp,
                              flat=[z[f"ade{n}.flat"] for n in range(len(comp))],
                              beta=[z[f"ade{n}.beta"] for n in range(len(comp))],
                              cbe=[z[f"ade{n}.cbe"] for n in range(len(comp))])
    sibc = SimpleNamespace(**{n: z[f"sibc.{n}"] for n in SIBC}) if meta["sibc"] else None
    return SimpleNamespace(
        grid=StoredGrid(z), dt=dt, batch=meta["batch"], idx=[z[f"idx{c}"] for c in AXES],
        eps_tab=z["eps_tab"], sig_tab=z["sig_tab"], ca_tab=z["ca_tab"], cb_tab=z["cb_tab"], drive=z["drive"],
        frequencies=z["frequencies"], walls=tuple(meta["walls"]), pml=SimpleNamespace(corrections=corr, coeffs=coeffs),
        channels=chans, probes=probes, ade=ade, sibc=sibc, steps=meta["steps"],
    )
