"""Compact fingerprints of compiled problems and engine states for the golden fixtures.

Large arrays are stored as SHA-256 digests of their bytes (bit-exact comparison) plus a few
float64 summary numbers (for a readable diff); small arrays are stored whole.
"""

from __future__ import annotations

import hashlib
from typing import Any

import numpy as np

SMALL = 4096  # arrays up to this many elements are stored whole


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _put(out: dict[str, Any], key: str, a: Any) -> None:
    a = np.asarray(a)
    out[key + ".sha"] = digest(a)
    out[key + ".dtype"] = str(a.dtype)
    out[key + ".shape"] = list(a.shape)
    if a.size <= SMALL:
        out[key] = a
    elif a.dtype.kind in "fc":
        out[key + ".l2"] = float(np.linalg.norm(a.astype(np.complex128 if a.dtype.kind == "c" else np.float64)))


def compiled_fingerprint(c: Any) -> dict[str, Any]:
    """Everything the engine consumes, fingerprinted."""
    out: dict[str, Any] = {"dt": np.float64(c.dt), "batch": c.batch}
    for ci, a in enumerate(c.idx):
        _put(out, f"idx{ci}", a)
    for name in ("eps_tab", "sig_tab", "ca_tab", "cb_tab", "drive", "frequencies"):
        _put(out, name, getattr(c, name))
    out["walls"] = list(c.walls)
    out["corrections"] = [
        [k.kind, k.c, k.a, k.b, k.sign, [list(r) for r in k.box]] for k in c.pml.corrections
    ]
    for ax, co in sorted(c.pml.coeffs.items()):
        for name in ("eb", "ec", "ek", "hb", "hc", "hk"):
            _put(out, f"pml{ax}.{name}", getattr(co, name))
    for i, ch in enumerate(c.channels):
        _put(out, f"ch{i}.comp", np.asarray(ch["comp"]))
        _put(out, f"ch{i}.flat", np.asarray(ch["flat"], dtype=np.int64))
        _put(out, f"ch{i}.amps", np.asarray(ch["amps"], dtype=np.float64))
    for i, p in enumerate(c.probes):
        out[f"probe{i}.meta"] = [p["name"], p["kind"], int(p["comp"])]
        _put(out, f"probe{i}.flat", np.asarray(p["flat"], dtype=np.int64))
        _put(out, f"probe{i}.weights", np.asarray(p["weights"], dtype=np.float64))
    if c.ade is not None:
        a = c.ade
        _put(out, "ade.kp", a.kp)
        _put(out, "ade.tau", a.tau)
        out["ade.comp"] = list(a.comp)
        for n, (fl, be, cbe) in enumerate(zip(a.flat, a.beta, a.cbe, strict=True)):
            _put(out, f"ade{n}.flat", np.asarray(fl, dtype=np.int64))
            _put(out, f"ade{n}.beta", be)
            _put(out, f"ade{n}.cbe", cbe)
    for i, q in enumerate(c.ports):
        if "sig_e" in q:  # mode port: impedance, loading and template
            out[f"port{i}.z"] = np.float64(q["r_ohm"])
            out[f"port{i}.eps_eff"] = np.float64(q["eps_eff"])
            _put(out, f"port{i}.sig_e", np.asarray(q["sig_e"], dtype=np.float64))
            _put(out, f"port{i}.e_t", np.asarray(q["e_t"], dtype=np.float64))
            out[f"port{i}.parts"] = list(q["probe_parts"])
    for name, parts in sorted(getattr(c, "probe_sums", {}).items()):
        out[f"sum.{name}"] = list(parts)
    if c.sibc is not None:
        s = c.sibc
        for name in ("comp", "flat", "hcomp", "hflat", "hsign", "mat", "r0", "rp", "cp", "gp"):
            _put(out, f"sibc.{name}", getattr(s, name))
    return out


def state_fingerprint(engine: Any) -> dict[str, Any]:
    """Fields (bit-exact digests of the engine's own precision), DFTs and energy."""
    out: dict[str, Any] = {"energy": np.float64(engine.energy())}
    for name, arr in zip(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"), (*engine.E, *engine.H), strict=True):
        _put(out, f"field.{name}", arr)
        out[f"field.{name}.l2"] = float(np.linalg.norm(arr.astype(np.float64)))
    for name, v in engine.results().items():
        out[f"dft.{name}"] = np.asarray(v, dtype=np.complex128)
    return out


def compare_compiled(ref: dict[str, Any], mine: dict[str, Any]) -> list[str]:
    """Keys whose values differ (bit for bit), as messages."""
    bad = []
    for key, v in ref.items():
        if key not in mine:
            bad.append(f"missing {key}")
            continue
        w = mine[key]
        if isinstance(v, np.ndarray) and v.dtype.kind in "fciub":
            wv = np.asarray(w)
            if wv.shape != v.shape or not np.array_equal(wv, v):
                bad.append(f"{key} differs")
        elif key.endswith(".l2"):
            if not np.isclose(float(v), float(w), rtol=1e-12, atol=0.0):
                bad.append(f"{key}: {v} vs {w}")
        elif isinstance(v, (float, np.floating)):
            if float(v) != float(w):
                bad.append(f"{key}: {v!r} vs {w!r}")
        elif _plain(v) != _plain(w):
            bad.append(f"{key}: {v!r} vs {w!r}")
    return bad


def _plain(v: Any) -> Any:
    if isinstance(v, np.ndarray):
        return v.tolist()
    if isinstance(v, (list, tuple)):
        return [_plain(x) for x in v]
    if isinstance(v, np.generic):
        return v.item()
    return v


def save(path: str, data: dict[str, Any]) -> None:
    """Store a fingerprint as ``.npz`` (arrays) with JSON-able metadata in ``__meta__``."""
    import json

    arrays = {k: v for k, v in data.items() if isinstance(v, np.ndarray)}
    meta = {k: _plain(v) for k, v in data.items() if not isinstance(v, np.ndarray)}
    np.savez_compressed(path, __meta__=np.array(json.dumps(meta)), **arrays)


def load(path: str) -> dict[str, Any]:
    import json

    with np.load(path, allow_pickle=False) as z:
        out: dict[str, Any] = json.loads(str(z["__meta__"]))
        for k in z.files:
            if k != "__meta__":
                out[k] = z[k]
    return out
