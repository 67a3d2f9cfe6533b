"""Touchstone files of S-parameters: v1.1 for one real reference impedance, v2.0 otherwise.

The format the reference's FDTD adapter writes (``packages/oa-fdtd/src/oa_fdtd/adapter/
touchstone.py:21-79``), kept identical so its readers take these files unchanged: real and
imaginary parts ("RI") to 12 significant digits, frequencies in Hz, port names in
``! Port[n] = name`` comments; two-port data in the order S11 S21 S12 S22 (v2.0 states it as
``[Two-Port Data Order] 21_12``), larger matrices row by row, four pairs per line.
"""

from __future__ import annotations

from collections.abc import Sequence
from pathlib import Path

import numpy as np
import numpy.typing as npt

ComplexArray = npt.NDArray[np.complex128]
FloatArray = npt.NDArray[np.float64]


def _ri(z: complex) -> str:
    return f"{z.real:.12e} {z.imag:.12e}"


def _entries(n: int) -> list[tuple[int, int]]:
    if n == 2:
        return [(0, 0), (1, 0), (0, 1), (1, 1)]
    return [(i, j) for i in range(n) for j in range(n)]


def format_touchstone(
    freqs: FloatArray, s: ComplexArray, z0: Sequence[float], names: Sequence[str], comments: Sequence[str] = ()
) -> str:
    """Touchstone text of ``s`` with shape ``(F, N, N)`` at ``freqs`` [Hz]."""
    n = s.shape[1]
    out = [f"! {c}" for c in comments]
    out += [f"! Port[{i + 1}] = {name}" for i, name in enumerate(names)]
    one_reference = len({float(z) for z in z0}) == 1
    if one_reference:
        out.append(f"# HZ S RI R {float(z0[0]):.12g}")
    else:
        out += ["[Version] 2.0", "# HZ S RI R 50", f"[Number of Ports] {n}"]
        if n == 2:
            out.append("[Two-Port Data Order] 21_12")
        out += [
            f"[Number of Frequencies] {len(freqs)}",
            "[Reference] " + " ".join(f"{float(z):.12g}" for z in z0),
            "[Matrix Format] Full",
            "[Network Data]",
        ]
    order = _entries(n)
    for k, f in enumerate(freqs):
        pairs = [_ri(complex(s[k, i, j])) for i, j in order]
        if n <= 2:
            out.append(f"{float(f):.12e} " + " ".join(pairs))
            continue
        for row in range(n):
            cells = pairs[row * n : (row + 1) * n]
            for c in range(0, len(cells), 4):
                lead = f"{float(f):.12e} " if row == 0 and c == 0 else "  "
                out.append(lead + " ".join(cells[c : c + 4]))
    if not one_reference:
        out.append("[End]")
    return "\n".join(out) + "\n"


def write_touchstone(
    path: Path, freqs: FloatArray, s: ComplexArray, z0: Sequence[float], names: Sequence[str], comments: Sequence[str] = ()
) -> None:
    Path(path).write_text(format_touchstone(freqs, s, z0, names, comments), encoding="utf-8")
