"""Quasi-TEM mode ports: the port plane's electrostatic modes and the per-edge port arrays.

Restates the reference's mode-port compiler (``packages/oa-fdtd/src/oa_fdtd/ports/modal.py``
``solve_modes :86-119``, ``ports/build.py`` ``solve_port_modes :94-162``,
``build_mode_port :165-244``) with the same numerical method, in code of its own:

* The plane's potential problem is solved with bilinear (Q1) finite elements on the port lattice
  refined at every physical conductor edge (lines graded by thirds towards each edge, where the
  static field is singular). Each element's stiffness is the tensor product of 1-D linear
  stiffness and mass matrices, scaled by the element's permittivity and aspect ratio. Nodes on a
  signal conductor are held at 1 V (one signal at a time), nodes on ground (other conductors,
  PEC regions, PEC walls) at 0 V, free boundary nodes are natural (PMC).
* The capacitance matrices with the dielectric (``C``) and in air (``C0``) give the modes
  (``C u = eps_eff C0 u``), their velocity and their impedance ``Z = 1 / (v u^T C u)``.
* The template of an in-plane E edge is minus the potential difference of its end nodes over its
  length (exact on the Yee edges, because the Q1 potential is linear along lattice lines). The
  port sheet's loading conductivity follows the edge permittivity, ``sigma_e = kappa max(eps_e,
  1)``, with ``kappa`` such that the sheet absorbs ``V^2 / Z``; the probe weights project the plane
  field on the same template, so ``V = V_s - Z I`` holds as for a lumped port.

The solve is setup-time host work (SciPy sparse LU); the engine sees only edge lists, loading
conductivities and probe weights, as for lumped ports.
"""

from __future__ import annotations

from dataclasses import dataclass, replace
from typing import Any

import numpy as np
import numpy.typing as npt
import scipy.linalg
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from open_analysis_gb300.grid import Grid

FloatArray = npt.NDArray[np.float64]
C_LIGHT = 299792458.0
EPS0_MODES = 8.8541878128e-12  # the permittivity constant of the mode solver [F/m]

# 1-D linear element on [0, 1]: stiffness and mass
_K1 = np.array([[1.0, -1.0], [-1.0, 1.0]])
_M1 = np.array([[2.0, 1.0], [1.0, 2.0]]) / 6.0
# element node order: (0, 0), (1, 0), (1, 1), (0, 1) in (u, v); index (a, b) of the tensor products
_ORDER = [(0, 0), (1, 0), (1, 1), (0, 1)]


def _tensor(ku: FloatArray, kv: FloatArray) -> FloatArray:
    out = np.empty((4, 4))
    for r, (ar, br) in enumerate(_ORDER):
        for c, (ac, bc) in enumerate(_ORDER):
            out[r, c] = ku[ar, ac] * kv[br, bc]
    return out


# d/du d/du integrated over the unit square, and d/dv d/dv
_SU = _tensor(_K1, _M1)
_SV = _tensor(_M1, _K1)


@dataclass
class ModeSet:
    """Modes of one port plane; ``phi`` is ``[mode, iu, iv]`` on the node lattice."""

    phi: FloatArray
    z: FloatArray
    eps_eff: FloatArray
    voltages: FloatArray
    cap: FloatArray
    cap_air: FloatArray


def stiffness(u: FloatArray, v: FloatArray, eps: FloatArray) -> sp.csr_matrix:
    """Q1 stiffness matrix on the lattice ``u x v`` (nodes flattened ``iu * (nv + 1) + iv``) with
    absolute permittivity ``eps (nu, nv)`` per element."""
    nu, nv = u.size - 1, v.size - 1
    hu, hv = np.diff(u), np.diff(v)
    iu, iv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    base = iu * (nv + 1) + iv
    corner = {(0, 0): base, (1, 0): base + (nv + 1), (1, 1): base + (nv + 1) + 1, (0, 1): base + 1}
    nodes = np.stack([corner[o] for o in _ORDER], axis=-1)
    su = (hv[None, :] / hu[:, None]) * eps
    sv = (hu[:, None] / hv[None, :]) * eps
    blocks = su[..., None, None] * _SU + sv[..., None, None] * _SV
    rows = np.broadcast_to(nodes[..., :, None], blocks.shape).ravel()
    cols = np.broadcast_to(nodes[..., None, :], blocks.shape).ravel()
    n = (nu + 1) * (nv + 1)
    return sp.csr_matrix((blocks.ravel(), (rows, cols)), shape=(n, n))


def _potentials(k: sp.csr_matrix, labels: npt.NDArray[np.int64], n_sig: int) -> tuple[FloatArray, FloatArray]:
    """Potential of each signal at 1 V (the others and ground at 0) and the capacitance matrix."""
    lab = labels.ravel()
    free = np.flatnonzero(lab < 0)
    held = np.flatnonzero(lab >= 0)
    phi = np.zeros((n_sig, lab.size))
    for s in range(n_sig):
        phi[s, lab == s + 1] = 1.0
    if free.size:
        kf = k[free]
        lu = spla.splu(kf[:, free].tocsc())
        kfh = kf[:, held]
        for s in range(n_sig):
            phi[s, free] = lu.solve(-(kfh @ phi[s, held]))
    kp = [k @ phi[s] for s in range(n_sig)]
    cap = np.array([[phi[a] @ kp[b] for b in range(n_sig)] for a in range(n_sig)])
    return phi.reshape((n_sig, *labels.shape)), cap


def solve_modes(u: FloatArray, v: FloatArray, eps_cell: FloatArray, labels: npt.NDArray[np.int64], n_sig: int) -> ModeSet:
    """Quasi-TEM modes of ``n_sig`` signal conductors on the lattice ``u x v``.

    ``eps_cell (nu, nv)`` relative permittivity; ``labels (nu + 1, nv + 1)``: -1 free, 0 ground,
    ``k`` signal ``k`` (1-based). Modes are ordered by effective permittivity; each voltage
    pattern is scaled to a largest magnitude of 1 with its first large entry positive."""
    if n_sig < 1:
        raise ValueError("a mode port needs at least one signal conductor")
    _, c_air = _potentials(stiffness(u, v, np.full_like(eps_cell, EPS0_MODES)), labels, n_sig)
    phi_s, c = _potentials(stiffness(u, v, eps_cell * EPS0_MODES), labels, n_sig)
    if n_sig == 1:
        pattern = np.ones((1, 1))
        eps_eff = np.array([c[0, 0] / c_air[0, 0]])
    else:
        w, vec = scipy.linalg.eigh(c, c_air)
        order = np.argsort(w)
        eps_eff, pattern = w[order], vec[:, order].T.copy()
        for m in range(n_sig):
            pattern[m] /= np.max(np.abs(pattern[m]))
            lead = pattern[m][int(np.argmax(np.abs(pattern[m]) > 0.5))]
            if lead < 0:
                pattern[m] = -pattern[m]
    speed = C_LIGHT / np.sqrt(eps_eff)
    z = np.array([1.0 / (speed[m] * (pattern[m] @ c @ pattern[m])) for m in range(eps_eff.size)])
    return ModeSet(np.tensordot(pattern, phi_s, axes=(1, 0)), z, eps_eff, pattern, c, c_air)


# ---------------------------------------------------------------------------------------- ports
def plane_index(g: Grid, axis: int, position: float) -> int:
    return int(np.argmin(np.abs(g.lines[axis] - position)))


def _box_nodes(cu: FloatArray, cv: FloatArray, lo: tuple[float, float], hi: tuple[float, float], tol: float) -> Any:
    inu = (cu >= lo[0] - tol) & (cu <= hi[0] + tol)
    inv = (cv >= lo[1] - tol) & (cv <= hi[1] + tol)
    return inu[:, None] & inv[None, :]


def _overlaps(lo: tuple[float, float], hi: tuple[float, float], box: Any, tol: float) -> bool:
    slo, shi = box
    return bool(lo[0] < shi[0] - tol and slo[0] < hi[0] - tol and lo[1] < shi[1] - tol and slo[1] < hi[1] - tol)


def physical_extent(g: Grid, cd: Any, tol: float) -> tuple[list[float], list[float]]:
    """A conductor box with its x and y faces moved out to the physical edge: a face on mesh line
    ``e`` goes to ``e + edge_frac (e' - e)``, ``e'`` the next line outward (not past the mesh)."""
    lo, hi = list(cd.lo), list(cd.hi)
    frac = float(getattr(cd, "edge_frac", 0.0))
    if frac <= 0.0:
        return lo, hi
    for a in (0, 1):
        lines = g.lines[a]
        for ext, step in ((lo, -1), (hi, 1)):
            i = int(np.argmin(np.abs(lines - ext[a])))
            if abs(lines[i] - ext[a]) <= tol and 0 <= i + step < lines.size:
                ext[a] = float(lines[i] + frac * (lines[i + step] - lines[i]))
    return lo, hi


def refine(base: FloatArray, extra: list[float], tol: float) -> tuple[FloatArray, npt.NDArray[np.intp]]:
    """``base`` plus every ``extra`` line strictly inside it, each graded by lines at ``h / 3^k``
    (k = 1..4) on both sides (``h``: its distance to the nearest base line, at most the smallest
    base spacing); returns the lines and where each base line lies in them."""
    inside = [x for x in extra if base[0] + tol < x < base[-1] - tol]
    grade = list(inside)
    for x in inside:
        away = np.abs(base - x)
        h = float(np.min(away[away > tol], initial=np.inf))
        if base.size > 1:
            h = min(h, float(np.min(np.diff(base))))
        for k in range(1, 5):
            grade += [x - h / 3.0**k, x + h / 3.0**k]
    new = [x for x in grade if base[0] + tol < x < base[-1] - tol and np.min(np.abs(base - x)) > tol]
    lines = np.unique(np.concatenate([base, np.asarray(new, dtype=np.float64)]))
    if lines.size > 1:
        lines = lines[np.concatenate([[True], np.diff(lines) > tol])]
    where = np.array([int(np.argmin(np.abs(lines - b))) for b in base], dtype=np.intp)
    return lines, where


def solve_port_modes(model: Any, g: Grid, port: Any, eps_cells: FloatArray) -> tuple[ModeSet, dict[str, Any]]:
    """Modes of a port's rectangle; ``eps_cells (nz, ny, nx)`` is the relative permittivity of
    the cells at the band centre."""
    n = port.axis
    ua, va = [a for a in range(3) if a != n]
    m = plane_index(g, n, port.position)
    tol = 1e-6 * float(min(np.min(g.d(a)) for a in range(3)))
    lu_, lv_ = g.lines[ua], g.lines[va]
    su = np.flatnonzero((lu_ >= port.lo[0] - tol) & (lu_ <= port.hi[0] + tol))
    sv = np.flatnonzero((lv_ >= port.lo[1] - tol) & (lv_ <= port.hi[1] + tol))
    if su.size < 2 or sv.size < 2:
        raise ValueError(f"mode port {port.name}: rectangle holds fewer than two lines per axis")
    u, v = lu_[su], lv_[sv]
    layer = min(max(m if port.direction > 0 else m - 1, 0), g.n[n] - 1)
    sel: list[Any] = [slice(None)] * 3
    sel[2 - n] = layer
    eps_plane = eps_cells[tuple(sel)].T[np.ix_(su[:-1], sv[:-1])]  # (iu, iv)
    pos = float(g.lines[n][m])
    boxes = [physical_extent(g, cd, tol) for cd in model.conductors if cd.lo[n] - tol <= pos <= cd.hi[n] + tol]
    boxes += [(list(r.lo), list(r.hi)) for r in model.regions if r.pec]
    extra_u = [b[k][ua] for b in boxes for k in (0, 1)] + [s[k][0] for s in port.signals for k in (0, 1)]
    extra_v = [b[k][va] for b in boxes for k in (0, 1)] + [s[k][1] for s in port.signals for k in (0, 1)]
    uu, iu = refine(u, extra_u, tol)
    vv, iv = refine(v, extra_v, tol)
    cu = np.clip(np.searchsorted(u, 0.5 * (uu[1:] + uu[:-1])) - 1, 0, u.size - 2)
    cv = np.clip(np.searchsorted(v, 0.5 * (vv[1:] + vv[:-1])) - 1, 0, v.size - 2)
    eps_fine = eps_plane[np.ix_(cu, cv)]
    labels = -np.ones((uu.size, vv.size), dtype=np.int64)
    joined: list[tuple[int, tuple[float, float], tuple[float, float]]] = []
    for lo, hi in boxes:
        if not lo[n] - tol <= pos <= hi[n] + tol:
            continue
        lo2, hi2 = (lo[ua], lo[va]), (hi[ua], hi[va])
        owner = next((k for k, s in enumerate(port.signals) if _overlaps(lo2, hi2, s, tol)), -1)
        if owner >= 0:
            joined.append((owner, lo2, hi2))  # part of that signal conductor, not ground
        else:
            labels[_box_nodes(uu, vv, lo2, hi2, tol)] = 0
    for a, lines, along in ((ua, uu, 0), (va, vv, 1)):
        for side in (0, 1):
            if model.walls[2 * a + side] != "pec":
                continue
            at = np.abs(lines - g.lines[a][0 if side == 0 else -1]) <= tol
            if along == 0:
                labels[at, :] = 0
            else:
                labels[:, at] = 0
    for k, (lo2, hi2) in enumerate(port.signals):
        labels[_box_nodes(uu, vv, lo2, hi2, tol)] = k + 1
    for k, lo2, hi2 in joined:
        labels[_box_nodes(uu, vv, lo2, hi2, tol)] = k + 1
    for k in range(len(port.signals)):
        if not np.any(labels[np.ix_(iu, iv)] == k + 1):
            raise ValueError(f"mode port {port.name}: signal {k} touches no node of the plane")
    full = solve_modes(uu, vv, eps_fine, labels, len(port.signals))
    return replace(full, phi=full.phi[:, iu][:, :, iv]), {"u_ax": ua, "v_ax": va, "plane": m, "su": su, "sv": sv}


def build_mode_port(g: Grid, port: Any, modes: ModeSet, geo: dict[str, Any], edge_eps: list[FloatArray]) -> dict[str, Any]:
    """Edge lists, template, loading conductivity and probe weights of one mode of ``port``."""
    if not 0 <= port.mode < modes.z.size:
        raise ValueError(f"mode port {port.name}: mode {port.mode} of {modes.z.size}")
    n, ua, va = port.axis, geo["u_ax"], geo["v_ax"]
    m, su, sv = geo["plane"], geo["su"], geo["sv"]
    phi = modes.phi[port.mode]
    z = float(modes.z[port.mode])
    pos = float(g.lines[n][m])
    lo3, hi3 = [0.0] * 3, [0.0] * 3
    lo3[n] = hi3[n] = pos
    lo3[ua], hi3[ua] = float(g.lines[ua][su[0]]), float(g.lines[ua][su[-1]])
    lo3[va], hi3[va] = float(g.lines[va][sv[0]]), float(g.lines[va][sv[-1]])
    comps, flats, tmpl, vol, eps_e = [], [], [], [], []
    for comp, other in ((ua, va), (va, ua)):
        flat, _ = g.points("E", comp, tuple(lo3), tuple(hi3))
        k, j, i = np.unravel_index(flat, g.shape)
        ijk = (i, j, k)
        cell, node = ijk[comp] - 1, ijk[other] - 1
        length = g.d(comp)[cell]
        c0 = su[0] if comp == ua else sv[0]
        n0 = sv[0] if comp == ua else su[0]
        cr, nr = cell - c0, node - n0
        dphi = (phi[cr + 1, nr] - phi[cr, nr]) if comp == ua else (phi[nr, cr + 1] - phi[nr, cr])
        tmpl.append(-dphi / length)
        vol.append(length * g.node_weights(other)[ijk[other]] * g.node_weights(n)[ijk[n]])
        eps_e.append(edge_eps[comp][k - 1, j - 1, i - 1])
        comps.append(np.full(flat.size, comp, np.int32))
        flats.append(flat)
    t_e = np.concatenate(tmpl)
    vol_e = np.concatenate(vol)
    s_e = np.maximum(np.concatenate(eps_e), 1.0)
    norm = float(np.sum(s_e * t_e**2 * vol_e))
    if norm <= 0:
        raise ValueError(f"mode port {port.name}: zero template (no field on the plane)")
    sigma = (1.0 / (z * norm)) * s_e
    return {
        "comp": np.concatenate(comps),
        "flat": np.concatenate(flats),
        "split": [f.size for f in flats],
        "sigma": sigma,
        "template": t_e,
        "weights": z * sigma * t_e * vol_e,
        "z": z,
        "eps_eff": float(modes.eps_eff[port.mode]),
        "voltages": modes.voltages[port.mode],
    }
