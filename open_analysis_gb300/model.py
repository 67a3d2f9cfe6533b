"""Engine-level problem description and the model compiler.

Mirrors ``packages/oa-fdtd/src/oa_fdtd/model.py``: the problem types (``Waveform :37-64``,
``Region :68-77``, ``Conductor :80-97``, ``LumpedPort :101-109``, ``ModePort :113-131``,
``SoftSource :135-142``, ``Probe :146-154``, ``Model :158-214``), the compiled arrays
(``AdeData :218-226``, ``SibcData :230-242``, ``Compiled :246-269``) and ``compile_model``
(``:501-768``). The compiled arrays are the engine's input contract, so the compiler reproduces
the reference's arrays exactly: the per-edge material average, the uint16 index into the table of
averaged (eps, sigma) pairs with 0 reserved for PEC, ``ca/cb`` from that table, the Debye ADE and
surface-impedance edge lists, the port, source and probe lists. The floating-point operation
order of the averaging and of the table keys follows the reference so that the tables agree bit
for bit (the fixtures under ``tests/golden`` pin this).

Materials are never stored per cell on the device: every E edge carries a uint16 index into the
table, and the kernels rebuild ``ca, cb`` from it.

Two implementations of the volume stages (per-cell materials, edge averages, the table and
index, the Debye edge lists) give the same arrays bit for bit: NumPy (``native=False``, the
reference's stages restated) and the engine library's native compiler (``native=True``,
``oafdtd_materials_build``: host threads, one uint16 region id per cell instead of float64
volumes). ``compile_model`` uses the native one when the library is built.
"""

from __future__ import annotations

import math
from collections.abc import Callable
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300.grid import EPS0, Grid
from open_analysis_gb300.pml import CpmlSpec, Pml, build_pml
from open_analysis_gb300.sibc import SibcFit, classify_box, fit_surface_impedance, outside_samples

FloatArray = npt.NDArray[np.float64]
WALL_KINDS = ("pec", "pmc", "cpml")
MAX_TABLE = 65535


class ModelError(ValueError):
    """Bad problem description; ``code`` is a stable ``FDTD_*`` identifier."""

    def __init__(self, code: str, message: str, hint: str = "") -> None:
        super().__init__(f"{code}: {message}")
        self.code, self.message, self.hint = code, message, hint


@dataclass(frozen=True)
class Waveform:
    """Excitation ``s(t)``: ``"gauss_mod"`` (modulated Gaussian, no DC) or ``"gauss"``.

    ``bandwidth`` is the -20 dB full width (gauss_mod) or the highest frequency (gauss);
    the pulse is centred ``delay_tau`` widths after t = 0.
    """

    kind: str = "gauss_mod"
    f0: float = 0.0
    bandwidth: float = 0.0
    delay_tau: float = 5.0

    @property
    def tau(self) -> float:
        if self.bandwidth <= 0:
            raise ModelError("FDTD_BAD_WAVEFORM", "bandwidth must be positive")
        width = math.sqrt(math.log(10.0)) / (math.pi * self.bandwidth)
        return 2.0 * width if self.kind == "gauss_mod" else width

    def __call__(self, t: FloatArray) -> FloatArray:
        tau = self.tau
        t0 = self.delay_tau * tau
        env = np.exp(-(((t - t0) / tau) ** 2))
        if self.kind == "gauss":
            return env  # type: ignore[no-any-return]
        return env * np.sin(2.0 * math.pi * self.f0 * (t - t0))  # type: ignore[no-any-return]


@dataclass(frozen=True)
class Region:
    """Material box (cells whose centre lies inside) or PEC box (edges inside, closed)."""

    lo: tuple[float, float, float]
    hi: tuple[float, float, float]
    eps_r: float = 1.0  # eps_inf when ``poles`` is given
    sigma: float = 0.0
    pec: bool = False
    poles: tuple[tuple[float, float], ...] = ()  # Debye (delta_eps, tau [s])


@dataclass(frozen=True)
class Conductor:
    """Copper box: PEC inside, surface-impedance boundary on its face edges."""

    lo: tuple[float, float, float]
    hi: tuple[float, float, float]
    sigma: float = 5.8e7
    thickness: float | None = None  # slab thickness for Zs; None = smallest box extent
    roughness_rms: float = 0.0
    k_func: Callable[[FloatArray], FloatArray] | None = None
    model: str = "thick_sibc"  # "thick_sibc" | "pec"
    edge_frac: float = 0.0


@dataclass(frozen=True)
class LumpedPort:
    """Resistive voltage source over all edges of one component inside the box."""

    name: str
    axis: int
    lo: tuple[float, float, float]
    hi: tuple[float, float, float]
    r_ohm: float = 50.0
    sign: float = 1.0


@dataclass(frozen=True)
class ModePort:
    """Quasi-TEM mode port on a plane (``open_analysis_gb300.modes``).

    The plane ``axis = position`` is cut by the in-plane rectangle ``lo .. hi`` (the two other
    axes in ascending order). The mode comes from a 2-D electrostatic solve with ``signals`` as the
    signal conductors (rectangles in the same axes); every other conductor, PEC region and PEC
    wall is ground. Ports with the same rectangle and signals but different ``mode`` give the modes
    of coupled conductors. The reference impedance is the modal one. ``direction`` +1: the
    structure lies towards +axis from the plane."""

    name: str
    axis: int
    position: float
    lo: tuple[float, float]
    hi: tuple[float, float]
    signals: tuple[tuple[tuple[float, float], tuple[float, float]], ...]
    mode: int = 0
    direction: int = 1
    sign: float = 1.0


@dataclass(frozen=True)
class SoftSource:
    """Additive source ``E += amplitude * s(t)`` on all edges of a component in the box."""

    name: str
    axis: int
    lo: tuple[float, float, float]
    hi: tuple[float, float, float]
    amplitude: float = 1.0


@dataclass(frozen=True)
class Probe:
    """Weighted sum of one field component over a box, recorded every step and DFT'd.

    ``weight``: ``"sum"``, ``"mean"`` or ``"line"`` (times the edge length along the axis).
    """

    name: str
    kind: str
    axis: int
    lo: tuple[float, float, float]
    hi: tuple[float, float, float]
    weight: str = "sum"


@dataclass
class Model:
    """A complete engine-level problem."""

    grid: Grid
    waveform: Waveform
    frequencies: FloatArray
    regions: list[Region] = field(default_factory=list)
    conductors: list[Conductor] = field(default_factory=list)
    walls: tuple[str, str, str, str, str, str] = ("pec",) * 6  # xlo xhi ylo yhi zlo zhi
    cpml: CpmlSpec = field(default_factory=CpmlSpec)
    ports: list[LumpedPort | ModePort] = field(default_factory=list)
    sources: list[SoftSource] = field(default_factory=list)
    mode_probes: list[ModePort] = field(default_factory=list)
    probes: list[Probe] = field(default_factory=list)
    drive: FloatArray | None = None  # (B, channels); channels = ports then sources
    courant: float = 0.95
    excite: tuple[str, ...] | None = None
    f_band: tuple[float, float] | None = None

    @property
    def band(self) -> tuple[float, float]:
        if self.f_band is not None:
            return self.f_band
        f = [float(v) for v in np.asarray(self.frequencies, dtype=np.float64).ravel()]
        return (min(f), max(f))

    @property
    def channels(self) -> int:
        return len(self.ports) + len(self.sources)

    def excited_indices(self) -> list[int]:
        """Indices of the driven ports, in batch order."""
        if self.excite is None:
            return list(range(len(self.ports)))
        names = [p.name for p in self.ports]
        unknown = [q for q in self.excite if q not in names]
        if unknown:
            raise ModelError("FDTD_BAD_DRIVE", f"excite names unknown ports {unknown}")
        return [names.index(q) for q in self.excite]

    def drive_matrix(self) -> FloatArray:
        if self.drive is not None:
            d = np.atleast_2d(np.asarray(self.drive, dtype=np.float64))
            if d.shape[1] != self.channels:
                raise ModelError("FDTD_BAD_DRIVE", "drive needs one column per port and source")
            return d
        if self.ports:
            rows = self.excited_indices()
            eye = np.eye(len(self.ports))[rows]
            return np.concatenate([eye, np.ones((len(rows), len(self.sources)))], axis=1)
        return np.ones((1, self.channels))


@dataclass
class AdeData:
    """Debye ADE edge lists, one entry per E component that has dispersive edges."""

    kp: FloatArray  # (P,) (1 - dt / 2 tau) / (1 + dt / 2 tau)
    tau: FloatArray  # (P,)
    comp: list[int]
    flat: list[npt.NDArray[np.int64]]
    beta: list[FloatArray]  # (P, ne) eps0 delta_p / (tau_p + dt / 2)
    cbe: list[FloatArray]  # (ne,) cb of the edge's table entry


@dataclass
class SibcData:
    """Surface-impedance edge list and its recursive-convolution tables."""

    comp: npt.NDArray[np.int32]
    flat: npt.NDArray[np.int64]
    hcomp: npt.NDArray[np.int32]  # (ne, 2)
    hflat: npt.NDArray[np.int64]  # (ne, 2)
    hsign: FloatArray  # (ne, 2); 0 = unused slot
    mat: npt.NDArray[np.int32]  # (ne,)
    r0: FloatArray  # (M,)
    rp: FloatArray  # (M, P)
    cp: FloatArray  # (P,)
    gp: FloatArray  # (P,)


@dataclass
class Compiled:
    """Everything the engines consume, as plain arrays."""

    grid: Grid
    dt: float
    idx: list[npt.NDArray[np.uint16]]
    eps_tab: FloatArray
    sig_tab: FloatArray
    ca_tab: FloatArray
    cb_tab: FloatArray
    walls: tuple[str, ...]
    pml: Pml
    channels: list[dict[str, Any]]
    probes: list[dict[str, Any]]
    ports: list[dict[str, Any]]
    drive: FloatArray
    frequencies: FloatArray
    ade: AdeData | None = None
    sibc: SibcData | None = None
    probe_sums: dict[str, list[str]] = field(default_factory=dict)

    @property
    def batch(self) -> int:
        return int(self.drive.shape[0])


# ------------------------------------------------------------------ compiler stages
def _pole_taus(model: Model) -> FloatArray:
    """Sorted union of all Debye relaxation times (rounded to 1e-18 s)."""
    taus = {round(t, 18) for r in model.regions if not r.pec for _, t in r.poles}
    return np.array(sorted(taus), dtype=np.float64)


def _cell_materials(model: Model, taus: FloatArray) -> tuple[FloatArray, FloatArray, list[FloatArray]]:
    """Per-cell eps, sigma and Debye strengths on ``(nz + 2, ny + 2, nx + 2)``; later regions
    overwrite earlier ones; ghost cells keep vacuum."""
    g = model.grid
    nx, ny, nz = g.n
    eps = np.ones((nz + 2, ny + 2, nx + 2))
    sig = np.zeros_like(eps)
    strengths = [np.zeros_like(eps) for _ in taus]
    centres = [g.centers(a) for a in range(3)]
    for reg in model.regions:
        if reg.pec:
            continue
        hit = [
            np.flatnonzero((centres[a] >= reg.lo[a]) & (centres[a] <= reg.hi[a])) + 1
            for a in range(3)
        ]
        box = np.ix_(hit[2], hit[1], hit[0])
        eps[box] = reg.eps_r
        sig[box] = reg.sigma
        by_tau = {round(t, 18): d for d, t in reg.poles}
        for pi, tau in enumerate(taus):
            strengths[pi][box] = by_tau.get(round(float(tau), 18), 0.0)
    return eps, sig, strengths


def _along(v: FloatArray, axis: int) -> FloatArray:
    """Broadcast a 1-D array along ``axis`` of a ``(z, y, x)`` array."""
    shape = [1, 1, 1]
    shape[2 - axis] = v.size
    return v.reshape(shape)


def _edge_average(g: Grid, comp: int, cell_arrays: list[FloatArray]) -> list[FloatArray]:
    """Area-weighted mean of the (up to) four cells around every ``comp`` edge.

    Result shape ``(nz + 1, ny + 1, nx + 1)``. The four neighbours are visited in the order
    (0,0), (0,1), (1,0), (1,1) of the offsets along the transverse axes ``p < q``; the sums run
    in that order (the table keys depend on it bit for bit).
    """
    n = g.n
    w = [g.cell_weights(a)[: n[a] + 2] for a in range(3)]
    p, q = [a for a in range(3) if a != comp]
    lattice = (n[2] + 1, n[1] + 1, n[0] + 1)
    sums = [np.zeros(lattice) for _ in cell_arrays]
    wsum = np.zeros(lattice)
    for dp in (0, 1):
        for dq in (0, 1):
            shift = [0, 0, 0]
            shift[p], shift[q] = dp, dq
            window = tuple(slice(1 - shift[ax], n[ax] + 2 - shift[ax]) for ax in (2, 1, 0))
            weight = np.ones(lattice) * _along(w[p][1 - dp : n[p] + 2 - dp], p)
            weight = weight * _along(w[q][1 - dq : n[q] + 2 - dq], q)
            for acc, arr in zip(sums, cell_arrays, strict=True):
                acc += weight * arr[window]
            wsum += weight
    return [s / wsum for s in sums]


def _box_indices(g: Grid, comp: int, lo: tuple[float, ...], hi: tuple[float, ...]) -> tuple[Any, ...]:
    """``np.ix_`` selector of the ``comp`` edges inside a closed box on the edge lattice."""
    sel: list[Any] = [None, None, None]
    for a in range(3):
        pos = g.coords(a, a != comp)
        tol = 1e-6 * float(np.min(g.d(a)))
        ids = np.flatnonzero((pos >= lo[a] - tol) & (pos <= hi[a] + tol))
        sel[2 - a] = ids if ids.size else np.array([], dtype=np.intp)
    return np.ix_(sel[0], sel[1], sel[2])


def _sibc_band(model: Model) -> tuple[float, float]:
    freqs = np.asarray(model.frequencies, dtype=np.float64)
    wf = model.waveform
    top = wf.f0 + 0.5 * wf.bandwidth if wf.kind == "gauss_mod" else wf.bandwidth
    f_hi = float(max(model.band[1], top))
    if model.f_band is not None:
        return max(f_hi * 1e-3, 1e5), f_hi
    return max(float(np.min(freqs)) * 0.5, f_hi * 1e-3, 1e5), f_hi


def _compile_conductors(
    model: Model, g: Grid, pec: list[npt.NDArray[np.bool_]], dt: float
) -> SibcData | None:
    """Mark copper interiors PEC and build the surface-impedance edge list (``pec`` is updated;
    the face edges are marked PEC too: the bulk update zeroes them and the SIBC pass sets them)."""
    if not model.conductors:
        return None
    f_lo, f_hi = _sibc_band(model)
    fit_of: dict[tuple[float, float, float, int], int] = {}
    fits: list[SibcFit] = []
    boxes = []
    for cd in model.conductors:
        edges = classify_box(g, cd.lo, cd.hi)
        for c in range(3):
            pec[c][edges.interior[c]] = True
        if cd.model == "pec":
            for c in range(3):
                pec[c][edges.surface[c]] = True
            continue
        if cd.model != "thick_sibc":
            raise ModelError("FDTD_BAD_CONDUCTOR", f"conductor model {cd.model!r}")
        thick = (
            cd.thickness
            if cd.thickness is not None
            else min(h - lo for lo, h in zip(cd.lo, cd.hi, strict=True))
        )
        if thick <= 0:
            raise ModelError("FDTD_BAD_CONDUCTOR", "conductor box has zero thickness")
        key = (cd.sigma, float(thick), cd.roughness_rms, id(cd.k_func))
        if key not in fit_of:
            fit_of[key] = len(fits)
            fits.append(
                fit_surface_impedance(
                    cd.sigma, thick, f_lo, f_hi, rms=cd.roughness_rms, roughness=cd.k_func
                )
            )
        boxes.append((edges, fit_of[key]))
    columns: list[list[np.ndarray]] = [[] for _ in range(9)]
    for edges, mat in boxes:
        for c in range(3):
            k, j, i = edges.surface[c]
            if k.size == 0:
                continue
            free = ~pec[c][k, j, i]  # interiors of any box, walls and PEC regions win
            if not free.any():
                continue
            k, j, i = k[free], j[free], i[free]
            p, hc, hf, hs = outside_samples(
                g, c, k, j, i, edges.face_a[c][free], edges.face_b[c][free]
            )
            for col, v in zip(
                columns, (np.full(p.size, c), p, hc, hf, hs, np.full(p.size, mat), k, j, i),
                strict=True,
            ):
                col.append(v)
    if not columns[0]:
        return None
    cat = [np.concatenate(col) for col in columns]
    key_all = cat[0].astype(np.int64) * (1 << 44) + cat[1]
    # a shared edge belongs to the last box that lists it
    _, first_rev = np.unique(key_all[::-1], return_index=True)
    last = np.sort(key_all.size - 1 - first_rev)
    cat = [v[last] for v in cat]
    order = np.argsort(cat[0].astype(np.int64) * (1 << 44) + cat[1], kind="stable")
    cat = [v[order] for v in cat]
    for c in range(3):
        m = cat[0] == c
        pec[c][cat[6][m], cat[7][m], cat[8][m]] = True
    n_poles = max(f.rp.size for f in fits)
    tau = fits[0].tau
    for f in fits[1:]:
        if f.tau.shape != tau.shape or not np.allclose(f.tau, tau):
            raise ModelError("FDTD_BAD_CONDUCTOR", "conductors need one common pole set")
    rp = np.zeros((len(fits), n_poles))
    for mi, f in enumerate(fits):
        rp[mi, : f.rp.size] = f.rp
    cp, gp = fits[0].recursion(dt)
    return SibcData(
        comp=cat[0].astype(np.int32),
        flat=cat[1].astype(np.int64),
        hcomp=cat[2].astype(np.int32),
        hflat=cat[3].astype(np.int64),
        hsign=cat[4].astype(np.float64),
        mat=cat[5].astype(np.int32),
        r0=np.array([f.r0 for f in fits]),
        rp=rp,
        cp=cp,
        gp=gp,
    )


def _compile_ade(
    g: Grid,
    dt: float,
    taus: FloatArray,
    edge_del: list[list[FloatArray]],
    pec: list[npt.NDArray[np.bool_]],
    idx: list[npt.NDArray[np.uint16]],
    cb_tab: FloatArray,
) -> AdeData | None:
    """Edge lists of the dispersive (any pole strength > 1e-12), non-PEC edges."""
    if taus.size == 0:
        return None
    tau = np.asarray(taus, dtype=np.float64)
    comps: list[int] = []
    flats: list[npt.NDArray[np.int64]] = []
    betas: list[FloatArray] = []
    cbes: list[FloatArray] = []
    sz, sy = g.shape[1] * g.shape[2], g.shape[2]
    for c in range(3):
        strength = np.zeros_like(edge_del[c][0])
        for d_p in edge_del[c]:
            strength += d_p
        mask = (strength > 1e-12) & ~pec[c]
        k, j, i = np.nonzero(mask)
        if k.size == 0:
            continue
        comps.append(c)
        flats.append(((k + 1) * sz + (j + 1) * sy + (i + 1)).astype(np.int64))
        betas.append(
            np.stack([EPS0 * edge_del[c][p][mask] / (tau[p] + 0.5 * dt) for p in range(tau.size)])
        )
        cbes.append(cb_tab[idx[c][k + 1, j + 1, i + 1]])
    if not comps:
        return None
    kp = (1.0 - 0.5 * dt / tau) / (1.0 + 0.5 * dt / tau)
    return AdeData(kp=kp, tau=tau, comp=comps, flat=flats, beta=betas, cbe=cbes)


def _material_table(
    g: Grid,
    edge_eps: list[FloatArray],
    edge_sig: list[FloatArray],
    pec: list[npt.NDArray[np.bool_]],
) -> tuple[list[npt.NDArray[np.uint16]], FloatArray, FloatArray]:
    """Unique (eps, sigma) pairs of the non-PEC edges (keys rounded to 12 decimals), sorted by
    eps then sigma; index 0 is PEC. Returns the per-component storage index arrays."""
    nx, ny, nz = g.n
    uniq_per: list[np.ndarray] = []
    inv_per: list[np.ndarray] = []
    for c in range(3):
        keep = ~pec[c]
        keys = np.round(edge_eps[c][keep], 12) + 1j * np.round(edge_sig[c][keep], 12)
        u, inv = np.unique(keys, return_inverse=True)
        uniq_per.append(u)
        inv_per.append(inv.ravel())
    table, merge = np.unique(np.concatenate(uniq_per), return_inverse=True)
    merge = merge.ravel()
    if table.size + 1 > MAX_TABLE:
        raise ModelError(
            "FDTD_TOO_MANY_MATERIALS",
            f"{table.size} averaged materials exceed the uint16 table",
            "Use fewer distinct materials or a more uniform grid.",
        )
    idx: list[npt.NDArray[np.uint16]] = []
    start = 0
    for c in range(3):
        global_ids = merge[start : start + uniq_per[c].size][inv_per[c]]
        start += uniq_per[c].size
        lattice = np.zeros((nz + 1, ny + 1, nx + 1), dtype=np.uint16)
        lattice[~pec[c]] = (global_ids + 1).astype(np.uint16)
        arr = np.zeros(g.shape, dtype=np.uint16)
        arr[1 : nz + 2, 1 : ny + 2, 1 : nx + 2] = lattice
        idx.append(arr)
    eps_tab = np.concatenate([[0.0], table.real])
    sig_tab = np.concatenate([[0.0], table.imag])
    return idx, eps_tab, sig_tab


def update_coefficients(eps_tab: FloatArray, sig_tab: FloatArray, dt: float) -> tuple[FloatArray, FloatArray]:
    """``ca = (1 - l) / (1 + l)``, ``cb = dt / eps / (1 + l)``, ``l = sigma dt / (2 eps)``; 0 for
    the PEC entry."""
    ep = eps_tab * EPS0
    loss = sig_tab * dt / (2.0 * np.where(ep > 0, ep, 1.0))
    ca = np.where(eps_tab > 0, (1.0 - loss) / (1.0 + loss), 0.0)
    cb = np.where(eps_tab > 0, dt / np.where(ep > 0, ep, 1.0) / (1.0 + loss), 0.0)
    return ca, cb


def _native_library() -> Any:
    """The engine library when it is built (it loads without a GPU), else None."""
    try:
        from open_analysis_gb300 import native as nat

        return nat.load() if nat.library_path().exists() else None
    except Exception:  # noqa: BLE001 - a missing or foreign library means the NumPy stages
        return None


def _native_materials(
    model: Model,
    g: Grid,
    dt: float,
    taus: FloatArray,
    pec: list[npt.NDArray[np.bool_]],
    loads: list[tuple[int, int, float]],
    threads: int = 0,
) -> tuple[list[npt.NDArray[np.uint16]], FloatArray, FloatArray, list[int], list[Any], list[FloatArray], list[FloatArray]]:
    """The volume stages on the engine library's native compiler: index arrays, eps and sigma
    tables, and per dispersive component its storage flat indices, Debye coefficients beta
    ``(poles, n)`` and the ``cb`` of each edge."""
    import ctypes as C

    from open_analysis_gb300 import native as nat

    lib = nat.load()
    nx, ny, nz = g.n
    regs = [r for r in model.regions if not r.pec]
    n_poles = int(taus.size)
    keep: list[Any] = []

    def dp(a: Any) -> Any:
        arr = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(arr)
        return arr.ctypes.data_as(C.POINTER(C.c_double))

    d = nat.MaterialDesc()
    d.nx, d.ny, d.nz = nx, ny, nz
    for a in range(3):
        d.cell_w[a] = dp(g.cell_weights(a)[: g.n[a] + 2])
        d.centres[a] = dp(g.centers(a))
        m8 = np.ascontiguousarray(pec[a]).view(np.uint8)
        keep.append(m8)
        d.pec[a] = m8.ctypes.data_as(C.POINTER(C.c_uint8))
    d.n_regions = len(regs)
    d.reg_lo = dp([r.lo for r in regs] or [[0.0, 0.0, 0.0]])
    d.reg_hi = dp([r.hi for r in regs] or [[0.0, 0.0, 0.0]])
    d.reg_eps = dp([r.eps_r for r in regs] or [0.0])
    d.reg_sig = dp([r.sigma for r in regs] or [0.0])
    strength = np.zeros((max(1, len(regs)), max(1, n_poles)))
    for ri, r in enumerate(regs):
        by_tau = {round(t, 18): dv for dv, t in r.poles}
        for pi, tau in enumerate(taus):
            strength[ri, pi] = by_tau.get(round(float(tau), 18), 0.0)
    d.n_poles = n_poles
    d.reg_strength = dp(strength[:, :n_poles] if n_poles else strength)
    d.static_fac = dp([dt / (2.0 * float(t) + dt) for t in taus] or [0.0])
    comp = np.array([ld[0] for ld in loads] or [0], dtype=np.int32)
    lat = np.array([ld[1] for ld in loads] or [0], dtype=np.int64)
    sig = np.array([ld[2] for ld in loads] or [0.0], dtype=np.float64)
    keep += [comp, lat, sig]
    d.n_loads = len(loads)
    d.load_comp = comp.ctypes.data_as(C.POINTER(C.c_int32))
    d.load_lattice = lat.ctypes.data_as(C.POINTER(C.c_int64))
    d.load_sig = sig.ctypes.data_as(C.POINTER(C.c_double))
    d.threads = int(threads)
    d.dt = float(dt)
    d.eps0 = float(EPS0)
    d.taus = dp(taus if n_poles else [0.0])
    handle = C.c_void_p()
    rc = lib.oafdtd_materials_build(C.byref(d), C.byref(handle))
    if rc == nat.E_TABLE:
        raise ModelError(
            "FDTD_TOO_MANY_MATERIALS",
            lib.oafdtd_last_error().decode(errors="replace"),
            "Use fewer distinct materials or a more uniform grid.",
        )
    nat.check(rc, "oafdtd_materials_build")
    try:
        n_mat = C.c_int32()
        ade_n = (C.c_int64 * 3)()
        nat.check(lib.oafdtd_materials_sizes(handle, C.byref(n_mat), ade_n), "oafdtd_materials_sizes")
        idx = [np.zeros(g.shape, dtype=np.uint16) for _ in range(3)]
        eps_tab = np.zeros(n_mat.value)
        sig_tab = np.zeros(n_mat.value)
        flats = [np.empty(int(ade_n[c]), dtype=np.int64) for c in range(3)]
        betas = [np.empty((n_poles, int(ade_n[c]))) for c in range(3)]
        cbes = [np.empty(int(ade_n[c])) for c in range(3)]
        u16 = C.POINTER(C.c_uint16)
        dpp = C.POINTER(C.c_double)
        nat.check(
            lib.oafdtd_materials_fetch(
                handle,
                *(a.ctypes.data_as(u16) for a in idx),
                eps_tab.ctypes.data_as(dpp),
                sig_tab.ctypes.data_as(dpp),
                *(f.ctypes.data_as(C.POINTER(C.c_int64)) if f.size else None for f in flats),
                *(x.ctypes.data_as(dpp) if x.size else None for x in betas),
                *(x.ctypes.data_as(dpp) if x.size else None for x in cbes),
            ),
            "oafdtd_materials_fetch",
        )
    finally:
        lib.oafdtd_materials_free(handle)
    comps = [c for c in range(3) if flats[c].size]
    return (idx, eps_tab, sig_tab, comps, [flats[c] for c in comps], [betas[c] for c in comps],
            [cbes[c] for c in comps])


def compile_model(model: Model, dtype: str = "float32", native: bool | None = None) -> Compiled:
    """Build the index arrays, tables, PML, channels and probes. Raises :class:`ModelError`.

    ``native``: run the volume stages on the engine library's native compiler (``True``), on
    NumPy (``False``), or on the native compiler when the library is built (``None``); the
    arrays are the same bit for bit."""
    del dtype  # the compiled arrays are float64 and uint16 whatever the engine precision
    g = model.grid
    nx, ny, nz = g.n
    if len(model.walls) != 6 or any(w not in WALL_KINDS for w in model.walls):
        raise ModelError("FDTD_BAD_WALLS", f"walls must be six of {WALL_KINDS}")
    n_dielectric = sum(1 for r in model.regions if not r.pec)
    has_modes = any(isinstance(p, ModePort) for p in model.ports) or bool(model.mode_probes)
    if native is None:
        # the native compiler numbers cells by region in uint16; mode ports read the per-edge
        # permittivity arrays of the NumPy stages
        native = _native_library() is not None and n_dielectric <= 65534 and not has_modes
    elif native and (n_dielectric > 65534 or has_modes):
        raise ModelError("FDTD_BAD_INPUT", "the native compiler takes at most 65534 dielectric regions and no mode ports")
    eps_min = min([1.0] + [r.eps_r for r in model.regions if not r.pec])
    dt = g.dt(model.courant, 299792458.0 / math.sqrt(eps_min))
    vacuum_only = not model.regions and not model.ports and not model.conductors
    taus = _pole_taus(model)

    lattice = (nz + 1, ny + 1, nx + 1)
    edge_eps: list[FloatArray] = []
    edge_sig: list[FloatArray] = []
    edge_del: list[list[FloatArray]] = []
    pec: list[npt.NDArray[np.bool_]] = []
    if not native:
        eps_c, sig_c, del_c = _cell_materials(model, taus)
    for c in range(3):
        if not native:
            if vacuum_only:
                edge_eps.append(np.ones(lattice))
                edge_sig.append(np.zeros(lattice))
                edge_del.append([])
            else:
                e, s, *ds = _edge_average(g, c, [eps_c, sig_c, *del_c])
                edge_eps.append(e)
                edge_sig.append(s)
                edge_del.append(ds)
        real_edges = np.zeros(lattice, dtype=bool)
        (x0, x1), (y0, y1), (z0, z1) = g.valid("E", c)
        real_edges[z0 - 1 : z1 - 1, y0 - 1 : y1 - 1, x0 - 1 : x1 - 1] = True
        pec.append(~real_edges)
    eps_mid: FloatArray | None = None
    if has_modes:
        # real relative permittivity of the cells at the band centre, for the plane solves
        w_mid = 2.0 * np.pi * 0.5 * sum(model.band)
        eps_mid = eps_c.copy()
        for pi, tau in enumerate(taus):
            eps_mid = eps_mid + del_c[pi] / (1.0 + (w_mid * float(tau)) ** 2)
        eps_mid = eps_mid[1:-1, 1:-1, 1:-1]
    if not native:
        del eps_c, sig_c, del_c
        # the static part of the Debye polarisation current joins eps: eps_inf + sum d_p dt/(2 tau+dt)
        for c in range(3):
            for pi, tau in enumerate(taus):
                edge_eps[c] += edge_del[c][pi] * (dt / (2.0 * float(tau) + dt))
    # tangential E on PEC and CPML outer walls
    for a in range(3):
        for side in (0, 1):
            if model.walls[2 * a + side] == "pmc":
                continue
            plane = 0 if side == 0 else g.n[a]
            for c in range(3):
                if c != a:
                    sel: list[Any] = [slice(None)] * 3
                    sel[2 - a] = plane
                    pec[c][tuple(sel)] = True
    for reg in model.regions:
        if reg.pec:
            for c in range(3):
                pec[c][_box_indices(g, c, reg.lo, reg.hi)] = True

    sibc = _compile_conductors(model, g, pec, dt)

    channels: list[dict[str, Any]] = []
    ports_info: list[dict[str, Any]] = []
    probes: list[dict[str, Any]] = []
    loads: list[tuple[int, int, float]] = []
    sz, sy = g.shape[1] * g.shape[2], g.shape[2]
    mode_cache: dict[Any, Any] = {}

    def mode_port(mp_: ModePort) -> dict[str, Any]:
        from open_analysis_gb300.modes import build_mode_port, solve_port_modes

        key = (mp_.axis, mp_.position, mp_.lo, mp_.hi, mp_.signals, mp_.direction)
        try:
            if key not in mode_cache:
                assert eps_mid is not None
                mode_cache[key] = solve_port_modes(model, g, mp_, eps_mid)
            modes, geo = mode_cache[key]
            return build_mode_port(g, mp_, modes, geo, edge_eps)
        except ValueError as exc:
            raise ModelError("FDTD_BAD_PORT", str(exc)) from exc

    def mode_parts(mp_: ModePort, arr: dict[str, Any], load: bool) -> list[str]:
        """One probe per field component of the plane (and the sheet's loading when ``load``)."""
        parts: list[str] = []
        start = 0
        for comp_seg, count in zip(sorted({int(v) for v in arr["comp"]}), arr["split"], strict=True):
            seg = slice(start, start + count)
            start += count
            fl = arr["flat"][seg]
            if load:
                kk, jj, ii = np.unravel_index(fl, g.shape)
                edge_sig[comp_seg][kk - 1, jj - 1, ii - 1] += arr["sigma"][seg]
            parts.append(f"V:{mp_.name}:{comp_seg}")
            probes.append({"name": parts[-1], "kind": "E", "comp": comp_seg, "flat": fl, "weights": arr["weights"][seg]})
        return parts

    for port in model.ports:
        if isinstance(port, ModePort):
            arr = mode_port(port)
            parts = mode_parts(port, arr, load=True)
            ports_info.append(
                {
                    "name": port.name,
                    "axis": port.axis,
                    "r_ohm": arr["z"],
                    "sign": port.sign,
                    "flat": arr["flat"],
                    "channel": len(channels),
                    "sig_e": arr["sigma"],
                    "e_t": arr["template"],
                    "probe_parts": parts,
                    "eps_eff": arr["eps_eff"],
                    "voltages": arr["voltages"],
                }
            )
            channels.append({"comp": arr["comp"], "flat": arr["flat"], "port": len(ports_info) - 1, "sign": port.sign})
            continue
        assert isinstance(port, LumpedPort)
        if port.r_ohm <= 0:
            raise ModelError("FDTD_BAD_PORT", f"port {port.name}: r_ohm must be positive")
        flat, counts = g.points("E", port.axis, port.lo, port.hi)
        k, rem = np.divmod(flat, sz)
        j, i = np.divmod(rem, sy)
        ijk = (i, j, k)
        a = port.axis
        t0, t1 = [t for t in range(3) if t != a]
        length = g.d(a)[ijk[a] - 1]
        area = g.node_weights(t0)[ijk[t0]] * g.node_weights(t1)[ijk[t1]]
        n_series = counts[a]
        total_len = float(length.sum()) / (flat.size / n_series)
        total_area = float(area.sum()) / n_series
        sig_eq = total_len / (port.r_ohm * total_area)
        if native:
            lat = ((k - 1) * (ny + 1) + (j - 1)) * (nx + 1) + (i - 1)
            loads += [(a, int(q), sig_eq) for q in lat]
        else:
            edge_sig[a][k - 1, j - 1, i - 1] += sig_eq
        ports_info.append(
            {
                "name": port.name,
                "axis": a,
                "r_ohm": port.r_ohm,
                "sign": port.sign,
                "flat": flat,
                "channel": len(channels),
                "sig_eq": sig_eq,
                "total_len": total_len,
                "total_area": total_area,
            }
        )
        channels.append({"comp": a, "flat": flat, "port": len(ports_info) - 1, "sign": port.sign})
        probes.append(
            {
                "name": f"V:{port.name}",
                "kind": "E",
                "comp": a,
                "flat": flat,
                "weights": length * area / total_area,
            }
        )
    probe_sums: dict[str, list[str]] = {}
    for mpb in model.mode_probes:
        probe_sums[f"V:{mpb.name}"] = mode_parts(mpb, mode_port(mpb), load=False)
    for src in model.sources:
        flat, _ = g.points("E", src.axis, src.lo, src.hi)
        channels.append({"comp": src.axis, "flat": flat, "amp": src.amplitude})
    for pr in model.probes:
        flat, _ = g.points(pr.kind, pr.axis, pr.lo, pr.hi)
        k, rem = np.divmod(flat, sz)
        j, i = np.divmod(rem, sy)
        ijk = (i, j, k)
        if pr.weight == "sum":
            w = np.ones(flat.size)
        elif pr.weight == "mean":
            w = np.full(flat.size, 1.0 / flat.size)
        elif pr.weight == "line":
            ax = pr.axis
            w = (g.d(ax)[ijk[ax] - 1] if pr.kind == "E" else g.node_weights(ax)[ijk[ax]]).astype(
                np.float64
            )
        else:
            raise ModelError("FDTD_BAD_PROBE", f"probe {pr.name}: weight {pr.weight!r}")
        probes.append({"name": pr.name, "kind": pr.kind, "comp": pr.axis, "flat": flat, "weights": w})

    if native:
        idx, eps_tab, sig_tab, comps, flats, betas, cbes = _native_materials(model, g, dt, taus, pec, loads)
        ca_tab, cb_tab = update_coefficients(eps_tab, sig_tab, dt)
        ade = None
        if taus.size and comps:
            tau = np.asarray(taus, dtype=np.float64)
            ade = AdeData(kp=(1.0 - 0.5 * dt / tau) / (1.0 + 0.5 * dt / tau), tau=tau, comp=comps, flat=flats,
                          beta=betas, cbe=cbes)
    else:
        idx, eps_tab, sig_tab = _material_table(g, edge_eps, edge_sig, pec)
        ca_tab, cb_tab = update_coefficients(eps_tab, sig_tab, dt)
        ade = _compile_ade(g, dt, taus, edge_del, pec, idx, cb_tab)

    for ch in channels:
        if np.ndim(ch["comp"]) == 0:
            mat = idx[ch["comp"]].ravel()[ch["flat"]]
        else:
            mat = np.zeros(ch["flat"].size, dtype=np.uint16)
            for cc in np.unique(ch["comp"]):
                on = ch["comp"] == cc
                mat[on] = idx[int(cc)].ravel()[ch["flat"][on]]
        if "port" in ch:
            info = ports_info[ch["port"]]
            if "sig_e" in info:  # mode port: the sheet's own loading times its template
                ch["amps"] = ch["sign"] * cb_tab[mat] * info["sig_e"] * info["e_t"]
            else:
                ch["amps"] = ch["sign"] * cb_tab[mat] * info["sig_eq"] / info["total_len"]
        else:
            ch["amps"] = ch["amp"] * np.ones(ch["flat"].size)
        ch["waveform"] = model.waveform
    pml = build_pml(g, model.walls, model.cpml, dt)
    return Compiled(
        grid=g,
        dt=dt,
        idx=idx,
        eps_tab=eps_tab,
        sig_tab=sig_tab,
        ca_tab=ca_tab,
        cb_tab=cb_tab,
        walls=model.walls,
        pml=pml,
        channels=channels,
        probes=probes,
        ports=ports_info,
        drive=model.drive_matrix(),
        frequencies=np.asarray(model.frequencies, dtype=np.float64),
        ade=ade,
        sibc=sibc,
        probe_sums=probe_sums,
    )
