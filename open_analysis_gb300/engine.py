"""``Gb300Engine``: the engine protocol over the sm_103a CUDA library.

Drop-in for the reference's ``CupyEngine`` (``packages/oa-fdtd/src/oa_fdtd/engine.py:67-506``):
same constructor arguments, same methods (``step, energy, results, series, get_fields,
peak_bytes``), same shapes, units and time stamps (H probes at (n+1/2) dt, E probes at (n+1) dt,
sources at (n+1/2) dt), same ``ValueError`` past ``max_steps``. It consumes a ``Compiled``
problem as-is; the library copies it to the device once and owns all device state.
"""

from __future__ import annotations

import ctypes as C
from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300 import native
from open_analysis_gb300.grid import MU0

FloatArray = npt.NDArray[np.float64]
CHUNK = 64


def estimate_bytes(c: Any, itemsize: int, max_steps: int = 200_000, record_series: bool = False) -> int:
    """Device bytes ``Gb300Engine`` allocates for a compiled problem: the role of the reference's
    ``estimate_bytes`` (``engine.py:29-40``), which the run driver checks against free device
    memory before it builds the engine, counted from this engine's own buffers.

    * six field arrays ``(B, Z, Y, X)`` twice (the fused sweep, the default wherever the grid has
      an interior free of CPML cells, reads one set and writes the other) and the three uint16
      index arrays ``(Z, Y, X)``;
    * dense Debye currents ``(P, B, nk, Y, X)`` per component over the z range ``nk`` of its
      dispersive edges;
    * one CPML psi array per correction: the slab width on its derivative axis, the full storage
      extent on the other two, per batch member;
    * surface impedance: a packed record per edge (32 bytes in float32, 48 in float64),
      ``J_prev (B, n)`` and ``v (P, B, n)``;
    * the edge list of injection targets and deferred Debye edges with their saved ``E^n``, the
      sampled wave table ``(channels, max_steps)``, the probe lists, the DFT accumulators
      ``(probes, B, F)`` complex128 and, when recording, the series ``(probes, B, max_steps)``;
    * the energy sum's float-float weights for float32 fields (per component, the x row and the
      y-z plane of pairs of float32);
    * the one-dimensional metrics, CPML coefficients, energy weights and partial sums, which are
      small; a fixed 1 MiB covers them and the per-allocation minimums.
    """
    g = c.grid
    Z, Y, X = g.shape
    B = int(c.batch)
    bs = Z * Y * X
    rb = int(itemsize)
    total = 2 * 6 * bs * B * rb + 3 * bs * 2
    ade_flat: list[np.ndarray] = [np.zeros(0, np.int64)] * 3
    if c.ade is not None:
        P = int(c.ade.tau.size)
        for comp, flat in zip(c.ade.comp, c.ade.flat, strict=True):
            fl = np.asarray(flat, np.int64)
            if fl.size == 0:
                continue
            ade_flat[int(comp)] = fl
            k = fl // (Y * X)
            total += P * B * int(k.max() - k.min() + 1) * Y * X * rb
    for corr in c.pml.corrections:
        ext = [X, Y, Z]
        ext[corr.a] = corr.box[corr.a][1] - corr.box[corr.a][0]
        total += B * ext[0] * ext[1] * ext[2] * rb
    none = np.zeros(0, np.int64)
    sibc_t = [none] * 3  # per component: surface-impedance edges and injection targets
    inj_t: list[list[np.ndarray]] = [[], [], []]
    if c.sibc is not None:
        s = c.sibc
        n_s = int(s.flat.size)
        total += n_s * (32 if rb == 4 else 48) + B * n_s * rb * (1 + int(s.cp.size))
        sibc_t = [np.asarray(s.flat, np.int64)[np.asarray(s.comp) == cc] for cc in range(3)]
    n_inj = 0
    for ch in c.channels:
        fl = np.asarray(ch["flat"], np.int64)
        comp = np.broadcast_to(np.asarray(ch["comp"]), fl.shape)
        n_inj += fl.size
        for cc in range(3):
            inj_t[cc].append(fl[comp == cc])
    inj_edges = n_def = 0
    for cc in range(3):
        inj = np.unique(np.concatenate(inj_t[cc] or [none]))
        inj_edges += inj.size
        n_def += int(np.isin(ade_flat[cc], np.concatenate([sibc_t[cc], inj])).sum())
    n_list = inj_edges + n_def
    total += n_list * (1 + 8 + 3 * 4) + n_inj * (4 + 8) + n_def * (8 + 1 + B * rb)
    n_chan = len(c.channels)
    total += n_chan * max_steps * 8 + B * n_chan * 8
    n_probe = len(c.probes)
    total += sum(np.asarray(q["flat"]).size for q in c.probes) * 16 + n_probe * 16
    total += n_probe * B * int(c.frequencies.size) * 16
    if record_series:
        total += n_probe * B * max_steps * 8
    if rb == 4:  # the float-float weights of the float32 energy sum: x row and y-z plane per component
        total += 6 * (X + Z * Y) * 8
    return int(total + (1 << 20))


def wave_table(c: Any, max_steps: int) -> FloatArray:
    """``s_c((n + 1/2) dt)`` for every channel and step (float64), evaluated as the reference's
    injection does; a vectorised evaluation is used only when it equals the per-step one."""
    t = (np.arange(max_steps) + 0.5) * c.dt
    out = np.zeros((len(c.channels), max_steps))
    for ci, ch in enumerate(c.channels):
        wf = ch["waveform"]
        vec = np.asarray(wf(t), dtype=np.float64)
        probe = np.unique(np.linspace(0, max_steps - 1, min(max_steps, 97)).astype(np.int64))
        scalar = np.array([float(wf(np.array([(int(n) + 0.5) * c.dt]))[0]) for n in probe])
        if not np.array_equal(vec[probe], scalar):
            vec = np.array([float(wf(np.array([(n + 0.5) * c.dt]))[0]) for n in range(max_steps)])
        out[ci] = vec
    return out


def _ptr(a: np.ndarray, ctype: Any) -> Any:
    return a.ctypes.data_as(C.POINTER(ctype))


def describe(c: Any, dtype: str = "float32", max_steps: int = 200_000,
             record_series: bool = False) -> tuple[native.Problem, list[Any]]:
    """The ``oafdtd_problem`` descriptor of a compiled problem: the ``Compiled`` arrays
    (``oa_fdtd/model.py:246-269``) flattened into the plain pointers and sizes of the C ABI, with
    the host buffers they point into (keep them alive until ``oafdtd_create`` returns). It reads
    only the attributes the reference's ``Compiled`` has, so a problem compiled by the reference
    goes through unchanged."""
    g = c.grid
    keep: list[Any] = []

    def arr(a: Any, dt: Any) -> np.ndarray:
        out = np.ascontiguousarray(np.asarray(a, dtype=dt))
        keep.append(out)
        return out

    p = native.Problem()
    p.abi_version = native.ABI_VERSION
    p.real_bytes = 4 if dtype == "float32" else 8
    p.nx, p.ny, p.nz = g.n
    p.pitch = g.pitch
    p.batch = c.batch
    p.dt = float(c.dt)
    p.dtmu = float(c.dt / MU0)
    for ci in range(3):
        p.idx[ci] = _ptr(arr(c.idx[ci], np.uint16), C.c_uint16)
    p.n_mat = int(c.eps_tab.size)
    p.ca_tab = _ptr(arr(c.ca_tab, np.float64), C.c_double)
    p.cb_tab = _ptr(arr(c.cb_tab, np.float64), C.c_double)
    p.eps_tab = _ptr(arr(c.eps_tab, np.float64), C.c_double)
    for a in range(3):
        p.inv_primal[a] = _ptr(arr(g.inv_primal(a), np.float64), C.c_double)
        p.inv_dual[a] = _ptr(arr(g.inv_dual(a), np.float64), C.c_double)
        p.node_w[a] = _ptr(arr(g.node_weights(a), np.float64), C.c_double)
        p.cell_w[a] = _ptr(arr(g.cell_weights(a), np.float64), C.c_double)
    p.pmc_mask = sum(1 << k for k in range(6) if c.walls[k] == "pmc")
    corr = c.pml.corrections
    p.n_corr = len(corr)
    if corr:
        cs = (native.Correction * len(corr))()
        for n, k in enumerate(corr):
            cs[n].kind = 0 if k.kind == "E" else 1
            cs[n].c, cs[n].a, cs[n].b = k.c, k.a, k.b
            cs[n].sign = float(k.sign)
            for ax in range(3):
                cs[n].lo[ax], cs[n].hi[ax] = k.box[ax]
        keep.append(cs)
        p.corr = C.cast(cs, C.POINTER(native.Correction))
    for a, co in c.pml.coeffs.items():
        for t, name in enumerate(("eb", "ec", "ek", "hb", "hc", "hk")):
            p.pml[a][t] = _ptr(arr(getattr(co, name), np.float64), C.c_double)
    # sources
    chans = c.channels
    p.n_chan = len(chans)
    p.max_steps = max_steps
    p.wave = _ptr(arr(wave_table(c, max_steps) if chans else np.zeros(1), np.float64), C.c_double)
    p.drive = _ptr(arr(c.drive, np.float64), C.c_double)
    comp, flat, amp, chan = [], [], [], []
    for ci, ch in enumerate(chans):
        fl = np.asarray(ch["flat"], dtype=np.int64)
        comp.append(np.broadcast_to(np.asarray(ch["comp"], np.int32), fl.shape))
        flat.append(fl)
        amp.append(np.asarray(ch["amps"], np.float64))
        chan.append(np.full(fl.size, ci, np.int32))
    cat = (lambda v, dt: np.concatenate(v).astype(dt) if v else np.zeros(0, dt))
    inj_comp, inj_flat = cat(comp, np.int32), cat(flat, np.int64)
    p.n_inj = int(inj_flat.size)
    p.inj_comp = _ptr(arr(inj_comp, np.int32), C.c_int32)
    p.inj_flat = _ptr(arr(inj_flat, np.int64), C.c_int64)
    p.inj_amp = _ptr(arr(cat(amp, np.float64), np.float64), C.c_double)
    p.inj_chan = _ptr(arr(cat(chan, np.int32), np.int32), C.c_int32)
    # probes
    probes = c.probes
    p.n_probe = len(probes)
    sizes = [np.asarray(q["flat"]).size for q in probes]
    p.probe_kind = _ptr(arr([0 if q["kind"] == "E" else 1 for q in probes] or [0], np.int32), C.c_int32)
    p.probe_comp = _ptr(arr([int(q["comp"]) for q in probes] or [0], np.int32), C.c_int32)
    p.probe_off = _ptr(arr(np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64), np.int64), C.c_int64)
    p.probe_flat = _ptr(
        arr(cat([np.asarray(q["flat"], np.int64) for q in probes], np.int64), np.int64), C.c_int64
    )
    p.probe_w = _ptr(
        arr(cat([np.asarray(q["weights"], np.float64) for q in probes], np.float64), np.float64),
        C.c_double,
    )
    p.n_freq = int(c.frequencies.size)
    p.omega = _ptr(arr(2.0 * np.pi * c.frequencies, np.float64), C.c_double)
    p.record_series = int(record_series)
    # Debye ADE
    if c.ade is not None:
        a = c.ade
        p.ade_poles = int(a.tau.size)
        p.ade_kp = _ptr(arr(a.kp, np.float64), C.c_double)
        for comp_, fl, be, cbe in zip(a.comp, a.flat, a.beta, a.cbe, strict=True):
            p.ade_n[comp_] = int(np.asarray(fl).size)
            p.ade_flat[comp_] = _ptr(arr(fl, np.int64), C.c_int64)
            p.ade_beta[comp_] = _ptr(arr(be, np.float64), C.c_double)
            p.ade_cbe[comp_] = _ptr(arr(cbe, np.float64), C.c_double)
    # surface impedance
    if c.sibc is not None:
        s = c.sibc
        p.sibc_n = int(s.flat.size)
        p.sibc_poles = int(s.cp.size)
        p.sibc_nmat = int(s.r0.size)
        p.sibc_comp = _ptr(arr(s.comp, np.int32), C.c_int32)
        p.sibc_flat = _ptr(arr(s.flat, np.int64), C.c_int64)
        p.sibc_hcomp = _ptr(arr(s.hcomp, np.int32), C.c_int32)
        p.sibc_hflat = _ptr(arr(s.hflat, np.int64), C.c_int64)
        p.sibc_hsign = _ptr(arr(s.hsign, np.float64), C.c_double)
        p.sibc_mat = _ptr(arr(s.mat, np.int32), C.c_int32)
        p.sibc_r0 = _ptr(arr(s.r0, np.float64), C.c_double)
        p.sibc_rp = _ptr(arr(s.rp, np.float64), C.c_double)
        p.sibc_cp = _ptr(arr(s.cp, np.float64), C.c_double)
        p.sibc_gp = _ptr(arr(s.gp, np.float64), C.c_double)
    return p, keep


class Gb300Engine:
    """Leapfrog Yee engine on one GB300 (the current CUDA device)."""

    name = "gb300"

    def __init__(
        self,
        c: Any,
        dtype: str = "float32",
        record_series: bool = False,
        max_steps: int = 200_000,
        use_graph: bool = True,
        **_: Any,
    ) -> None:
        self.c = c
        self.dtype = str(np.dtype(dtype))
        if self.dtype not in ("float32", "float64"):
            raise ValueError("dtype must be float32 or float64")
        self.record_series = bool(record_series)
        self.max_steps = int(max_steps)
        self._lib = native.load()
        self._h = C.c_void_p()
        g = c.grid
        self.B = c.batch
        self.shape = (self.B, *g.shape)
        prob, keep = describe(c, self.dtype, self.max_steps, self.record_series)
        # host buffers the library copies
        self.h2d_bytes = int(sum(a.nbytes for a in keep if isinstance(a, np.ndarray)))
        native.check(self._lib.oafdtd_create(C.byref(prob), C.byref(self._h)), "create")
        del keep
        self.set_graph(use_graph)
        self._probes = list(c.probes)

    # ------------------------------------------------------------------ protocol
    @property
    def step_count(self) -> int:
        n = C.c_int64()
        native.check(self._lib.oafdtd_step_count(self._h, C.byref(n)), "step_count")
        return int(n.value)

    def step(self, n: int = 1) -> None:
        if self.step_count + n > self.max_steps:
            raise ValueError("step count exceeds max_steps (wave table length)")
        native.check(self._lib.oafdtd_step(self._h, int(n)), "step")

    def step_async(self, n: int) -> None:
        """Queue ``n`` steps on the engine's stream and return; ``wait()`` synchronises. Engines
        on one device then run side by side (independent instances of a sweep)."""
        if self.step_count + n > self.max_steps:
            raise ValueError("step count exceeds max_steps (wave table length)")
        native.check(self._lib.oafdtd_step_async(self._h, int(n)), "step_async")

    def wait(self) -> None:
        native.check(self._lib.oafdtd_wait(self._h), "wait")

    # ------------------------------------------------------------------ snapshot / restore
    def snapshot(self) -> bytes:
        """The run's whole device state as bytes (see ``restore``)."""
        n = C.c_int64()
        native.check(self._lib.oafdtd_snapshot_bytes(self._h, C.byref(n)), "snapshot_bytes")
        buf = C.create_string_buffer(int(n.value))
        native.check(self._lib.oafdtd_snapshot(self._h, buf), "snapshot")
        return buf.raw

    def restore(self, state: bytes) -> None:
        """Put a ``snapshot`` of an engine of the same problem and configuration back."""
        buf = C.create_string_buffer(bytes(state), len(state))
        native.check(self._lib.oafdtd_restore(self._h, buf), "restore")

    def step_timed(self, n: int) -> float:
        """``step(n)``; returns the device time of its launches [ms] (CUDA events on the engine's
        own stream)."""
        if self.step_count + n > self.max_steps:
            raise ValueError("step count exceeds max_steps (wave table length)")
        ms = C.c_double()
        native.check(self._lib.oafdtd_step_timed(self._h, int(n), C.byref(ms)), "step_timed")
        return float(ms.value)

    def energy(self) -> float:
        out = C.c_double()
        native.check(self._lib.oafdtd_energy(self._h, C.byref(out)), "energy")
        return float(out.value)

    def results(self) -> dict[str, npt.NDArray[np.complex128]]:
        nf = self.c.frequencies.size
        buf = np.zeros((max(len(self._probes), 1), self.B, max(nf, 1), 2))
        native.check(self._lib.oafdtd_dft(self._h, _ptr(buf, C.c_double)), "dft")
        acc = buf[..., 0] + 1j * buf[..., 1]
        return {q["name"]: acc[pi, :, :nf].copy() for pi, q in enumerate(self._probes)}

    def series(self) -> dict[str, FloatArray]:
        if not self.record_series:
            return {}
        steps = self.step_count
        if steps == 0 or not self._probes:
            return {}
        buf = np.zeros((len(self._probes), self.B, steps))
        native.check(self._lib.oafdtd_series(self._h, _ptr(buf, C.c_double)), "series")
        return {q["name"]: buf[pi].copy() for pi, q in enumerate(self._probes)}

    def field(self, comp: int) -> FloatArray:
        out = np.zeros(self.shape)
        native.check(self._lib.oafdtd_fields(self._h, int(comp), _ptr(out, C.c_double)), "fields")
        return out

    def get_fields(self) -> dict[str, FloatArray]:
        names = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
        return {n: self.field(k) for k, n in enumerate(names)}

    # ------------------------------------------------------------------ z-slab decomposition
    def half_h(self) -> None:
        """The H half of a step (H update, CPML-H, ghosts, H probes), synchronised."""
        native.check(self._lib.oafdtd_step_half(self._h, 0), "step_half")

    def half_e(self) -> None:
        """The E half of a step (E update, CPML-E, Debye, SIBC, injection, E probes)."""
        native.check(self._lib.oafdtd_step_half(self._h, 1), "step_half")

    def plane(self, comp: int, k: int) -> FloatArray:
        """Component ``comp`` (0..5 = Ex..Hz) at storage plane ``k``, shape (B, y, x)."""
        out = np.zeros((self.B, self.shape[2], self.shape[3]))
        native.check(self._lib.oafdtd_plane(self._h, int(comp), int(k), _ptr(out, C.c_double)), "plane")
        return out

    def set_plane(self, comp: int, k: int, values: FloatArray) -> None:
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(values, np.float64), (self.B, self.shape[2], self.shape[3])))
        native.check(self._lib.oafdtd_set_plane(self._h, int(comp), int(k), _ptr(a, C.c_double)), "set_plane")

    def plane_to_device(self, comp: int, k: int, dst: int) -> None:
        """Copy plane ``k`` of ``comp`` into device memory at address ``dst`` (``B x y x x``
        values of the engine's precision, for example ``torch_tensor.data_ptr()``)."""
        native.check(self._lib.oafdtd_plane_device(self._h, int(comp), int(k), C.c_void_p(int(dst))), "plane_device")

    def plane_from_device(self, comp: int, k: int, src: int) -> None:
        """Overwrite plane ``k`` of ``comp`` from device memory at address ``src``."""
        native.check(self._lib.oafdtd_set_plane_device(self._h, int(comp), int(k), C.c_void_p(int(src))), "set_plane_device")

    def set_field(self, comp: int, values: FloatArray) -> None:
        """Overwrite one component (0..5 = Ex..Hz) with ``values`` of shape ``(B, z, y, x)``,
        rounded to the engine's precision. No counterpart in the reference engine."""
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(values, dtype=np.float64), self.shape))
        native.check(self._lib.oafdtd_set_field(self._h, int(comp), _ptr(a, C.c_double)), "set_field")

    def peak_bytes(self) -> int:
        out = C.c_int64()
        native.check(self._lib.oafdtd_peak_bytes(self._h, C.byref(out)), "peak_bytes")
        return int(out.value)

    # ------------------------------------------------------------------ tuning and profiling
    def set_graph(self, on: bool) -> None:
        native.check(self._lib.oafdtd_set_graph(self._h, int(bool(on))), "set_graph")

    def set_tuning(self, tile_z: int = 0, variant: int = -1) -> None:
        """Planes marched per block (0 keeps) and the sweep variant (3 the fused H + E sweep of
        the interior, 2 staged by TMA, 1 staged by cp.async, 0 register marching, -1 keeps)."""
        native.check(self._lib.oafdtd_set_tuning(self._h, int(tile_z), int(variant)), "set_tuning")

    def get_tuning(self) -> tuple[int, int]:
        """The current launch shape: (planes per block, sweep variant)."""
        tz, v = C.c_int32(), C.c_int32()
        native.check(self._lib.oafdtd_get_tuning(self._h, C.byref(tz), C.byref(v)), "get_tuning")
        return int(tz.value), int(v.value)

    def set_profiling(self, on: bool) -> None:
        native.check(self._lib.oafdtd_set_profiling(self._h, int(bool(on))), "set_profiling")

    KERNELS = ("h_sweep", "h_slab", "ghosts", "pre_e", "e_sweep", "e_slab", "edges", "probe_e", "fused", "step")

    def kernel_bytes(self) -> dict[str, float]:
        """Algorithmic DRAM bytes per time step of each kernel class (keys of ``kernel_times``;
        ``step`` is their sum) under the current sweep variant."""
        out = np.zeros(len(self.KERNELS))
        native.check(self._lib.oafdtd_kernel_bytes(self._h, _ptr(out, C.c_double), len(out)), "kernel_bytes")
        return dict(zip(self.KERNELS, out.tolist(), strict=True))

    def graph_kernels(self) -> int:
        """Kernel launches in one replay of the captured 64-step graph (0 before a capture)."""
        out = C.c_int64()
        native.check(self._lib.oafdtd_graph_kernels(self._h, C.byref(out)), "graph_kernels")
        return int(out.value)

    def kernel_times(self) -> dict[str, float]:
        """Average device ms per time step of each kernel class over the last ``step`` call."""
        out = np.zeros(len(self.KERNELS))
        native.check(self._lib.oafdtd_kernel_times(self._h, _ptr(out, C.c_double), len(out)), "kernel_times")
        return dict(zip(self.KERNELS, out.tolist(), strict=True))

    def model_bytes(self) -> float:
        """Algorithmic DRAM bytes of one time step under the engine's traffic model."""
        out = C.c_double()
        native.check(self._lib.oafdtd_model_bytes(self._h, C.byref(out)), "model_bytes")
        return float(out.value)

    def close(self) -> None:
        if self._h:
            self._lib.oafdtd_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass
