"""Learned S-parameter surrogate for via-transition sweeps, with the FDTD engine as fallback and judge.

The reference has no surrogate; this module extends its sweep path (parameters -> S-parameters),
built on the engine and judged by it:

* :func:`via_params` / :func:`via_instance` — a via transition with seven parameters (drill, pad,
  antipad, stack height, eps_inf, delta_eps of a single-pole Debye dielectric, stub length) drawn
  uniformly from a seed, on a fixed cell grid (default 200 x 200 x 120). Lateral sizes snap to
  whole 2-cell steps and vertical ones to whole cells *before* the model is built
  (:func:`meshed`), so the parameters the network sees are exactly the geometry FDTD simulates.
* :func:`generate` — S11 and S21 at every DFT frequency of many instances from the engine's
  batched runner (:func:`open_analysis_gb300.batch.run_batched`), host compiles overlapped with
  the GPU in a ``spawn`` process pool.
* :class:`Mlp` — the network (7 -> 512 x 6 tanh -> 4 F outputs: S11 and S21, real and
  imaginary parts, with the TEM line propagation divided out, :func:`line_factor`) trained on the
  GPU by the engine library's own kernels: BF16 tensor-core GEMMs with FP32 accumulation and fused
  bias / activation / activation-derivative epilogues, the MSE gradient, bias sums and Adam on
  FP32 master weights (``oafdtd_mlp_*`` in ``include/oafdtd.h``). One epoch of training steps is
  captured once as a CUDA graph and replayed. PyTorch only owns the device buffers and draws the
  epoch's shuffle.
* :class:`Ensemble` — eight independently initialised networks trained side by side (early
  stopping on a validation fold); their spread is the predicted uncertainty, scaled by a factor
  calibrated against FDTD on a calibration fold; :meth:`Ensemble.save` / :meth:`Ensemble.load`.
* :func:`surrogate_sweep` — answers a sweep: instances whose predicted error bound exceeds the
  tolerance (0.05 dB by default) are run by FDTD instead (the fallback), so every returned S is
  either FDTD's or predicted within the bound.

Error measure: ``20 log10(1 + max |S_pred - S_fdtd|)`` dB over both S-parameters and every
frequency, the largest change in dB that the complex error can make to a unit-scale S-parameter
(0.05 dB <=> |dS| <= 5.773e-3). It bounds the dB error of any S-parameter near 0 dB (the
transmission); near deep reflection nulls no absolute bound can bound the dB error, so the
measure is taken relative to full scale.
"""

from __future__ import annotations

import math
import time
from collections.abc import Sequence
from concurrent.futures import ProcessPoolExecutor
from dataclasses import dataclass, field
from multiprocessing import get_context
from typing import Any

import numpy as np
import numpy.typing as npt

from open_analysis_gb300 import native
from open_analysis_gb300.errors import AccelError, ErrorInfo
from open_analysis_gb300.grid import Grid, uniform_lines
from open_analysis_gb300.model import Conductor, LumpedPort, Model, Region, Waveform
from open_analysis_gb300.pml import CpmlSpec

FloatArray = npt.NDArray[np.float64]
ComplexArray = npt.NDArray[np.complex128]

PARAM_NAMES = ("drill", "pad", "antipad", "stack", "eps_inf", "delta_eps", "stub")
PARAM_RANGES = np.array(
    [
        (0.15e-3, 0.40e-3),
        (0.30e-3, 0.70e-3),
        (0.50e-3, 1.20e-3),
        (0.80e-3, 2.40e-3),
        (3.2, 4.5),
        (0.1, 0.5),
        (0.0, 1.60e-3),
    ]
)
BARREL = 0.5 / 0.5902  # square barrel side per drill diameter (the conformal radius of the drill)
TAU = 8e-12  # Debye relaxation time of the dielectric [s]
STRIP = 0.2e-3  # distance from each trace to its nearest plane [m]
TOL_DB = 0.05


def db_error(s_pred: npt.ArrayLike, s_ref: npt.ArrayLike, axis: Any = None) -> Any:
    """``20 log10(1 + max |s_pred - s_ref|)``: the error measure in dB (see the module doc)."""
    d = np.abs(np.asarray(s_pred) - np.asarray(s_ref))
    return 20.0 * np.log10(1.0 + d.max(axis=axis))


TOL_LIN = 10.0 ** (TOL_DB / 20.0) - 1.0


# ------------------------------------------------------------------------------------ structures
@dataclass(frozen=True)
class ViaGrid:
    """Cells per axis, lateral cell [m], vertical cell [m], DFT frequencies, CPML cells, the
    source pulse's delay in pulse widths, and the time simulated [s] (:attr:`steps`)."""

    nx: int = 200
    ny: int = 200
    nz: int = 120
    h: float = 25e-6
    dz: float = 40e-6
    n_freq: int = 256
    cpml: int = 10
    delay_tau: float = 4.0
    span: float = 450e-12

    def grid(self) -> Grid:
        return Grid(uniform_lines(self.nx, self.h), uniform_lines(self.ny, self.h), uniform_lines(self.nz, self.dz))

    @property
    def steps(self) -> int:
        """Time steps that cover :attr:`span` at the 0.95 Courant step of this grid."""
        return int(math.ceil(self.span / self.grid().dt(0.95)))

    def check(self) -> None:
        # the tallest stack plus the longest stub plus 10 cells above and 8 below must fit
        need = int(round(PARAM_RANGES[3, 1] / self.dz) + round(PARAM_RANGES[6, 1] / self.dz)) + 18
        if self.nz < need:
            raise ValueError(f"nz = {self.nz} cannot hold the tallest stack and stub ({need} cells)")


def via_params(n: int, seed: int = 4096) -> FloatArray:
    """``(n, 7)`` parameters drawn uniformly from :data:`PARAM_RANGES` (seeded)."""
    rng = np.random.default_rng(seed)
    lo, hi = PARAM_RANGES[:, 0], PARAM_RANGES[:, 1]
    return lo + (hi - lo) * rng.random((n, 7))


def meshed(p: npt.ArrayLike, g: ViaGrid = ViaGrid()) -> FloatArray:
    """The parameters as the mesh holds them: barrel side, pad and antipad in whole 2-cell steps
    (boxes centred on a node), stack height and stub in whole vertical cells; eps_inf and
    delta_eps unchanged. Works on one vector or an ``(n, 7)`` array."""
    q = np.array(p, dtype=np.float64, copy=True)
    two = 2.0 * g.h
    side = np.maximum(np.round(q[..., 0] * BARREL / two), 1.0) * two
    q[..., 0] = side / BARREL
    q[..., 1] = np.maximum(np.round(q[..., 1] / two), 1.0) * two
    q[..., 2] = np.maximum(np.round(q[..., 2] / two), 1.0) * two
    q[..., 3] = np.maximum(np.round(q[..., 3] / g.dz), 8.0) * g.dz
    q[..., 6] = np.round(q[..., 6] / g.dz) * g.dz
    return q


def via_instance(p: npt.ArrayLike, g: ViaGrid = ViaGrid()) -> Model:
    """One via transition: a stripline trace on the top layer, a via through three antipadded
    planes, a stripline trace on the bottom layer, and a via stub below it.

    z (from the top PEC wall down): top trace 10 cells below the wall; the bottom trace
    ``stack`` below it; the barrel continues ``stub`` below the bottom trace; the rest down to
    the bottom PEC wall is dielectric. The planes: one :data:`STRIP` below the top trace, one
    :data:`STRIP` above the bottom trace, one midway; so the ports' geometry does not change
    with the stack, only the core and the via do. Lateral walls are CPML. All copper (planes, pads, barrel,
    traces) is surface-impedance copper (sigma 5.8e7 S/m). Port 1 (driven) at the top trace's
    end, port 2 at the bottom trace's end, both 50 ohm.
    """
    g.check()
    q = meshed(p, g)
    drill, pad, antipad, stack, eps_inf, delta_eps, stub = (float(v) for v in q)
    h, dz = g.h, g.dz
    m = Model(
        g.grid(),
        Waveform("gauss_mod", 10.05e9, 19.9e9, delay_tau=g.delay_tau),
        np.linspace(0.1e9, 20e9, g.n_freq),
        walls=("cpml", "cpml", "cpml", "cpml", "pec", "pec"),
        cpml=CpmlSpec(cells=g.cpml),
        courant=0.95,
    )
    m.excite = ("p1",)
    z = lambda k: k * dz  # noqa: E731
    kt = g.nz - 10
    kb = kt - int(round(stack / dz))
    ks = kb - int(round(stub / dz))
    d1 = max(2, int(round(STRIP / dz)))  # each trace's reference plane, a fixed distance away
    planes = [kb + d1, (kb + kt) // 2, kt - d1]
    big = 1.0
    m.regions.append(Region((-big, -big, -big), (big, big, big), eps_inf, poles=((delta_eps, TAU),)))
    cx, cy = (g.nx // 2) * h, (g.ny // 2) * h
    cu = dict(sigma=5.8e7, thickness=35e-6)
    ha = 0.5 * antipad
    for k in planes:
        lo_z, hi_z = z(k), z(k + 1)
        for lo, hi in (
            ((-big, -big, lo_z), (cx - ha, big, hi_z)),
            ((cx + ha, -big, lo_z), (big, big, hi_z)),
            ((cx - ha, -big, lo_z), (cx + ha, cy - ha, hi_z)),
            ((cx - ha, cy + ha, lo_z), (cx + ha, big, hi_z)),
        ):
            m.conductors.append(Conductor(lo, hi, **cu))
    side = drill * BARREL
    m.conductors.append(Conductor((cx - side / 2, cy - side / 2, z(ks)), (cx + side / 2, cy + side / 2, z(kt + 1)), **cu))
    for k in (kb, kt):
        m.conductors.append(Conductor((cx - pad / 2, cy - pad / 2, z(k)), (cx + pad / 2, cy + pad / 2, z(k + 1)), **cu))
    w = 0.2e-3
    x1, x2 = (g.cpml + 4) * h, (g.nx - g.cpml - 4) * h
    m.conductors.append(Conductor((x1, cy - w / 2, z(kt)), (cx, cy + w / 2, z(kt + 1)), **cu))
    m.conductors.append(Conductor((cx, cy - w / 2, z(kb)), (x2, cy + w / 2, z(kb + 1)), **cu))
    m.ports.append(LumpedPort("p1", 2, (x1, cy, z(planes[2] + 1)), (x1, cy, z(kt)), 50.0))
    m.ports.append(LumpedPort("p2", 2, (x2, cy, z(kb + 1)), (x2, cy, z(planes[0])), 50.0))
    return m


# ------------------------------------------------------------------------------------ FDTD data
def _compile(args: tuple[FloatArray, ViaGrid, str]) -> Any:
    from open_analysis_gb300.model import compile_model

    p, g, dtype = args
    return compile_model(via_instance(p, g), dtype)


@dataclass
class Dataset:
    """Parameters as meshed ``(n, 7)``, ``S[n, 2, F]`` (S11, S21), the frequencies, and the
    seconds the engine spent (stepping + read-back; compiles and engine creation apart)."""

    params: FloatArray
    s: ComplexArray
    freqs: FloatArray
    seconds: float = 0.0
    create_seconds: float = 0.0
    compile_seconds: float = 0.0
    steps: int = 0
    extra: dict[str, Any] = field(default_factory=dict)

    def save(self, path: str) -> None:
        np.savez_compressed(path, params=self.params, s=self.s.astype(np.complex64), freqs=self.freqs,
                            seconds=self.seconds, steps=self.steps)

    @staticmethod
    def load(path: str) -> Dataset:
        """A saved dataset (its S-parameters were stored as complex64)."""
        d = np.load(path)
        return Dataset(d["params"], d["s"].astype(np.complex128), d["freqs"], float(d["seconds"]), steps=int(d["steps"]),
                       extra={"stored": "complex64"})

    def subset(self, idx: npt.ArrayLike) -> Dataset:
        i = np.asarray(idx)
        return Dataset(self.params[i], self.s[i], self.freqs, steps=self.steps, extra=dict(self.extra))

    def same_as(self, s: ComplexArray, idx: npt.ArrayLike | slice = slice(None)) -> bool:
        """Whether ``s`` equals these S-parameters (rows ``idx``) bit for bit, or after rounding to
        complex64 when they came from a saved file."""
        mine = self.s[idx]
        if self.extra.get("stored") == "complex64":
            return bool(np.array_equal(np.asarray(s).astype(np.complex64), mine.astype(np.complex64)))
        return bool(np.array_equal(s, mine))


def generate(
    params: npt.ArrayLike,
    g: ViaGrid = ViaGrid(),
    steps: int | None = None,
    chunk: int = 32,
    workers: int = 8,
    dtype: str = "float32",
    batched: bool = True,
    tune: bool = True,
) -> Dataset:
    """S11 and S21 of every instance from the GPU engine: ``chunk`` instances at a time through
    :func:`~open_analysis_gb300.batch.run_batched` (or ``run_looped`` with ``batched=False``),
    the next chunk compiling in the process pool meanwhile. With ``tune`` the launch shape comes
    from the autotuner once (:func:`~open_analysis_gb300.batch.tune_shape`, counted with the
    engine creation time). ``steps`` defaults to the grid's :attr:`ViaGrid.steps`."""
    from open_analysis_gb300.batch import run_batched, run_looped, tune_shape

    steps = g.steps if steps is None else int(steps)
    p = meshed(np.atleast_2d(np.asarray(params, dtype=np.float64)), g)
    n = p.shape[0]
    out = np.zeros((n, 2, g.n_freq), np.complex128)
    seconds = create = comp_wait = 0.0
    runner = run_batched if batched else run_looped
    shape = None
    chunks = [list(range(a, min(a + chunk, n))) for a in range(0, n, chunk)]
    with ProcessPoolExecutor(max_workers=max(1, workers), mp_context=get_context("spawn")) as pool:

        def submit(idx: list[int]) -> list[Any]:
            return [pool.submit(_compile, (p[i], g, dtype)) for i in idx]

        pending = submit(chunks[0]) if chunks else []
        for ci, idx in enumerate(chunks):
            t0 = time.perf_counter()
            compiled = [f.result() for f in pending]
            comp_wait += time.perf_counter() - t0
            pending = submit(chunks[ci + 1]) if ci + 1 < len(chunks) else []
            models = [via_instance(p[i], g) for i in idx]
            if shape is None and tune:
                t_tune = time.perf_counter()
                shape = tune_shape(compiled, dtype)
                create += time.perf_counter() - t_tune
            run = runner(models, compiled, steps, dtype, shape)
            seconds += run.seconds
            create += run.create_seconds
            for k, i in enumerate(idx):
                out[i, 0] = run.s[k][0, 0]
                out[i, 1] = run.s[k][1, 0]
    freqs = np.linspace(0.1e9, 20e9, g.n_freq)
    return Dataset(p, out, freqs, seconds, create, comp_wait, steps)


# ------------------------------------------------------------------------------------ network
def _torch() -> Any:
    import torch

    if not torch.cuda.is_available():
        raise AccelError(ErrorInfo("ACCEL_NO_DEVICE", "the surrogate trains on a CUDA device", "surrogate"))
    return torch


def _align(n: int, a: int = 64) -> int:
    return (n + a - 1) // a * a


# hidden activation -> (forward epilogue, backward epilogue) of oafdtd_mlp_gemm
ACTS = {"relu": (1, 2), "tanh": (3, 4)}


def cosine_lr(epoch: int, epochs: int, lr: float, lr_end: float) -> float:
    """Learning rate of ``epoch``: a half cosine from ``lr`` (first epoch) to ``lr_end`` (last)."""
    frac = epoch / max(1, epochs - 1)
    return lr_end + 0.5 * (lr - lr_end) * (1.0 + math.cos(math.pi * frac))


class Mlp:
    """``members`` tanh (or ReLU) networks ``sizes[0] -> ... -> sizes[-1]`` of the same widths on the
    GPU, trained side by side and evaluated by the engine library's kernels: every launch covers
    all members (the GEMMs are grouped, one Adam launch updates every parameter). Member ``k`` is
    initialised from seed ``seed + 101 k``.

    Weights ``W[l]`` are ``(fan_in, fan_out)`` FP32 masters with BF16 copies and transposed BF16
    copies the GEMMs read; a member's weights and biases live in one flat block of ``n_params``
    floats, the members' blocks side by side. Every GEMM is C = A . B^T with both operands
    K-contiguous (``oafdtd_mlp_gemm_tn``): the forward reads the transposed weights, the weight
    gradients the transposed activations and output gradients, which the epilogues and a small
    transpose kernel write. Problems with M a multiple of 128 and N, K multiples of 64 (batch 256,
    widths of 512) run on the tcgen05 tensor cores, all members in one persistent launch. Every
    width is padded to a multiple of 8 (the input with zero columns, so the extra weights see zero
    inputs and zero gradients)."""

    def __init__(self, sizes: Sequence[int], batch: int = 256, seed: int = 0, device: int = 0, act: str = "tanh",
                 members: int = 1) -> None:
        torch = _torch()
        self.torch = torch
        self.lib = native.load()
        if act not in ACTS:
            raise ValueError(f"activation {act!r}: one of {sorted(ACTS)}")
        if members < 1:
            raise ValueError("an ensemble has at least one member")
        self.act, self.dact = ACTS[act]
        self.act_name = act
        self.members = int(members)
        self.n_in = int(sizes[0])
        self.sizes = [_align(int(s), 8) for s in sizes]
        if self.sizes[1:] != [int(s) for s in sizes[1:]]:
            raise ValueError("hidden and output widths must be multiples of 8")
        self.batch = int(batch)
        self.dev = torch.device("cuda", device)
        self.layout: list[tuple[int, int, int, int]] = []  # (w offset, fan_in, fan_out, b offset)
        off = 0
        for a, b in zip(self.sizes[:-1], self.sizes[1:], strict=True):
            wo = off
            off = _align(off + a * b)
            self.layout.append((wo, a, b, off))
            off = _align(off + b)
        self.n_params = off
        flat = np.zeros((self.members, off), np.float32)
        n_layers = len(self.layout)
        gain = 2.0 if act == "relu" else 1.0  # He / Glorot-style variance per fan-in
        for k in range(self.members):
            rng = np.random.default_rng(seed + 101 * k)
            for l, (wo, a, b, _) in enumerate(self.layout):
                fan_in = self.n_in if l == 0 else a
                std = math.sqrt(gain / fan_in) if l < n_layers - 1 else math.sqrt(1.0 / fan_in) * 0.5
                w = (rng.standard_normal((a, b)) * std).astype(np.float32)
                if l == 0:
                    w[self.n_in :] = 0.0
                flat[k, wo : wo + a * b] = w.reshape(-1)
        f32, bf = torch.float32, torch.bfloat16
        self.p32 = torch.from_numpy(flat.reshape(-1)).to(self.dev)
        self.p16 = self.p32.to(bf)
        # every layer's BF16 weights also transposed, (fan_out, fan_in): the forward GEMM reads its
        # B operand K-contiguous, the layout the tcgen05 kernel takes
        self.p16T = torch.zeros_like(self.p16)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._refresh_t(self._stream())
        self.grad = torch.zeros(self.members * off, dtype=f32, device=self.dev)
        self.m1 = torch.zeros_like(self.grad)
        self.m2 = torch.zeros_like(self.grad)
        self.step_no = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.lr = torch.full((1,), 1e-3, dtype=f32, device=self.dev)
        self.gen = torch.Generator(device=self.dev)
        self.gen.manual_seed(seed + 1)
        self._train: dict[str, Any] | None = None
        self.graph: Any = None

    def pad(self, x: npt.ArrayLike) -> npt.NDArray[np.float32]:
        """Inputs ``(..., n, n_in)`` as ``(..., n, sizes[0])`` float32 with zero padding columns."""
        x = np.asarray(x, np.float32)
        out = np.zeros((*x.shape[:-1], self.sizes[0]), np.float32)
        out[..., : self.n_in] = x
        return out

    # ---- pointers (member 0; member k is k * n_params elements further on)
    def _w(self, l: int, half: bool = True) -> int:
        wo = self.layout[l][0]
        t = self.p16 if half else self.p32
        return t.data_ptr() + wo * t.element_size()

    def _wT(self, l: int) -> int:
        return self.p16T.data_ptr() + self.layout[l][0] * self.p16T.element_size()

    def _b(self, l: int) -> int:
        return self.p32.data_ptr() + self.layout[l][3] * 4

    def _gw(self, l: int) -> int:
        return self.grad.data_ptr() + self.layout[l][0] * 4

    def _gb(self, l: int) -> int:
        return self.grad.data_ptr() + self.layout[l][3] * 4

    def _stream(self) -> int:
        return int(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def flat(self, member: int = 0) -> Any:
        """Member ``member``'s FP32 parameters (a view of the device buffer)."""
        return self.p32[member * self.n_params : (member + 1) * self.n_params]

    def weights(self, member: int = 0) -> tuple[list[FloatArray], list[FloatArray]]:
        """A member's FP32 master weights and biases on the host (``W[l]`` is ``(fan_in, fan_out)``)."""
        flat = self.flat(member).detach().cpu().numpy().astype(np.float64)
        return self.split(flat)

    def set_weights(self, w: Sequence[FloatArray], b: Sequence[FloatArray], member: int = 0) -> None:
        flat = np.zeros(self.n_params, np.float32)
        for (wo, a, n, bo), wl, bl in zip(self.layout, w, b, strict=True):
            flat[wo : wo + a * n] = np.asarray(wl, np.float32).reshape(-1)
            flat[bo : bo + n] = np.asarray(bl, np.float32)
        self.flat(member).copy_(self.torch.from_numpy(flat).to(self.dev))
        self.load_flat(self.p32)

    def load_flat(self, flat32: Any, member: int | None = None) -> None:
        """Set the weights and biases from a flat FP32 device tensor: every member's (``member``
        None, the whole buffer) or one member's block; the BF16 and transposed copies follow."""
        if member is None:
            if flat32.data_ptr() != self.p32.data_ptr():
                self.p32.copy_(flat32)
        else:
            self.flat(member).copy_(flat32)
        self.p16.copy_(self.p32.to(self.torch.bfloat16))
        self._refresh_t(self._stream())

    # ---- kernels
    def _refresh_t(self, s: int) -> None:
        """The transposed BF16 weights from the current BF16 weights, every member."""
        p = self.n_params
        for l, (_, a, b, _) in enumerate(self.layout):
            native.check(self.lib.oafdtd_mlp_transpose(self._w(l), a, b, b, self._wT(l), a, self.members, p, p, s),
                         "transpose")

    def _gemm_tn(self, a: int, b: int, c32: int, c16: int, c16t: int, bias: int, mask: int, m: int, n: int, k: int,
                 lda: int, ldb: int, ldc: int, ldct: int, act: int, s: int, sa: int, sb: int, sc: int, sct: int,
                 sbias: int) -> None:
        """C_g (m x n) = A_g (m x k) . B_g^T with B_g (n x k) for every member g (the s* arguments:
        elements between members)."""
        native.check(self.lib.oafdtd_mlp_gemm_tn(a, b, c32 or None, c16 or None, c16t or None, bias or None,
                                                 mask or None, m, n, k, lda, ldb, ldc, ldct, act, 0.0, self.members,
                                                 sa, sb, sc, sct, sbias, self.status.data_ptr(), s),
                     "oafdtd_mlp_gemm_tn")

    def _forward(self, x16: int, acts: list[Any], y32: int, m: int, s: int, acts_t: list[Any] | None = None) -> None:
        """acts[l] (BF16, members x m x sizes[l+1]) for the hidden layers, and transposed into
        acts_t[l] (members x sizes[l+1] x m) when given (training: the weight gradients read
        them); y32 the FP32 output (members x m x sizes[-1]). x16: members x m x sizes[0]. Each
        layer is X . W = X . (W^T)^T on the transposed weights."""
        inp = x16
        n_layers = len(self.layout)
        p = self.n_params
        for l, (_, a, b, _) in enumerate(self.layout):
            last = l == n_layers - 1
            ct = 0 if last or acts_t is None else acts_t[l].data_ptr()
            self._gemm_tn(inp, self._wT(l), y32 if last else 0, 0 if last else acts[l].data_ptr(), ct, self._b(l), 0,
                          m, b, a, a, a, b, m, 0 if last else self.act, s, m * a, p, m * b, b * m, p)
            if not last:
                inp = acts[l].data_ptr()

    def _buffers(self, m: int) -> dict[str, Any]:
        torch = self.torch
        bf, f32 = torch.bfloat16, torch.float32
        g, out = self.members, self.sizes[-1]

        def z(*shape: int, dt: Any = bf) -> Any:
            return torch.zeros((g, *shape), dtype=dt, device=self.dev)

        return {
            "x16": z(m, self.sizes[0]),
            "x16T": z(self.sizes[0], m),
            "acts": [z(m, b) for b in self.sizes[1:-1]],
            "actsT": [z(b, m) for b in self.sizes[1:-1]],
            "g16T": z(out, m),
            "dz16T": [z(b, m) for b in self.sizes[1:-1]],
            "y": z(m, out, dt=f32),
            "t": z(m, out, dt=f32),
            "g32": z(m, out, dt=f32),
            "g16": z(m, out),
            "dz32": [z(m, b, dt=f32) for b in self.sizes[1:-1]],
            "dz16": [z(m, b) for b in self.sizes[1:-1]],
            "row_loss": z(m, dt=f32),
        }

    def _backward(self, buf: dict[str, Any], m: int, s: int) -> None:
        lib, g, p = self.lib, self.members, self.n_params
        y, t = buf["y"], buf["t"]
        out, n_in = self.sizes[-1], self.sizes[0]
        native.check(lib.oafdtd_mlp_mse_grad(y.data_ptr(), t.data_ptr(), g * m, out, buf["g32"].data_ptr(),
                                             buf["g16"].data_ptr(), buf["row_loss"].data_ptr(), g, s), "mse_grad")
        g32, g16, gT = buf["g32"].data_ptr(), buf["g16"].data_ptr(), buf["g16T"].data_ptr()
        native.check(lib.oafdtd_mlp_transpose(g16, m, out, out, gT, m, g, m * out, out * m, s), "transpose")
        native.check(lib.oafdtd_mlp_transpose(buf["x16"].data_ptr(), m, n_in, n_in, buf["x16T"].data_ptr(), m, g,
                                              m * n_in, n_in * m, s), "transpose")
        for l in range(len(self.layout) - 1, -1, -1):
            _, a, b, _ = self.layout[l]
            inp = buf["x16"].data_ptr() if l == 0 else buf["acts"][l - 1].data_ptr()
            inp_t = buf["x16T"].data_ptr() if l == 0 else buf["actsT"][l - 1].data_ptr()
            # dW = inp^T . g = (inp^T) . (g^T)^T  (a x b), from the transposed activations and g
            self._gemm_tn(inp_t, gT, self._gw(l), 0, 0, 0, 0, a, b, m, m, m, b, a, 0, s, a * m, b * m, p, 0, 0)
            native.check(lib.oafdtd_mlp_colsum(g32, m, b, b, self._gb(l), g, m * b, p, s), "colsum")
            if l == 0:
                break
            # dZ[l-1] = (g . W^T) times the activation's derivative at the layer input  (m x a);
            # W (a x b) is the B operand (N x K) as stored; the transposed dZ feeds layer l-1's dW
            dz32, dz16 = buf["dz32"][l - 1].data_ptr(), buf["dz16"][l - 1].data_ptr()
            dzt = buf["dz16T"][l - 1].data_ptr()
            self._gemm_tn(g16, self._w(l), dz32, dz16, dzt, 0, inp, m, a, b, b, b, a, m, self.dact, s,
                          m * b, p, m * a, a * m, 0)
            g32, g16, gT = dz32, dz16, dzt

    def _per_member(self, v: npt.ArrayLike) -> npt.NDArray[np.float32]:
        """Host rows ``(m, c)`` for every member alike, or ``(members, m, c)`` per member."""
        v = np.asarray(v, np.float32)
        if v.ndim == 2:
            v = np.broadcast_to(v, (self.members, *v.shape))
        if v.shape[0] != self.members:
            raise ValueError(f"{v.shape[0]} row sets for {self.members} members")
        return np.ascontiguousarray(v)

    def gradients(self, x: npt.ArrayLike, t: npt.ArrayLike) -> tuple[Any, FloatArray]:
        """Loss and the flat gradient buffer for one batch given on the host (checks and tests):
        ``x (m, n_in)`` and ``t (m, sizes[-1])`` for every member, or per member with a leading
        member axis. One member: ``(loss, flat)``; more: ``(losses[members], flat[members, n_params])``."""
        torch = self.torch
        x = self._per_member(self.pad(x))
        t = self._per_member(t)
        m = x.shape[1]
        buf = self._buffers(m)
        buf["x16"].copy_(torch.from_numpy(x).to(self.dev).to(torch.bfloat16))
        buf["t"].copy_(torch.from_numpy(t).to(self.dev))
        s = self._stream()
        self._forward(buf["x16"].data_ptr(), buf["acts"], buf["y"].data_ptr(), m, s, buf["actsT"])
        self._backward(buf, m, s)
        torch.cuda.synchronize(self.dev)
        self.check_status()
        losses = buf["row_loss"].sum(dim=1).cpu().numpy().astype(np.float64) / (m * self.sizes[-1])
        flat = self.grad.detach().cpu().numpy().astype(np.float64).reshape(self.members, self.n_params)
        if self.members == 1:
            return float(losses[0]), flat[0]
        return losses, flat

    def split(self, flat: FloatArray) -> tuple[list[FloatArray], list[FloatArray]]:
        """One member's flat buffer as per-layer ``(W, b)`` lists."""
        return ([flat[wo : wo + a * b].reshape(a, b) for wo, a, b, _ in self.layout],
                [flat[bo : bo + b] for _, _, b, bo in self.layout])

    def _adam(self, s: int, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
        lib = self.lib
        native.check(lib.oafdtd_mlp_count(self.step_no.data_ptr(), s), "count")
        native.check(lib.oafdtd_mlp_adam(self.p32.data_ptr(), self.p16.data_ptr(), self.grad.data_ptr(),
                                         self.m1.data_ptr(), self.m2.data_ptr(), self.members * self.n_params,
                                         self.lr.data_ptr(), b1, b2, eps, self.step_no.data_ptr(), s), "adam")
        self._refresh_t(s)

    def adam_step(self, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
        """One Adam step of every member on the current gradient buffer (the step number moves on
        by one)."""
        self.lr.fill_(lr)
        self._adam(self._stream(), b1, b2, eps)

    def check_status(self) -> None:
        """Raise when a bounded wait of a tcgen05 GEMM gave up since the last check (its result
        is incomplete); clears the word."""
        if int(self.status.item()) != 0:
            self.status.zero_()
            raise AccelError(ErrorInfo("ACCEL_TIMEOUT", "a tensor-core GEMM gave up waiting for its operands",
                                       "surrogate"))

    # ---- training
    def _train_step(self, tr: dict[str, Any], j: int, s: int) -> None:
        lib, m, g = self.lib, self.batch, self.members
        idx = tr["perm"].data_ptr() + j * g * m * 4
        buf = tr["buf"]
        native.check(lib.oafdtd_mlp_gather(tr["x"].data_ptr(), self.sizes[0], idx, g * m, None, buf["x16"].data_ptr(),
                                           s), "gather")
        native.check(lib.oafdtd_mlp_gather(tr["t"].data_ptr(), self.sizes[-1], idx, g * m, buf["t"].data_ptr(), None,
                                           s), "gather")
        self._forward(buf["x16"].data_ptr(), buf["acts"], buf["y"].data_ptr(), m, s, buf["actsT"])
        self._backward(buf, m, s)
        self._adam(s)

    def prepare(self, x: npt.ArrayLike, t: npt.ArrayLike, graph: bool = True,
                rows: Sequence[npt.ArrayLike] | None = None) -> None:
        """Upload the training set ``x (n, n_in)`` -> ``t (n, sizes[-1])`` (both already scaled)
        and capture one epoch of training steps as a CUDA graph. Every member draws its batches
        from all rows, or from its own subset ``rows[k]`` (bagging); an epoch is as many batches
        as the smallest subset holds."""
        torch = self.torch
        x = self.pad(x)
        t = np.asarray(t, np.float32)
        n = x.shape[0]
        subsets = [np.arange(n)] * self.members if rows is None else [np.asarray(r, np.int64) for r in rows]
        if len(subsets) != self.members:
            raise ValueError(f"{len(subsets)} row subsets for {self.members} members")
        nb = min(len(r) for r in subsets) // self.batch
        if nb < 1:
            raise ValueError(f"{min(len(r) for r in subsets)} training rows are fewer than one batch of {self.batch}")
        self.stream = torch.cuda.Stream(self.dev)
        tr = {
            "n": n,
            "nb": nb,
            "x": torch.from_numpy(x).to(self.dev),
            "t": torch.from_numpy(t).to(self.dev),
            "rows": [torch.from_numpy(r.astype(np.int64)).to(self.dev) for r in subsets],
            # batch j of member k: perm[j, k, :]
            "perm": torch.zeros((nb, self.members, self.batch), dtype=torch.int32, device=self.dev),
            "buf": self._buffers(self.batch),
        }
        self._train = tr
        self.graph = None
        if graph:
            self.stream.wait_stream(torch.cuda.current_stream(self.dev))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(self.stream):
                with torch.cuda.graph(g, stream=self.stream):
                    self._epoch()
            self.graph = g
        torch.cuda.synchronize(self.dev)

    def _epoch(self) -> None:
        tr = self._train
        assert tr is not None
        s = self._stream()
        for j in range(tr["nb"]):
            self._train_step(tr, j, s)

    def run_epoch(self, lr: float) -> None:
        """Queue one epoch on this network's stream: set the learning rate, draw every member's
        shuffle, replay the captured steps. Returns without waiting."""
        torch = self.torch
        tr = self._train
        assert tr is not None
        nb, m = tr["nb"], self.batch
        with torch.cuda.stream(self.stream):
            self.lr.fill_(lr)
            for k, r in enumerate(tr["rows"]):
                pick = r[torch.randperm(r.numel(), generator=self.gen, device=self.dev)[: nb * m]]
                tr["perm"][:, k, :].copy_(pick.view(nb, m).to(torch.int32))
            if self.graph is not None:
                self.graph.replay()
            else:
                self._epoch()

    def last_loss(self) -> Any:
        """Mean squared error of the last training batch, per member (a float for one member);
        waits for this network's stream."""
        tr = self._train
        assert tr is not None
        self.stream.synchronize()
        v = tr["buf"]["row_loss"].sum(dim=1).cpu().numpy().astype(np.float64) / (self.batch * self.sizes[-1])
        return float(v[0]) if self.members == 1 else v

    def fit(self, x: npt.ArrayLike, t: npt.ArrayLike, epochs: int, lr: float = 1e-3, lr_end: float = 1e-5,
            graph: bool = True, log_every: int = 0, rows: Sequence[npt.ArrayLike] | None = None) -> list[Any]:
        """Train: Adam, batches of ``batch`` rows drawn without replacement each epoch, learning
        rate along a cosine from ``lr`` to ``lr_end`` (:func:`cosine_lr`). Returns the last
        batch's loss at every ``log_every``-th epoch."""
        self.prepare(x, t, graph, rows)
        losses: list[Any] = []
        for e in range(epochs):
            self.run_epoch(cosine_lr(e, epochs, lr, lr_end))
            if log_every and (e % log_every == 0 or e == epochs - 1):
                losses.append(self.last_loss())
        self.torch.cuda.synchronize(self.dev)
        self.check_status()
        return losses

    def predict_device(self, x: npt.ArrayLike, chunk: int = 4096) -> Any:
        """Outputs for ``x (n, n_in)`` (scaled inputs) as an FP32 device tensor ``(members, n,
        sizes[-1])``."""
        torch = self.torch
        x = self.pad(x)
        n, g = x.shape[0], self.members
        out = torch.empty((g, n, self.sizes[-1]), dtype=torch.float32, device=self.dev)
        s = self._stream()
        for a in range(0, n, chunk):
            m = min(chunk, n - a)
            x16 = torch.from_numpy(x[a : a + m]).to(self.dev).to(torch.bfloat16).expand(g, m, -1).contiguous()
            acts = [torch.empty((g, m, b), dtype=torch.bfloat16, device=self.dev) for b in self.sizes[1:-1]]
            y = out[:, a : a + m] if g == 1 or n == m else torch.empty((g, m, self.sizes[-1]), dtype=torch.float32,
                                                                         device=self.dev)
            self._forward(x16.data_ptr(), acts, y.data_ptr(), m, s)
            if y.data_ptr() != out[:, a : a + m].data_ptr():
                out[:, a : a + m].copy_(y)
        self.check_status()
        return out

    def predict(self, x: npt.ArrayLike, chunk: int = 4096) -> FloatArray:
        """Outputs for ``x (n, n_in)`` (scaled inputs): ``(n, sizes[-1])`` for one member,
        ``(members, n, sizes[-1])`` for more; FP32 on the GPU, float64 on return."""
        out = self.predict_device(x, chunk).cpu().numpy().astype(np.float64)
        return out[0] if self.members == 1 else out


# ------------------------------------------------------------------------------------ ensemble
def scale_params(p: npt.ArrayLike) -> FloatArray:
    """Parameters -> [-1, 1] over :data:`PARAM_RANGES`."""
    lo, hi = PARAM_RANGES[:, 0], PARAM_RANGES[:, 1]
    return 2.0 * (np.asarray(p, np.float64) - lo) / (hi - lo) - 1.0


def s_to_rows(s: npt.ArrayLike) -> FloatArray:
    """``S[n, 2, F]`` complex -> ``(n, 4 F)`` real rows (S11 re, S11 im, S21 re, S21 im)."""
    s = np.asarray(s)
    return np.concatenate([s[:, 0].real, s[:, 0].imag, s[:, 1].real, s[:, 1].imag], axis=1)


def rows_to_s(y: npt.ArrayLike) -> ComplexArray:
    y = np.asarray(y)
    f = y.shape[1] // 4
    return np.stack([y[:, :f] + 1j * y[:, f : 2 * f], y[:, 2 * f : 3 * f] + 1j * y[:, 3 * f :]], axis=1)


@dataclass
class Prediction:
    s: ComplexArray          # ensemble mean, (n, 2, F)
    spread: FloatArray       # largest complex standard deviation over members, per instance
    bound_db: FloatArray     # predicted error bound in dB (calibrated spread)
    seconds: float


def line_factor(params: npt.ArrayLike, g: ViaGrid) -> ComplexArray:
    """``(n, 2, F)`` factors that remove the known TEM propagation along the striplines:
    ``exp(+2 j k L1)`` for S11 and ``exp(+j k (L1 + L2 + stack))`` for S21, with
    ``k = (w / c) sqrt(eps(w))`` of the single-pole Debye dielectric (``eps_inf + delta_eps /
    (1 + j w tau)``, the ``exp(+j w t)`` convention of the engine's DFT), ``L1`` and ``L2`` the
    trace lengths from the ports to the via and ``stack`` the via's height. What is left to learn
    (the via and port discontinuities) varies slowly with the parameters; the division is exact,
    and ``|1 / factor| <= 1``, so an error bound on the normalised S bounds the error on S."""
    from open_analysis_gb300.grid import C0

    q = np.atleast_2d(np.asarray(params, np.float64))
    w = 2.0 * np.pi * np.linspace(0.1e9, 20e9, g.n_freq)
    eps = q[:, 4:5] + q[:, 5:6] / (1.0 + 1j * w * TAU)
    k = w * np.sqrt(eps) / C0
    l1 = (g.nx // 2 - g.cpml - 4) * g.h
    l2 = (g.nx - g.cpml - 4 - g.nx // 2) * g.h
    return np.stack([np.exp(2j * k * l1), np.exp(1j * k * (l1 + l2 + q[:, 3:4]))], axis=1)


class Ensemble:
    """``members`` networks ``7 -> width x depth -> 4 F``, independently initialised and shuffled;
    the mean is the prediction, the members' spread (scaled by :attr:`scale`, calibrated against
    FDTD) the error bound. With ``bag < 1`` every member trains on its own random subset of that
    fraction of the training rows (bagging), so that the spread also carries the uncertainty of
    where the data lie. The networks learn S with the line propagation divided out
    (:func:`line_factor`), each column less its mean, all columns over one common scale (so that
    the loss weighs absolute errors in S alike)."""

    def __init__(self, g: ViaGrid, members: int = 8, width: int = 512, depth: int = 6, batch: int = 256, seed: int = 0,
                 act: str = "tanh", bag: float = 1.0) -> None:
        self.g = g
        self.bag = bag
        self.seed = seed
        self.sizes = [7] + [width] * depth + [4 * g.n_freq]
        self.net = Mlp(self.sizes, batch, seed=seed, act=act, members=members)
        self.mu = np.zeros(4 * g.n_freq)
        self.sigma = 1.0
        self.scale = 1.0
        self.train_seconds = 0.0
        self.val_scores: list[float] = []

    def fit(self, data: Dataset, epochs: int = 2000, lr: float = 1e-3, lr_end: float = 1e-5,
            val: Dataset | None = None, checks: int = 30) -> list[list[float]]:
        """Train every member on ``data``, side by side: one captured epoch covers all members
        (grouped GEMMs). With ``val``, every member is scored on it ``checks`` times along the way
        and keeps the weights of its best score (early stopping). Returns each member's training
        loss at those points."""
        rows = s_to_rows(data.s * line_factor(data.params, self.g))
        self.mu = rows.mean(axis=0)
        self.sigma = float(np.sqrt(np.mean((rows - self.mu) ** 2))) + 1e-9
        x = scale_params(data.params)
        t = (rows - self.mu) / self.sigma
        xv = tv = None
        if val is not None:
            xv = scale_params(val.params)
            tv = (s_to_rows(val.s * line_factor(val.params, self.g)) - self.mu) / self.sigma
        t0 = time.perf_counter()
        rng = np.random.default_rng(self.seed + 7)
        net, members = self.net, self.net.members
        rows = None
        if self.bag < 1.0:
            size = max(net.batch, int(self.bag * len(x)))
            rows = [np.sort(rng.choice(len(x), size=size, replace=False)) for _ in range(members)]
        net.prepare(x, t, rows=rows)
        logs: list[list[float]] = [[] for _ in range(members)]
        best = [math.inf] * members
        keep: list[Any] = [None] * members
        every = max(1, epochs // checks)
        for e in range(epochs):
            net.run_epoch(cosine_lr(e, epochs, lr, lr_end))
            if (e + 1) % every == 0 or e == epochs - 1:
                losses = np.atleast_1d(net.last_loss())  # waits for the training stream
                pred = net.predict(xv).reshape(members, *tv.shape) if xv is not None else None
                for k in range(members):
                    logs[k].append(float(losses[k]))
                    if pred is not None:
                        score = float(np.mean((pred[k] - tv) ** 2))
                        if score < best[k]:
                            best[k], keep[k] = score, net.flat(k).clone()
        net.stream.synchronize()
        for k in range(members):
            if keep[k] is not None:
                net.flat(k).copy_(keep[k])
        net.load_flat(net.p32)
        self.val_scores = best
        self.train_seconds = time.perf_counter() - t0
        return logs

    def raw(self, params: npt.ArrayLike) -> tuple[ComplexArray, FloatArray, float]:
        """The ensemble mean of S ``(n, 2, F)``, the largest complex standard deviation over the
        members per instance, and the seconds all of it took. The members' outputs stay on the
        GPU: scaling, the line factors, mean and spread run there in float64."""
        torch = self.net.torch
        t0 = time.perf_counter()
        params = np.atleast_2d(np.asarray(params, np.float64))
        n, f = len(params), self.g.n_freq
        y = self.net.predict_device(scale_params(params)).to(torch.float64)  # (members, n, 4 F)
        y = y * self.sigma + torch.from_numpy(np.asarray(self.mu, np.float64)).to(y.device)
        s11 = torch.complex(y[..., :f], y[..., f : 2 * f])
        s21 = torch.complex(y[..., 2 * f : 3 * f], y[..., 3 * f :])
        fac = torch.from_numpy(line_factor(params, self.g)).to(y.device)  # (n, 2, F)
        stack = torch.stack([s11, s21], dim=2) / fac  # (members, n, 2, F)
        mean = stack.mean(dim=0)
        dev = torch.sqrt((torch.abs(stack - mean) ** 2).mean(dim=0))  # complex std per (n, 2, F)
        spread = dev.reshape(n, -1).amax(dim=1)
        out = mean.cpu().numpy(), spread.cpu().numpy()
        return out[0], out[1], time.perf_counter() - t0

    def save(self, path: str) -> None:
        """Write the trained ensemble (grid, widths, activation, every member's FP32 weights,
        the target scaling and the calibrated scale) to an npz file."""
        g = self.g
        np.savez_compressed(
            path,
            grid=np.array([g.nx, g.ny, g.nz, g.n_freq, g.cpml]),
            cell=np.array([g.h, g.dz, g.delay_tau, g.span]),
            sizes=np.array(self.sizes),
            act=np.array(self.net.act_name),
            batch=np.array(self.net.batch),
            weights=self.net.p32.detach().cpu().numpy().reshape(self.net.members, self.net.n_params),
            mu=self.mu,
            sigma=np.array(self.sigma),
            scale=np.array(self.scale),
        )

    @staticmethod
    def load(path: str) -> Ensemble:
        """An ensemble written by :meth:`save`, ready to predict (on the current CUDA device)."""
        d = np.load(path)
        nx, ny, nz, n_freq, cpml = (int(v) for v in d["grid"])
        h, dz, delay_tau, span = (float(v) for v in d["cell"])
        g = ViaGrid(nx=nx, ny=ny, nz=nz, h=h, dz=dz, n_freq=n_freq, cpml=cpml, delay_tau=delay_tau, span=span)
        sizes = [int(v) for v in d["sizes"]]
        act = str(d["act"])
        w = d["weights"]
        ens = Ensemble(g, members=w.shape[0], width=sizes[1], depth=len(sizes) - 2, batch=int(d["batch"]), act=act)
        if ens.sizes != sizes:
            raise ValueError(f"{path}: layer widths {sizes} are not an ensemble of this kind")
        net = ens.net
        if w.shape[1] != net.n_params:
            raise ValueError(f"{path}: {w.shape[1]} weights a member where the network holds {net.n_params}")
        net.load_flat(net.torch.from_numpy(w.reshape(-1).astype(np.float32)).to(net.dev))
        ens.mu, ens.sigma, ens.scale = d["mu"], float(d["sigma"]), float(d["scale"])
        return ens

    def calibrate(self, data: Dataset, quantile: float = 1.0) -> float:
        """Scale the spread so that it bounds the true error (FDTD's) on ``data``: the
        ``quantile`` of error / spread over the instances (1.0: the largest)."""
        mean, spread, _ = self.raw(data.params)
        err = np.abs(mean - data.s).reshape(len(data.s), -1).max(axis=1)
        self.scale = float(np.quantile(err / np.maximum(spread, 1e-12), quantile))
        return self.scale

    def predict(self, params: npt.ArrayLike) -> Prediction:
        mean, spread, sec = self.raw(params)
        return Prediction(mean, spread, 20.0 * np.log10(1.0 + self.scale * spread), sec)


@dataclass
class SweepAnswer:
    """S of every instance, which came from FDTD, and the time of each part [s]."""

    s: ComplexArray
    fdtd: npt.NDArray[np.bool_]
    predict_seconds: float
    fdtd_seconds: float
    fdtd_create_seconds: float

    @property
    def seconds(self) -> float:
        return self.predict_seconds + self.fdtd_seconds + self.fdtd_create_seconds


def surrogate_sweep(ens: Ensemble, params: npt.ArrayLike, g: ViaGrid = ViaGrid(), steps: int | None = None,
                    tol_db: float = TOL_DB, chunk: int = 32) -> SweepAnswer:
    """Answer a sweep: the ensemble's prediction where its calibrated bound is within ``tol_db``,
    the engine's batched FDTD everywhere else (``steps`` as the ensemble's data: by default the
    grid's :attr:`ViaGrid.steps`)."""
    p = meshed(np.atleast_2d(np.asarray(params, np.float64)), g)
    pred = ens.predict(p)
    out = pred.s.copy()
    fb = pred.bound_db > tol_db
    fsec = fcreate = 0.0
    if fb.any():
        d = generate(p[fb], g, steps, chunk=chunk)
        out[fb] = d.s
        fsec, fcreate = d.seconds, d.create_seconds
    return SweepAnswer(out, fb, pred.seconds, fsec, fcreate)


# ------------------------------------------------------------------------------------ experiment
HALF = ViaGrid(nx=100, ny=100, nz=70, h=50e-6, dz=80e-6, n_freq=256, cpml=8, span=560e-12)


def experiment(
    g: ViaGrid,
    n: int,
    seed: int = 4096,
    fixed: dict[str, float] | None = None,
    split: tuple[float, float, float] = (0.8, 0.05, 0.05),
    members: int = 8,
    width: int = 512,
    depth: int = 6,
    batch: int = 256,
    epochs: int = 3000,
    lrs: Sequence[float] = (1e-3, 3e-4),
    act: str = "tanh",
    bag: float = 1.0,
    quantile: float = 1.0,
    tol_db: float = TOL_DB,
    plain_sample: int = 32,
    chunk: int = 64,
    workers: int = 12,
    data: Dataset | None = None,
) -> dict[str, Any]:
    """The surrogate's whole cycle on via transitions, judged by FDTD.

    Generate ``n`` instances with the batched engine (or take ``data``); split them in order into
    training, validation, calibration and held-out folds (``split`` gives the first three
    fractions); train one ensemble per learning rate in ``lrs`` with early stopping on the
    validation fold and keep the one that scores best there; calibrate its bound on the
    calibration fold; answer the held-out fold with :func:`surrogate_sweep` and judge every
    answer against FDTD; time a loop of the plain engine over ``plain_sample`` held-out
    instances. Parameters named in ``fixed`` are held at the given value. Returns a report of
    plain numbers."""
    p = via_params(n, seed)
    for name, v in (fixed or {}).items():
        p[:, PARAM_NAMES.index(name)] = v
    steps = g.steps
    t0 = time.perf_counter()
    if data is None:
        data = generate(p, g, steps, chunk=chunk, workers=workers)
    gen_wall = time.perf_counter() - t0
    n_tr, n_val, n_cal = (int(f * n) for f in split)
    train = data.subset(range(n_tr))
    val = data.subset(range(n_tr, n_tr + n_val))
    cal = data.subset(range(n_tr + n_val, n_tr + n_val + n_cal))
    test = data.subset(range(n_tr + n_val + n_cal, n))
    ens, logs, chosen, train_seconds = None, None, None, 0.0
    for rate in lrs:
        cand = Ensemble(g, members=members, width=width, depth=depth, batch=batch, seed=seed, act=act, bag=bag)
        lg = cand.fit(train, epochs=epochs, lr=rate, lr_end=rate / 50, val=val)
        train_seconds += cand.train_seconds
        if ens is None or np.mean(cand.val_scores) < np.mean(ens.val_scores):
            ens, logs, chosen = cand, lg, rate
    assert ens is not None and logs is not None
    # the gate at several calibration quantiles, judged on the held-out fold (no FDTD needed:
    # its answers are known); the sweep below runs with ``quantile``
    cal_mean, cal_spread, _ = ens.raw(cal.params)
    ratio = np.abs(cal_mean - cal.s).reshape(len(cal.s), -1).max(axis=1) / np.maximum(cal_spread, 1e-12)
    raw_mean, raw_spread, _ = ens.raw(test.params)
    raw_db = db_error(raw_mean, test.s, axis=(1, 2))
    gates = {}
    for q in sorted({1.0, 0.98, 0.95, 0.9, quantile}, reverse=True):
        sc = float(np.quantile(ratio, q))
        ok = 20.0 * np.log10(1.0 + sc * raw_spread) <= tol_db
        gates[f"{q:g}"] = {"scale": sc, "accepted": float(ok.mean()), "violations": int(np.sum(raw_db[ok] > tol_db)),
                           "accepted_worst_db": float(raw_db[ok].max()) if ok.any() else None}
    ens.calibrate(cal, quantile)
    ans = surrogate_sweep(ens, test.params, g, steps, tol_db=tol_db, chunk=chunk)
    if not test.same_as(ans.s[ans.fdtd], ans.fdtd):
        raise RuntimeError("the FDTD fallback did not reproduce the engine's own S-parameters")
    err_db = db_error(ans.s, test.s, axis=(1, 2))
    k = min(plain_sample, len(test.s))
    # the fallback above and this loop both take their launch shape from the autotuner
    plain = generate(test.params[:k], g, steps, chunk=chunk, workers=workers, batched=False)
    if not test.same_as(plain.s, slice(0, k)):
        raise RuntimeError("the plain engine and the batched engine disagree")
    plain_rate = k / (plain.seconds + plain.create_seconds)
    # the network's own rate: every member on a large batch of new parameter points
    probe = via_params(8192, seed + 1)
    ens.raw(probe[:256])  # first call pays for allocations
    t_net = time.perf_counter()
    ens.raw(probe)
    net_rate = probe.shape[0] / (time.perf_counter() - t_net)
    batched_rate = n / (data.seconds + data.create_seconds) if data.seconds else float("nan")
    sur_rate = len(test.s) / ans.seconds
    acc = ~ans.fdtd
    return {
        "grid": [g.nx, g.ny, g.nz],
        "cells": [g.h, g.h, g.dz],
        "steps": steps,
        "n": n,
        "seed": seed,
        "fixed": fixed or {},
        "folds": {"train": n_tr, "val": n_val, "cal": n_cal, "test": len(test.s)},
        "network": ens.sizes,
        "activation": act,
        "members": members,
        "bag": bag,
        "gates": gates,
        "batch": batch,
        "epochs": epochs,
        "lr": chosen,
        "val_scores": ens.val_scores,
        "train_seconds": train_seconds,
        "final_loss": [lg[-1] for lg in logs],
        "scale": ens.scale,
        "tol_db": tol_db,
        "accepted": float(acc.mean()),
        "accepted_worst_db": float(err_db[acc].max()) if acc.any() else None,
        "answers_within_tol": float(np.mean(err_db <= tol_db)),
        "answers_worst_db": float(err_db.max()),
        "network_alone_worst_db": float(raw_db.max()),
        "network_alone_median_db": float(np.median(raw_db)),
        "network_alone_within_tol": float(np.mean(raw_db <= tol_db)),
        "spread_median": float(np.median(raw_spread)),
        "generate_wall_seconds": gen_wall,
        "generate_engine_seconds": data.seconds + data.create_seconds,
        "plain_sweeps_per_s": plain_rate,
        "batched_sweeps_per_s": batched_rate,
        "surrogate_sweeps_per_s": sur_rate,
        "network_sweeps_per_s": net_rate,
        "surrogate_seconds": {"predict": ans.predict_seconds, "fdtd": ans.fdtd_seconds, "create": ans.fdtd_create_seconds},
        "gain_vs_plain": sur_rate / plain_rate,
        "gain_vs_batched": sur_rate / batched_rate if batched_rate == batched_rate else None,
    }


# (groups, M, N, K): one member's training GEMM, the 8-member ensemble's grouped one, and larger
GEMM_SHAPES = ((1, 256, 512, 512), (8, 256, 512, 512), (8, 512, 512, 256), (1, 4096, 512, 512),
               (1, 65536, 512, 512), (1, 65536, 1024, 512), (1, 16384, 4096, 4096))


def gemm_rates(shapes: Sequence[tuple[int, int, int, int]] = GEMM_SHAPES, reps: int = 20) -> list[dict[str, Any]]:
    """Time the two GEMM kernels on BF16 A (M x K) and B + bias, tanh, BF16 out, per group, with
    CUDA events over ``reps`` launches after three warm-up launches, and check them against the
    FP32 product: ``oafdtd_mlp_gemm`` (mma.sync, B as K x N, one launch per group) and
    ``oafdtd_mlp_gemm_tn`` (B as N x K; tcgen05 where the shape allows, all groups in one launch).
    Returns per shape and kernel the microseconds per call, TFLOP/s and the largest error."""
    torch = _torch()
    lib = native.load()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0)
    out = []
    for groups, m, n, k in shapes:
        a = torch.randn(groups, m, k, device="cuda", generator=gen).to(torch.bfloat16)
        b = torch.randn(groups, k, n, device="cuda", generator=gen).to(torch.bfloat16)
        bt = b.transpose(1, 2).contiguous()
        c = torch.empty(groups, m, n, device="cuda", dtype=torch.bfloat16)
        bias = torch.zeros(groups, n, device="cuda")
        s = int(torch.cuda.current_stream().cuda_stream)

        def mma_sync() -> None:
            for gi in range(groups):
                native.check(lib.oafdtd_mlp_gemm(a[gi].data_ptr(), b[gi].data_ptr(), None, c[gi].data_ptr(),
                                                 bias[gi].data_ptr(), None, m, n, k, k, n, n, 0, 0, 3, 0.0, s),
                             "oafdtd_mlp_gemm")

        def tcgen05() -> None:
            native.check(lib.oafdtd_mlp_gemm_tn(a.data_ptr(), bt.data_ptr(), None, c.data_ptr(), None, bias.data_ptr(),
                                                None, m, n, k, k, k, n, m, 3, 0.0, groups, m * k, n * k, m * n, 0, n,
                                                None, s), "oafdtd_mlp_gemm_tn")

        want = torch.tanh(torch.bmm(a.float(), b.float()))
        for name, launch in (("mma_sync", mma_sync), ("gemm_tn", tcgen05)):
            for _ in range(3):
                launch()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record()
            for _ in range(reps):
                launch()
            t1.record()
            torch.cuda.synchronize()
            us = 1e3 * t0.elapsed_time(t1) / reps
            err = float((c.float() - want).abs().max().item())
            out.append({"kernel": name, "groups": groups, "m": m, "n": n, "k": k, "us": us,
                        "tflops": 2.0 * groups * m * n * k / us / 1e6, "max_err": err})
    return out


def main(argv: Sequence[str] | None = None) -> int:
    """``python -m open_analysis_gb300.surrogate [--n N] [--grid full|half] [--out report.json]
    [--data dataset.npz] [--save dataset.npz]``: the surrogate experiment on via transitions;
    ``--gemm-rates``: the GEMM's throughput by shape."""
    import argparse
    import json

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--grid", choices=["full", "half"], default="half")
    ap.add_argument("--seed", type=int, default=4096)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--members", type=int, default=8)
    ap.add_argument("--bag", type=float, default=1.0)
    ap.add_argument("--quantile", type=float, default=1.0)
    ap.add_argument("--data", default="", help="reuse a dataset written by --save")
    ap.add_argument("--save", default="", help="write the generated dataset (npz)")
    ap.add_argument("--out", default="")
    ap.add_argument("--gemm-rates", action="store_true", help="time the training GEMM by shape and exit")
    a = ap.parse_args(argv)
    if a.gemm_rates:
        for r in gemm_rates():
            print(json.dumps(r))
        return 0
    g = ViaGrid(span=560e-12) if a.grid == "full" else HALF
    data = Dataset.load(a.data) if a.data else None
    if data is None and a.save:
        p = via_params(a.n, a.seed)
        data = generate(p, g, g.steps, chunk=64, workers=12)
        data.save(a.save)
    rep = experiment(g, a.n, a.seed, epochs=a.epochs, members=a.members, bag=a.bag, quantile=a.quantile, data=data)
    rep["dataset"] = a.data or a.save or None
    text = json.dumps(rep, indent=1)
    print(text)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
