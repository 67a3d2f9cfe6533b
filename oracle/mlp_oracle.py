"""CPU oracle of the S-parameter surrogate's network: forward pass, backward pass and Adam in FP64.

TEST INFRASTRUCTURE ONLY. Nothing in the product (``open_analysis_gb300``) imports this module;
only ``tests/`` use it, as the checker of the GPU training kernels. It is never a fallback.

The reference has no learned surrogate, so there is no reference file to follow: this is the
published algorithm restated, a fully connected ReLU network trained by back-propagation on the
mean squared error with Adam (Kingma & Ba, "Adam: A Method for Stochastic Optimization", 2015,
Algorithm 1, with the bias corrections applied to the moments). Its own correctness is pinned by
central finite differences of the FP64 loss (``tests/test_surrogate.py``).

``bf16=True`` rounds at the points where the GPU stores BF16 (inputs, weights, hidden activations,
the loss gradient and the pre-activation gradients fed to the next GEMM), with IEEE
round-to-nearest-even, and sums in FP64: the GPU's FP32 accumulation then differs from it only by
summation rounding. ``bf16=False`` is the exact FP64 network.

Layout (the GPU's): weights ``W[l]`` of shape ``(fan_in, fan_out)``, ``Y = X @ W + b``.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import numpy.typing as npt

FloatArray = npt.NDArray[np.float64]


def bf16_round(x: npt.ArrayLike) -> FloatArray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


@dataclass
class Grads:
    loss: float
    dw: list[FloatArray]
    db: list[FloatArray]


def _act(z: FloatArray, act: str) -> FloatArray:
    return np.maximum(z, 0.0) if act == "relu" else np.tanh(z)


def _dact(a: FloatArray, act: str) -> FloatArray:
    """The activation's derivative, from its output ``a``."""
    return (a > 0.0).astype(np.float64) if act == "relu" else 1.0 - a * a


def forward(w: list[FloatArray], b: list[FloatArray], x: FloatArray, bf16: bool = True,
            act: str = "relu") -> tuple[FloatArray, list[FloatArray]]:
    """Output ``Y`` (no activation on the last layer) and the layer inputs (``acts[0] = x``);
    hidden activation ``act`` is ``"relu"`` or ``"tanh"``."""
    r = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    a = r(x)
    acts = [a]
    n = len(w)
    for l in range(n):
        z = a @ r(w[l]) + b[l]
        if l == n - 1:
            return (z.astype(np.float32).astype(np.float64) if bf16 else z), acts
        a = r(_act(z, act))
        acts.append(a)
    raise ValueError("empty network")


def loss_and_grads(w: list[FloatArray], b: list[FloatArray], x: FloatArray, t: FloatArray, bf16: bool = True,
                   act: str = "relu") -> Grads:
    """Mean squared error over all outputs and its gradients with respect to every W and b."""
    r = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    y, acts = forward(w, b, x, bf16, act)
    m, n_out = y.shape
    d = y - t
    loss = float(np.sum(d * d) / (m * n_out))
    g = 2.0 * d / (m * n_out)
    g16 = r(g)
    dw: list[FloatArray] = [np.empty(0)] * len(w)
    db: list[FloatArray] = [np.empty(0)] * len(w)
    g_full = g
    for l in range(len(w) - 1, -1, -1):
        dw[l] = acts[l].T @ g16
        db[l] = g_full.sum(axis=0)
        if l == 0:
            break
        da = g16 @ r(w[l]).T
        dz = da * _dact(acts[l], act)
        g_full, g16 = dz, r(dz)
    return Grads(loss, dw, db)


@dataclass
class AdamState:
    m1: list[FloatArray]
    m2: list[FloatArray]
    step: int = 0


def adam(params: list[FloatArray], grads: list[FloatArray], st: AdamState, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
    """One Adam step in place (Kingma & Ba 2015, Algorithm 1)."""
    st.step += 1
    c1, c2 = 1.0 - b1**st.step, 1.0 - b2**st.step
    for p, g, m1, m2 in zip(params, grads, st.m1, st.m2, strict=True):
        m1 *= b1
        m1 += (1.0 - b1) * g
        m2 *= b2
        m2 += (1.0 - b2) * g * g
        p -= lr * (m1 / c1) / (np.sqrt(m2 / c2) + eps)
