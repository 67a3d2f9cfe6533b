"""The surrogate's GPU kernels against the CPU oracle, and what the trained network gains.

* GEMM: BF16 operands with FP32 accumulation against FP64 sums of the same BF16 values, every
  transpose combination, ragged sizes, each epilogue; the same for the K-major entry point
  (``oafdtd_mlp_gemm_tn``) on tcgen05 tile shapes and on ragged shapes it hands to the fallback,
  with its transposed BF16 output; the transpose kernel.
* One training batch at tcgen05 shapes (batch 256, widths 512): loss and gradients against the
  oracle.
* One training batch: loss and every weight and bias gradient against ``oracle/mlp_oracle.py``
  (rounded to BF16 where the GPU stores BF16), and against the exact FP64 network (stated).
* Adam: one step against the oracle's.
* The gain test: a small via-transition sweep generated by the engine trains an ensemble; on
  held-out instances the surrogate answers where its calibrated bound allows, FDTD elsewhere; the
  answers are judged against FDTD and the sweep rate compared with looping the plain engine.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle.mlp_oracle import AdamState, adam, bf16_round, loss_and_grads

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lib():  # type: ignore[no-untyped-def]
    from open_analysis_gb300 import native

    return native.load()


def _dev(a: np.ndarray, dtype):  # type: ignore[no-untyped-def]
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda().to(dtype)


# ragged (scalar staging); multiples of 8 with 32-row tiles; enough tiles for 64-row tiles
SHAPES = [(77, 134, 203), (96, 136, 264), (1024, 1280, 72)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("act", [0, 1, 2, 3, 4])
def test_gemm_matches_fp64_sums_of_bf16_operands(shape: tuple[int, int, int], ta: int, tb: int, act: int) -> None:
    lib = _lib()
    rng = np.random.default_rng(10 * ta + tb + 100 * act + shape[0])
    m, n, k = shape
    a = bf16_round(rng.standard_normal((k, m) if ta else (m, k)))
    b = bf16_round(rng.standard_normal((n, k) if tb else (k, n)))
    bias = rng.standard_normal(n).astype(np.float32)
    mask = bf16_round(rng.standard_normal((m, n)))
    ref = (a.T if ta else a) @ (b.T if tb else b) + bias
    if act == 1:
        ref = np.maximum(ref, 0)
    if act == 2:
        ref = np.where(mask > 0, ref, 0)
    if act == 3:
        ref = np.tanh(ref)
    if act == 4:
        ref = ref * (1.0 - mask * mask)
    da, db_ = _dev(a, torch.bfloat16), _dev(b, torch.bfloat16)
    dbias, dmask = _dev(bias, torch.float32), _dev(mask, torch.bfloat16)
    c32 = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    c16 = torch.zeros((m, n), dtype=torch.bfloat16, device="cuda")
    rc = lib.oafdtd_mlp_gemm(da.data_ptr(), db_.data_ptr(), c32.data_ptr(), c16.data_ptr(), dbias.data_ptr(),
                             dmask.data_ptr(), m, n, k, a.shape[1], b.shape[1], n, ta, tb, act, 0.0, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = c32.cpu().numpy().astype(np.float64)
    scale = np.sqrt(k) * 4 * (1.0 if act != 4 else np.abs(mask).max() ** 2 + 1.0)
    assert np.abs(got - ref).max() <= 2e-6 * scale
    np.testing.assert_array_equal(c16.float().cpu().numpy(), bf16_round(got))


def test_gemm_rejects_bad_arguments() -> None:
    lib = _lib()
    x = torch.zeros(16, dtype=torch.bfloat16, device="cuda")
    assert lib.oafdtd_mlp_gemm(x.data_ptr(), x.data_ptr(), None, None, None, None, 4, 4, 4, 4, 4, 4, 0, 0, 0, 0.0, None) == -1
    y = torch.zeros(16, dtype=torch.float32, device="cuda")
    assert lib.oafdtd_mlp_gemm(x.data_ptr(), x.data_ptr(), y.data_ptr(), None, None, None, 4, 4, 4, 4, 4, 4, 0, 0, 2, 0.0, None) == -1


# tcgen05 tiles (M, N multiples of 128, K of 64) and ragged shapes the fallback takes
TN_SHAPES = [(256, 512, 512), (128, 128, 64), (256, 1024, 512), (384, 256, 192), (77, 134, 203), (256, 512, 8)]


@pytest.mark.parametrize("shape", TN_SHAPES)
@pytest.mark.parametrize("act", [0, 2, 3, 4])
def test_gemm_tn_matches_fp64_sums_of_bf16_operands(shape: tuple[int, int, int], act: int) -> None:
    """C = A . B^T with A (M x K) and B (N x K), both K-contiguous: FP32 C, BF16 C and its
    transpose, each epilogue; the status word stays zero."""
    lib = _lib()
    rng = np.random.default_rng(1000 + act + shape[0] + shape[2])
    m, n, k = shape
    a = bf16_round(rng.standard_normal((m, k)))
    b = bf16_round(rng.standard_normal((n, k)))
    bias = rng.standard_normal(n).astype(np.float32)
    mask = bf16_round(rng.standard_normal((m, n)))
    ref = a @ b.T + bias
    if act == 2:
        ref = np.where(mask > 0, ref, 0)
    if act == 3:
        ref = np.tanh(ref)
    if act == 4:
        ref = ref * (1.0 - mask * mask)
    da, db_ = _dev(a, torch.bfloat16), _dev(b, torch.bfloat16)
    dbias, dmask = _dev(bias, torch.float32), _dev(mask, torch.bfloat16)
    c32 = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    c16 = torch.zeros((m, n), dtype=torch.bfloat16, device="cuda")
    c16t = torch.zeros((n, m), dtype=torch.bfloat16, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.oafdtd_mlp_gemm_tn(da.data_ptr(), db_.data_ptr(), c32.data_ptr(), c16.data_ptr(), c16t.data_ptr(),
                                dbias.data_ptr(), dmask.data_ptr(), m, n, k, k, k, n, m, act, 0.0, 1, 0, 0, 0, 0, 0,
                                status.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = c32.cpu().numpy().astype(np.float64)
    scale = np.sqrt(k) * 4 * (1.0 if act != 4 else np.abs(mask).max() ** 2 + 1.0)
    assert np.abs(got - ref).max() <= 2e-6 * scale
    np.testing.assert_array_equal(c16.float().cpu().numpy(), bf16_round(got))
    np.testing.assert_array_equal(c16t.float().cpu().numpy(), c16.float().cpu().numpy().T)


def test_transpose16() -> None:
    lib = _lib()
    rng = np.random.default_rng(4)
    for rows, cols in ((256, 512), (77, 134), (8, 1024)):
        x = _dev(rng.standard_normal((rows, cols)), torch.bfloat16)
        y = torch.zeros((cols, rows), dtype=torch.bfloat16, device="cuda")
        assert lib.oafdtd_mlp_transpose(x.data_ptr(), rows, cols, cols, y.data_ptr(), rows, 1, 0, 0, None) == 0
        torch.cuda.synchronize()
        assert torch.equal(y, x.t())
    xs = _dev(rng.standard_normal((3, 64, 40)), torch.bfloat16)
    ys = torch.zeros((3, 40, 64), dtype=torch.bfloat16, device="cuda")
    assert lib.oafdtd_mlp_transpose(xs.data_ptr(), 64, 40, 40, ys.data_ptr(), 64, 3, 64 * 40, 40 * 64, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(ys, xs.transpose(1, 2))


# (groups, M, N, K): 64-column tcgen05 tiles (few tiles), 128-column ones with several tiles per CTA
# (512 tiles), and a ragged shape on the mma.sync kernels
GROUPED = [(8, 256, 512, 512), (3, 128, 192, 128), (16, 512, 1024, 128), (4, 72, 40, 24)]


@pytest.mark.parametrize("shape", GROUPED)
@pytest.mark.parametrize("act", [3, 4])
def test_grouped_gemm_tn_matches_each_group(shape: tuple[int, int, int, int], act: int) -> None:
    """Every group of one grouped launch against its own FP64 product, with padding between the
    groups' blocks (the strides are larger than the blocks) left untouched."""
    lib = _lib()
    groups, m, n, k = shape
    rng = np.random.default_rng(77 + groups + act)
    pad_a, pad_b, pad_c = 64, 128, 256  # elements between one group's block and the next
    sa, sb, sc, sct, sbias = m * k + pad_a, n * k + pad_b, m * n + pad_c, n * m + pad_c, n + 64
    a = bf16_round(rng.standard_normal((groups, sa)))
    b = bf16_round(rng.standard_normal((groups, sb)))
    bias = rng.standard_normal((groups, sbias)).astype(np.float32)
    mask = bf16_round(rng.standard_normal((groups, sc)))
    da, db_ = _dev(a, torch.bfloat16), _dev(b, torch.bfloat16)
    dbias, dmask = _dev(bias, torch.float32), _dev(mask, torch.bfloat16)
    c32 = torch.full((groups, sc), 7.0, dtype=torch.float32, device="cuda")
    c16 = torch.full((groups, sc), 7.0, dtype=torch.bfloat16, device="cuda")
    c16t = torch.full((groups, sct), 7.0, dtype=torch.bfloat16, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.oafdtd_mlp_gemm_tn(da.data_ptr(), db_.data_ptr(), c32.data_ptr(), c16.data_ptr(), c16t.data_ptr(),
                                dbias.data_ptr(), dmask.data_ptr(), m, n, k, k, k, n, m, act, 0.0, groups, sa, sb, sc,
                                sct, sbias, status.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got32 = c32.cpu().numpy().astype(np.float64)
    got16 = c16.float().cpu().numpy()
    got16t = c16t.float().cpu().numpy()
    for gi in range(groups):
        ag = a[gi, : m * k].reshape(m, k)
        bg = b[gi, : n * k].reshape(n, k)
        ref = ag @ bg.T + bias[gi, :n]
        mk = mask[gi, : m * n].reshape(m, n)
        ref = np.tanh(ref) if act == 3 else ref * (1.0 - mk * mk)
        scale = np.sqrt(k) * 4 * (1.0 if act != 4 else np.abs(mk).max() ** 2 + 1.0)
        g32 = got32[gi, : m * n].reshape(m, n)
        assert np.abs(g32 - ref).max() <= 2e-6 * scale, gi
        np.testing.assert_array_equal(got16[gi, : m * n].reshape(m, n), bf16_round(g32))
        np.testing.assert_array_equal(got16t[gi, : m * n].reshape(n, m), bf16_round(g32).T)
        assert np.all(got32[gi, m * n :] == 7.0) and np.all(got16[gi, m * n :] == 7.0)
        assert np.all(got16t[gi, m * n :] == 7.0)


def test_grouped_training_batch_matches_the_oracle_per_member() -> None:
    """Three members in one grouped network, each on its own batch: every member's loss and
    gradients against the oracle run on that member's weights and rows alone."""
    from open_analysis_gb300.surrogate import Mlp

    net = Mlp([7, 512, 512, 128], batch=256, seed=5, act="tanh", members=3)
    rng = np.random.default_rng(9)
    x = rng.uniform(-1, 1, (3, 256, 7))
    t = rng.standard_normal((3, 256, 128))
    losses, flat = net.gradients(x, t)
    assert flat.shape == (3, net.n_params)
    for k in range(3):
        w, b = net.weights(k)
        ref = loss_and_grads(w, b, net.pad(x[k]), t[k].astype(np.float32), bf16=True, act="tanh")
        assert abs(losses[k] - ref.loss) <= 1e-5 * ref.loss, k
        gw, gb = net.split(flat[k])
        for l in range(len(w)):
            for got, want in ((gw[l], ref.dw[l]), (gb[l], ref.db[l])):
                rel = np.linalg.norm(got - want) / np.linalg.norm(want)
                assert rel <= 5e-3, (k, l, rel)


def test_training_batch_on_tcgen05_shapes_matches_the_oracle() -> None:
    """Batch 256 and hidden widths of 512: the forward, weight-gradient and input-gradient GEMMs
    of the hidden layers run on tcgen05; loss and gradients against the oracle."""
    from open_analysis_gb300.surrogate import Mlp

    net = Mlp([7, 512, 512, 128], batch=256, seed=2, act="tanh")
    w, b = net.weights()
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, (256, 7))
    t = rng.standard_normal((256, 128))
    loss, flat = net.gradients(x, t)
    gw, gb = net.split(flat)
    ref = loss_and_grads(w, b, net.pad(x), t.astype(np.float32), bf16=True, act="tanh")
    assert abs(loss - ref.loss) <= 1e-5 * ref.loss
    for l in range(len(w)):
        for got, want in ((gw[l], ref.dw[l]), (gb[l], ref.db[l])):
            rel = np.linalg.norm(got - want) / np.linalg.norm(want)
            assert rel <= 5e-3, (l, rel)


def _small_net(seed: int = 0, act: str = "tanh"):  # type: ignore[no-untyped-def]
    from open_analysis_gb300.surrogate import Mlp

    return Mlp([7, 96, 80, 64, 40], batch=48, seed=seed, act=act)


@pytest.mark.parametrize("act", ["relu", "tanh"])
def test_training_gradients_match_the_oracle(act: str) -> None:
    net = _small_net(act=act)
    w, b = net.weights()
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (48, 7))
    t = rng.standard_normal((48, 40))
    loss, flat = net.gradients(x, t)
    gw, gb = net.split(flat)
    xp = net.pad(x)  # the input padded to 8 columns, as the network sees it
    ref = loss_and_grads(w, b, xp, t.astype(np.float32), bf16=True, act=act)
    exact = loss_and_grads(w, b, np.pad(x, ((0, 0), (0, 1))), t, bf16=False, act=act)
    assert abs(loss - ref.loss) <= 1e-5 * ref.loss
    worst, worst_exact = 0.0, 0.0
    for l in range(len(w)):
        for got, want, full in ((gw[l], ref.dw[l], exact.dw[l]), (gb[l], ref.db[l], exact.db[l])):
            rel = np.linalg.norm(got - want) / np.linalg.norm(want)
            assert rel <= 5e-3, (l, rel)  # FP32 accumulation order and a few BF16 re-roundings
            rel_exact = np.linalg.norm(got - full) / np.linalg.norm(full)
            assert rel_exact <= 1e-1, (l, rel_exact)  # the cost of BF16 storage itself
            worst, worst_exact = max(worst, rel), max(worst_exact, rel_exact)
    print(f"{act} gradient rel-L2: vs BF16-rounded oracle {worst:.2e}, vs exact FP64 network {worst_exact:.2e}")


def test_adam_step_matches_the_oracle() -> None:
    net = _small_net(seed=3)
    rng = np.random.default_rng(6)
    x, t = rng.uniform(-1, 1, (48, 7)), rng.standard_normal((48, 40))
    w0, b0 = net.weights()
    _, flat = net.gradients(x, t)
    net.adam_step(lr=2e-3)
    net.adam_step(lr=2e-3)  # second step on the same gradient: exercises the bias corrections
    torch.cuda.synchronize()
    w1, b1 = net.weights()
    params = [*w0, *b0]
    gw, gb = net.split(flat)
    st = AdamState([np.zeros_like(p) for p in params], [np.zeros_like(p) for p in params])
    adam(params, [*gw, *gb], st, lr=2e-3)
    adam(params, [*gw, *gb], st, lr=2e-3)
    for got, want in zip([*w1, *b1], params, strict=True):
        np.testing.assert_allclose(got, want, rtol=0, atol=2e-6)


def test_training_fits_a_smooth_map() -> None:
    from open_analysis_gb300.surrogate import Mlp

    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, (512, 7))
    t = np.stack([np.sin(x @ rng.standard_normal(7) * 0.7 + k) for k in range(32)], axis=1)
    net = Mlp([7, 256, 256, 256, 32], batch=128, seed=1)
    losses = net.fit(x, t, epochs=300, lr=2e-3, lr_end=1e-4, log_every=50)
    assert losses[-1] < 0.02 * losses[0], losses
    pred = net.predict(x[:64])
    assert np.sqrt(np.mean((pred - t[:64]) ** 2)) < 0.05


def test_surrogate_gains_over_the_plain_engine() -> None:
    """A three-parameter sweep (stack height, eps_inf, delta_eps; drill, pad, antipad and stub
    fixed) of small via transitions: the ensemble answers held-out instances within its bound,
    FDTD the rest; every answer is judged against FDTD, and the sweep rate is compared with the
    batched engine alone and with a loop of the plain engine over the same instances."""
    from open_analysis_gb300.surrogate import TOL_DB, ViaGrid, experiment

    g = ViaGrid(nx=48, ny=48, nz=60, h=50e-6, dz=100e-6, n_freq=32, cpml=6, span=560e-12)
    fixed = {"drill": 0.3e-3, "pad": 0.5e-3, "antipad": 0.9e-3, "stub": 0.6e-3}
    n = 384
    rep = experiment(g, n, seed=21, fixed=fixed, split=(256 / n, 32 / n, 32 / n), batch=64, epochs=3000,
                     lrs=(1e-3,), chunk=64)
    print({k: rep[k] for k in ("accepted", "accepted_worst_db", "network_alone_median_db", "network_alone_within_tol",
                               "scale", "gain_vs_batched", "gain_vs_plain", "train_seconds")})
    assert rep["answers_within_tol"] == 1.0 and rep["answers_worst_db"] <= TOL_DB
    assert rep["network_alone_median_db"] <= TOL_DB
    assert rep["accepted"] >= 0.25
    assert rep["gain_vs_batched"] > 1.2 and rep["gain_vs_plain"] > rep["gain_vs_batched"]


def test_ensemble_save_and_load_predict_the_same(tmp_path) -> None:  # type: ignore[no-untyped-def]
    from open_analysis_gb300.surrogate import Dataset, Ensemble, ViaGrid, via_params

    g = ViaGrid(nx=48, ny=48, nz=60, h=50e-6, dz=100e-6, n_freq=8, cpml=6, span=560e-12)
    rng = np.random.default_rng(3)
    p = via_params(96, seed=9)
    s = (rng.standard_normal((96, 2, 8)) + 1j * rng.standard_normal((96, 2, 8))) * 0.1
    ens = Ensemble(g, members=2, width=64, depth=2, batch=32, seed=4)
    ens.fit(Dataset(p, s, np.linspace(0.1e9, 20e9, 8)), epochs=20)
    ens.scale = 3.5
    path = str(tmp_path / "ens.npz")
    ens.save(path)
    back = Ensemble.load(path)
    a, b = ens.predict(p[:10]), back.predict(p[:10])
    assert back.scale == 3.5 and back.sizes == ens.sizes
    np.testing.assert_array_equal(a.s, b.s)
    np.testing.assert_array_equal(a.bound_db, b.bound_db)
