"""The surrogate's tensor-core kernels against the CPU oracle.

- GEMM (tcgen05, accumulator in TMEM): C = A . B^T for BF16 A, B equals the
  FP64 product of the same BF16 values within 1e-5 relative (FP32
  accumulation), over tile-aligned and ragged shapes and a long K.
- Training gradients (forward + backward on the tensor cores): against the
  FP64 oracle that rounds the same quantities to BF16, per-layer relative
  error (Frobenius) <= 5e-3; against the plain FP64 network <= 5e-2. The
  oracle's own backward is checked by finite differences.
- Training lowers the loss on a smooth target.
"""
import ctypes as C

import numpy as np
import pytest

from omg_audio_gb300 import _lib
from omg_audio_gb300.surrogate import Mlp

pytestmark = pytest.mark.gpu


def _gemm(ctx, a, b):
    from oracle import mlp_oracle as MO
    m, k = a.shape
    n = b.shape[0]
    ab, bb = MO.bf16_bits(a), MO.bf16_bits(b)
    c = np.zeros((m, n), np.float32)
    rc = _lib.lib().omg_tc_gemm(ctx.h, ab.ctypes.data, bb.ctypes.data, c.ctypes.data, m, n, k)
    ctx._check(rc, "omg_tc_gemm")
    return c, MO.bf16(a) @ MO.bf16(b).T


@pytest.mark.parametrize("m,n,k", [(128, 256, 256), (128, 16, 16), (300, 192, 38), (256, 48, 4096),
                                   (129, 17, 70), (4096, 256, 256)])
def test_tc_gemm_matches_fp64(ctx, m, n, k):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    c, ref = _gemm(ctx, a, b)
    scale = np.sqrt((np.abs(a) ** 2).sum(1))[:, None] * np.sqrt((np.abs(b) ** 2).sum(1))[None, :]
    assert np.max(np.abs(c - ref) / scale) <= 1e-5


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-30))


def test_training_gradients_match_the_oracle(ctx):
    from oracle import mlp_oracle as MO
    net = Mlp(ctx, n_in=38, hidden=64, n_hidden=3, n_out=48, members=1, seed=5)
    rng = np.random.default_rng(11)
    x = rng.standard_normal((256, 38)).astype(np.float32)
    y = rng.standard_normal((256, 48)).astype(np.float32)
    loss, grads = net.grad(x, y)
    layers = net.layers(0)
    ol, og = MO.loss_and_grads(layers, x, y, bf=True)
    assert abs(loss - ol) <= 1e-4 * abs(ol)
    for (gW, gb), (oW, ob) in zip(grads, og):
        assert _rel(gW, oW) <= 5e-3
        assert _rel(gb, ob) <= 5e-3
    _, pg = MO.loss_and_grads(layers, x, y, bf=False)
    for (gW, gb), (pW, pb) in zip(grads, pg):
        assert _rel(gW, pW) <= 5e-2
    net.close()


def test_oracle_backward_by_finite_differences():
    from oracle import mlp_oracle as MO
    rng = np.random.default_rng(3)
    layers = [(rng.standard_normal((8, 5)) * 0.5, rng.standard_normal(8) * 0.1),
              (rng.standard_normal((4, 8)) * 0.5, rng.standard_normal(4) * 0.1)]
    x, y = rng.standard_normal((16, 5)), rng.standard_normal((16, 4))
    _, g = MO.loss_and_grads(layers, x, y, bf=False)
    h = 1e-6
    for li, (W, b) in enumerate(layers):
        for (i, j) in [(0, 0), (1, 2), (W.shape[0] - 1, W.shape[1] - 1)]:
            Wp = W.copy(); Wp[i, j] += h
            Wm = W.copy(); Wm[i, j] -= h
            lp = MO.loss_and_grads([*layers[:li], (Wp, b), *layers[li + 1:]], x, y, bf=False)[0]
            lm = MO.loss_and_grads([*layers[:li], (Wm, b), *layers[li + 1:]], x, y, bf=False)[0]
            assert abs((lp - lm) / (2 * h) - g[li][0][i, j]) <= 1e-6 * max(1.0, abs(g[li][0][i, j]))


def test_training_lowers_the_loss(ctx):
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, (8192, 38)).astype(np.float32)
    w = rng.standard_normal((38, 48)).astype(np.float32) / 6
    w2 = rng.standard_normal((38, 48)).astype(np.float32) / 6
    y = np.tanh(x @ w) + 0.1 * np.sin(3 * (x @ w2))
    net = Mlp(ctx, n_in=38, hidden=128, n_hidden=3, n_out=48, members=2, seed=1)
    net.set_data(x, y)
    losses = net.train(epochs=12, batch=1024, lr=3e-3, lr_final=3e-4)
    assert losses.shape == (2, 12)
    assert np.all(losses[:, -1] < 0.1 * losses[:, 0])
    mean, std = net.predict(x[:512])
    assert np.sqrt(np.mean((mean - y[:512]) ** 2)) < 0.1
    assert np.all(std >= 0)
    net.close()
