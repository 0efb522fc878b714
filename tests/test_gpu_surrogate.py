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


@pytest.mark.parametrize("rows,hidden", [(256, 64), (2048, 256)])
def test_training_gradients_match_the_oracle(ctx, rows, hidden):
    """256 rows: one K chunk per dW GEMM; 2048 rows: dW split over the grid
    (atomic accumulation) and the pipelined GEMM at the training widths."""
    from oracle import mlp_oracle as MO
    net = Mlp(ctx, n_in=38, hidden=hidden, n_hidden=3, n_out=48, members=1, seed=5)
    rng = np.random.default_rng(11)
    x = rng.standard_normal((rows, 38)).astype(np.float32)
    y = rng.standard_normal((rows, 48)).astype(np.float32)
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
    assert np.all(losses[:, -1] < 0.25 * losses[:, 0]), losses
    mean, std = net.predict(x[:512])
    assert np.sqrt(np.mean((mean - y[:512]) ** 2)) < 0.5 * np.std(y), np.sqrt(np.mean((mean - y[:512]) ** 2))
    assert np.all(std >= 0)
    net.close()


def test_room_surrogate_gains_over_sabine_falls_back_and_checkpoints(tmp_path):
    """Trained on tracer echograms of the config-1 room family (small: 32k rooms
    at 1024 rays), the surrogate's RT60 beats the Sabine formula (the method
    without the network) against the tracer at 4096 rays; a room outside the
    training family is answered by the tracer; a checkpoint reloads to the same
    predictions."""
    from omg_audio_gb300 import Context, TraceConfig
    from omg_audio_gb300 import surrogate as S
    with Context(TraceConfig(n_bands=3, n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200,
                             energy_floor=1e-6, timeout_ms=60000)) as ctx:
        train = S.sample_rooms(32768, seed=3)
        bins, _ = S.trace_rooms(ctx, train, 1024, seed=10)
        sur = S.RoomSurrogate(ctx, members=2, hidden=256)
        sur.fit(train, S.edc_db(bins, 0.001), epochs=40, batch=2048, lr=2e-3, lr_final=2e-5)
        test = S.sample_rooms(512, seed=4)
        bt, _ = S.trace_rooms(ctx, test, 4096, seed=20)
        rt = S.rt60_from_edc(S.edc_db(bt, 0.001))
        pred, std, ok = sur.predict(test)
        err = np.abs(S.rt60_from_edc(pred) / rt - 1)
        sab = np.abs(S.features(test)[:, S.SABINE_COLS] / rt - 1)
        assert np.nanmedian(err) < 0.75 * np.nanmedian(sab), (np.nanmedian(err), np.nanmedian(sab))
        assert np.nanmedian(err) < 0.08
        assert ok.mean() > 0.9
        # a room outside the family: the tracer answers it
        odd = test.take(np.arange(3))
        odd.size[0] = [30.0, 20.0, 10.0]
        edc, used = sur.answer(odd, n_rays=1024, seed=1)
        assert not used[0] and used[1:].all()
        ref, _ = S.trace_rooms(ctx, odd.take([0]), 1024, seed=1)
        assert np.array_equal(edc[0], S.edc_db(ref, 0.001)[0].astype(np.float32))
        # checkpoint round trip
        path = str(tmp_path / "surrogate.bin")
        sur.net.save(path)
        net2 = S.Mlp.load(ctx, path)
        m2, s2 = net2.predict(S.features(test))
        m1, s1 = sur.net.predict(S.features(test))
        assert np.array_equal(m1, m2) and np.array_equal(s1, s2)
        net2.close()
        sur.net.close()


@pytest.mark.parametrize("m,n,k,split", [(4096, 256, 256, 1), (256, 256, 4096, 8)])
def test_tc_gemm_bench_times_the_training_shapes(ctx, m, n, k, split):
    """omg_tc_gemm_bench runs the GEMM at a training shape and reports a
    positive device time per launch."""
    ms = C.c_float()
    rc = _lib.lib().omg_tc_gemm_bench(ctx.h, m, n, k, split, 20, C.byref(ms))
    ctx._check(rc, "omg_tc_gemm_bench")
    assert 0.0 < ms.value < 50.0
