"""The echogram's host bookkeeping (omg_audio_gb300/tracer.py: Echogram.ema and
late_direction, tracer.rs:46-77) against the oracle's f32 restatement, on the
CPU: random echograms from several start times, a start beyond the last bin
and before the first, a silent echogram, and the blend's end points."""
import numpy as np

from omg_audio_gb300.tracer import Echogram


def _random(rng, n_bins=300, nb=3):
    e = Echogram(n_bins, nb, 0.010)
    e.bins[:] = rng.exponential(1.0, (n_bins, nb)).astype(np.float32) * np.exp(-np.arange(n_bins) / 60.0)[:, None]
    e.dirs[:] = (rng.normal(size=(n_bins, 3)) * e.bins[:, 1:2]).astype(np.float32)
    return e


def test_late_direction_equals_the_oracle(oracle):
    O = oracle
    rng = np.random.default_rng(7)
    for k in range(6):
        e = _random(rng)
        e.dirs[:, 0] += 0.3 * e.bins[:, 1]   # a net direction, so the anisotropy is not noise only
        for from_s in (0.0, 0.05, 0.08, 0.5, 2.99, 5.0, -1.0):
            for mid in (0, 1, 2):
                d, an = e.late_direction(from_s, mid)
                od, oan = O.late_direction(e.bins, e.dirs, e.bin_dt, from_s, mid=mid, f32=True)
                assert np.array_equal(d, od), (k, from_s, mid, d, od)
                assert np.float32(an) == np.float32(oan), (k, from_s, mid, an, oan)
    d, an = Echogram(300, 3, 0.010).late_direction(0.05)
    assert np.array_equal(d, [1.0, 0.0, 0.0]) and an == 0.0


def test_ema_end_points_and_one_step():
    rng = np.random.default_rng(8)
    a, b = _random(rng), _random(rng)
    a0, d0 = a.bins.copy(), a.dirs.copy()
    a.ema(b, 0.0)
    assert np.array_equal(a.bins, a0)
    a.ema(b, 1.0)
    # a + (b - a) in f32, as the reference writes it: b to within two roundings
    for got, old, want in ((a.bins, a0, b.bins), (a.dirs, d0, b.dirs)):
        tol = 2 * np.spacing(np.maximum(np.abs(old), np.abs(want)))
        assert np.all(np.abs(got - want) <= tol)
    c = _random(rng)
    want = c.bins + np.float32(0.25) * (b.bins - c.bins)
    c.ema(b, 0.25)
    assert c.bins.dtype == np.float32 and np.array_equal(c.bins, want)
