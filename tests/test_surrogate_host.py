"""The surrogate's host-side pieces (omg_audio_gb300/surrogate.py), on the CPU.

- The training family: sizes, absorption, openness and poses inside their
  ranges, 0 to 4 open apertures equally often, and the absorption mixture the
  sampler documents: rooms whose surfaces are all hard are common, where
  independent draws never give them.
- The city's room/source pairs as shoeboxes: rooms no larger than one cell,
  the listener at the cell's centre, the source 1 m inside the walls, windows
  only on the building's perimeter.
- The aperture boxes: flush with their walls, within the wall, area = w x h.
- The inputs: the Sabine columns follow Sabine's formula, each aperture panel
  absorbing its openness over its area as the tracer's panel does; family rooms
  are in range and rooms outside the family are not.
- The EDC and its RT60 on an exponential decay of known RT60, beside the
  oracle's estimate_reverb (the reference's T20, tracer.rs:205-257) on the
  same bins.
"""
import numpy as np

from omg_audio_gb300 import surrogate as S


def test_family_ranges_and_apertures():
    r = S.sample_rooms(20000, seed=1)
    n = len(r)
    assert r.size.shape == (n, 3) and r.alpha.shape == (n, 6, 3) and r.openness.shape == (n, 4)
    assert np.all(r.size >= S.SIZE_LO) and np.all(r.size <= S.SIZE_HI)
    assert np.all(r.alpha >= S.ALPHA_LO) and np.all(r.alpha <= S.ALPHA_HI)
    assert np.all(r.openness >= 0.0) and np.all(r.openness <= 1.0)
    for p in (r.src, r.lis):
        assert np.all(p >= 1.0) and np.all(p <= r.size - 1.0)
    share = np.bincount((r.openness > 0).sum(1), minlength=5) / n
    assert np.all(np.abs(share - 0.2) < 0.02), share
    again = S.sample_rooms(20000, seed=1)
    assert np.array_equal(again.alpha, r.alpha) and np.array_equal(again.src, r.src)


def test_family_mixture_holds_uniformly_hard_rooms():
    r = S.sample_rooms(20000, seed=2)
    a = r.alpha.reshape(len(r), -1)
    hard = (a.max(1) < 0.06).mean()
    narrow = (a.max(1) / a.min(1) < 6.0).mean()
    ind = np.random.default_rng(2).uniform(S.ALPHA_LO, S.ALPHA_HI, a.shape)
    assert hard > 0.04, hard
    assert (ind.max(1) < 0.06).mean() == 0.0
    assert narrow > 0.45 and (ind.max(1) / ind.min(1) < 6.0).mean() < 0.2


def test_city_rooms_are_cells_of_their_buildings():
    buildings = np.array([[0.0, 0.0, 40.0, 25.0, 12.0, 3.0],
                          [60.0, 10.0, 14.0, 10.0, 9.0, 3.0],
                          [100.0, -30.0, 31.0, 23.0, 20.0, 4.0]])
    sources = np.array([[-5.0, 5.0, 1.5], [50.0, 50.0, 2.0]])
    absorption = {"facade": np.linspace(0.01, 0.08, 8), "ground": np.full(8, 0.02), "slab": np.full(8, 0.05)}
    r = S.city_rooms(buildings, sources, absorption, window_frac=0.4)
    assert len(r) == 6
    assert np.all(r.size[:, 0] <= S.CITY_CELL[0] + 1e-9) and np.all(r.size[:, 1] <= S.CITY_CELL[1] + 1e-9)
    assert np.allclose(r.size[:, 2], np.repeat(buildings[:, 5], 2))
    assert np.allclose(r.lis[:, :2], 0.5 * r.size[:, :2])
    assert np.all(r.src >= 1.0 - 1e-9) and np.all(r.src <= r.size - 1.0 + 1e-9)
    assert np.all(np.isin(r.openness, [0.0, 0.4]))
    # the first building (40 x 25 m: 3 x 3 cells) seen from (-5, 5): its x- wall cell, on the perimeter
    assert r.openness[0, 0] == 0.4 and r.openness[0, 1] == 0.0
    assert np.allclose(r.alpha[:, 0:4, :], absorption["facade"][list(S.CITY_BANDS)])
    assert np.allclose(r.alpha[:, 4, :], 0.02) and np.allclose(r.alpha[:, 5, :], 0.05)


def test_aperture_boxes_sit_on_their_walls():
    size = np.array([[4.0, 4.0, 2.5], [16.0, 12.0, 6.0], [1.5, 9.0, 1.8]])
    mn, mx, area = S.aperture_boxes(size)
    for i, (sx, sy, sz) in enumerate(size):
        for k in range(4):
            axis = 0 if k < 2 else 1
            other = 1 - axis
            wall = 0.0 if k % 2 == 0 else size[i, axis]
            assert mn[i, k, axis] <= wall <= mx[i, k, axis]
            assert mx[i, k, axis] - mn[i, k, axis] <= 0.052
            w = mx[i, k, other] - mn[i, k, other]
            h = mx[i, k, 2] - mn[i, k, 2]
            assert 0 < w <= S.APERTURE_W and mn[i, k, other] > 0 and mx[i, k, other] < size[i, other]
            assert 0 < h <= S.APERTURE_H and h < sz
            assert np.isclose(area[i, k], w * h)


def test_sabine_columns_and_the_family_range():
    r = S.sample_rooms(64, seed=5)
    r.openness[:] = 0.5
    r.alpha[:] = 0.1
    x = S.features(r)
    sx, sy, sz = r.size.T
    _, _, ap = S.aperture_boxes(r.size)
    # every side wall carries its aperture panel, which absorbs its openness
    # (the tracer's panel material) over its area instead of the wall's 0.1
    absorb = 0.1 * 2 * (sx * sy + sy * sz + sx * sz) + (0.5 - 0.1) * ap.sum(1)
    want = 0.161 * sx * sy * sz / absorb
    assert np.allclose(x[:, S.SABINE_COLS], want[:, None], rtol=1e-5)
    assert S.in_range(x).all()
    big = x.copy()
    big[0, 0] = S.SIZE_HI[0] + 1.0
    soft = x.copy()
    soft[1, 3 + 7] = S.ALPHA_HI + 0.05
    assert not S.in_range(big)[0] and S.in_range(big)[1:].all()
    assert not S.in_range(soft)[1]


def test_rt60_of_an_exponential_decay(oracle):
    O = oracle
    bin_dt, n_bins = 0.001, 4000
    rt = np.array([0.3, 0.8, 1.6])
    t = (np.arange(n_bins) + 0.5) * bin_dt
    bins = np.exp(-np.log(1e6) * t[:, None] / rt[None, :])   # -60 dB over rt
    edc = S.edc_db(bins, bin_dt)
    assert edc.shape == (S.N_TIMES, 3)
    assert np.all(np.diff(edc, axis=0) <= 1e-9)
    got = S.rt60_from_edc(edc)
    assert np.allclose(got, rt, rtol=0.01), got
    ref, _, _ = O.estimate_reverb(bins, bin_dt, level_f32=False)
    assert np.allclose(got, ref, rtol=0.02), (got, ref)
