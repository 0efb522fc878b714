"""Wire formats on the host: ParamBlock's flat layout (params.rs:67-141) and
the web bridge's flat jobs (omg-web/src/lib.rs:150-202, 365-416) through the C
library against the oracle's restatement. No device work: these entry points
are host-only."""
import math

import numpy as np
import pytest

from oracle import wire_oracle as WO


@pytest.fixture(scope="module")
def W(built_lib):
    from omg_audio_gb300 import wire
    return wire


def _random_block(rng, n_taps, remote):
    taps = [(int(rng.integers(0, 1 << 32)), float(np.float32(rng.uniform(0, 0.3))),
             [float(np.float32(v)) for v in rng.normal(size=3)], [float(np.float32(v)) for v in rng.uniform(0, 1, 3)])
            for _ in range(n_taps)]
    rem = None
    if remote:
        rem = ([float(np.float32(v)) for v in rng.uniform(0.1, 3, 3)],
               [float(np.float32(v)) for v in rng.uniform(0, 1, 3)],
               [float(np.float32(v)) for v in rng.normal(size=9)])
    return {"version": int(rng.integers(0, 1 << 62)), "taps": taps,
            "rt60": [float(np.float32(v)) for v in rng.uniform(0.1, 5, 3)],
            "level": [float(np.float32(v)) for v in rng.uniform(0, 0.7, 3)], "remote": rem}


def _to_lib(W, pb):
    return W.ParamBlock([W.Tap(k, d, tuple(di), tuple(g)) for (k, d, di, g) in pb["taps"]], tuple(pb["rt60"]),
                        tuple(pb["level"]), None if pb["remote"] is None else W.RemoteReverb(*map(tuple, pb["remote"])),
                        pb["version"])


def test_layout_constants(W):
    from omg_audio_gb300 import _lib
    assert (W.FLAT_HEADER, W.FLAT_PER_TAP) == (WO.FLAT_HEADER, WO.FLAT_PER_TAP) == (24, 9)
    assert W.BOX_JOB_F32S == WO.GPU_JOB_F32S == 57
    assert W.WORLD_JOB_F32S == WO.WLATE_JOB_F32S == 1034
    assert (_lib.WEB_BOX_JOB_VERSION, _lib.WEB_WORLD_JOB_VERSION) == (2, 3)
    for n in (0, 1, 7, 100):
        assert W.ParamBlock(taps=[W.Tap(0, 0.0, (0, 0, 0), (0, 0, 0))] * n).flat_len() == 24 + 9 * n


@pytest.mark.parametrize("n_taps,remote", [(0, False), (1, True), (5, False), (33, True)])
def test_param_block_write_matches_the_oracle(W, n_taps, remote):
    rng = np.random.default_rng(n_taps * 7 + remote)
    for _ in range(20):
        pb = _random_block(rng, n_taps, remote)
        got = _to_lib(W, pb).write_flat()
        ref = WO.write_flat(pb)
        assert got.dtype == np.float32 and got.shape == ref.shape
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("n_taps,remote", [(0, True), (3, False), (12, True)])
def test_param_block_read_matches_the_oracle(W, n_taps, remote):
    rng = np.random.default_rng(100 + n_taps)
    for _ in range(20):
        flat = WO.write_flat(_random_block(rng, n_taps, remote))
        # a few words the writer never produces: the reader's casts decide them
        flat[0] = rng.choice([np.nan, -3.0, 1e30, 12345.75, flat[0]])
        if n_taps:
            flat[24] = rng.choice([np.nan, -1.5, 7.9, 5e9, flat[24]])
        got = W.ParamBlock.read_flat(flat)
        ref = WO.read_flat(flat)
        assert got.version == ref["version"]
        assert list(got.rt60) == ref["rt60"] and list(got.level) == ref["level"]
        assert (got.remote is None) == (ref["remote"] is None)
        if got.remote is not None:
            assert [list(got.remote.rt60), list(got.remote.send), list(got.remote.sh)] == list(map(list, ref["remote"]))
        assert len(got.taps) == len(ref["taps"])
        for t, (k, d, di, g) in zip(got.taps, ref["taps"]):
            assert (t.key, t.delay_s, list(t.dir), list(t.gains)) == (k, d, di, g)


def test_param_block_round_trip_and_short_input(W):
    from omg_audio_gb300 import _lib
    pb = W.ParamBlock([W.Tap(7, 0.012, (0.0, 1.0, 0.0), (0.5, 0.25, 0.125))], (1.2, 0.9, 0.6), (0.3, 0.2, 0.1),
                      W.RemoteReverb((2.0, 1.5, 1.0), (0.1, 0.05, 0.02), tuple(range(9))), 42)
    back = W.ParamBlock.read_flat(pb.write_flat())
    assert back.version == 42 and back.taps[0].key == 7 and back.remote.sh == tuple(float(v) for v in range(9))
    assert np.allclose(back.rt60, pb.rt60) and np.allclose(back.taps[0].gains, pb.taps[0].gains)
    flat = pb.write_flat()
    with pytest.raises(_lib.OmgError):
        W.ParamBlock.read_flat(flat[:-1])          # one tap announced, 8 of its 9 words present
    with pytest.raises(IndexError):
        WO.read_flat(flat[:-1])
    with pytest.raises(_lib.OmgError):
        W.ParamBlock.read_flat(flat[:20])          # shorter than the header


def test_param_block_from_late_states(W):
    from omg_audio_gb300 import _lib
    st = [_lib.omg_late_state() for _ in range(3)]
    for i, s in enumerate(st):
        for b in range(8):
            s.rt60[b] = 0.5 + i + 0.1 * b
            s.level[b] = 0.01 * (b + 1) + i
        s.version = 10 * i
    blocks = W.ParamBlock.from_late_states(st)
    for i, pb in enumerate(blocks):
        assert pb.version == 10 * i and pb.remote is None and pb.taps == []
        assert np.array_equal(np.float32(pb.rt60), np.float32([st[i].rt60[b] for b in range(3)]))
        assert np.array_equal(np.float32(pb.level), np.float32([st[i].level[b] for b in range(3)]))


def test_flat_job_packing_matches_the_oracle(W):
    from omg_audio_gb300.materials import Material
    rng = np.random.default_rng(5)
    walls = [Material(tuple(rng.uniform(0.02, 0.4, 3)), 0.1, tuple(rng.uniform(0, 0.2, 3))) for _ in range(6)]
    seed = int(rng.integers(0, 1 << 32))
    a = W.box_job(17, (10, 7, 4), walls, (2, 3, 1.5), (7, 4, 1.2), 4096, seed, energy=(1.0, 0.5, 0.25))
    b = WO.pack_box_job(17, 4096, seed, (10, 7, 4), (2, 3, 1.5), (7, 4, 1.2), (1.0, 0.5, 0.25),
                        [(w.absorption, w.scattering, w.transmission) for w in walls])
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    d = WO.decode_box_job(a)
    assert d["n_rays"] == 4096 and d["id"] == 17
    assert d["seed"] == int(np.float32(seed))  # an f32 word holds the seed: 24 significant bits survive
    pan = [((1, 1, 0), (2, 1.1, 2), tuple(rng.uniform(0, 0.3, 3)), 0.05, tuple(rng.uniform(0, 0.3, 3)))
           for _ in range(70)]
    wa = W.world_job(3, (1, 2, 1), (5, 6, 1.5), 8192, 0xC6D2,
                     [(mn, mx, Material(ab, sc, tr)) for (mn, mx, ab, sc, tr) in pan])
    wb = WO.pack_world_job(3, 8192, 0xC6D2, (1, 2, 1), (5, 6, 1.5), pan)
    assert np.array_equal(wa.view(np.uint32), wb.view(np.uint32))
    assert len(WO.decode_world_job(wa)["panels"]) == 64   # capped as the proxy caps it


def test_js_and_rust_casts():
    assert WO.js_to_uint32(4294967296.0) == 0 and WO.js_to_uint32(-1.0) == 4294967295
    assert WO.js_to_uint32(float("nan")) == 0 and WO.js_to_uint32(3.99) == 3
    assert WO.rust_as_uint(float("nan"), 32) == 0 and WO.rust_as_uint(-2.0, 32) == 0
    assert WO.rust_as_uint(5e9, 32) == 4294967295 and WO.rust_as_uint(math.inf, 64) == (1 << 64) - 1
    assert WO.uint_to_f32((1 << 24) + 1) == float(1 << 24) and WO.uint_to_f32((1 << 24) + 3) == float((1 << 24) + 4)
