"""The web bridge's flat trace jobs through the C ABI (omg_trace_web_box_jobs,
omg_trace_web_world_jobs): a queue of jobs packed as the wasm proxies pack them
(omg-web/src/lib.rs:170-193, 386-412) is traced in one batch, and each
injection record equals the structured entry point's result for the job as the
JS driver decodes it (web/gpu.js:181-199, 420-437), and the f32 oracle's.

Tolerances: segment counts exact; bins within 1e-5 relative (bins holding
>= 1e-6 of the band total: the sums are compensated FP32, whose last bits
depend on the order of the atomic adds); direction sums within 1e-4.
"""
import numpy as np
import pytest

from omg_audio_gb300 import _lib, wire
from omg_audio_gb300 import workloads as W
from omg_audio_gb300.materials import Material
from oracle import wire_oracle as WO

from test_gpu_parity import gpu_scene, oparams, oracle_mesh, rel_bins
from test_oracle_golden import omat

pytestmark = pytest.mark.gpu


def _box_queue(seed=11, n=6):
    rng = np.random.default_rng(seed)
    jobs, dec = [], []
    for i in range(n):
        size = tuple(float(v) for v in rng.uniform([4, 3, 2.5], [16, 12, 6]))
        walls = [Material(tuple(rng.uniform(0.02, 0.4, 3)), float(rng.uniform(0, 0.3)),
                          tuple(rng.uniform(0, 0.2, 3)) if w == 1 else (0.0, 0.0, 0.0)) for w in range(6)]
        src = tuple(float(rng.uniform(1, s - 1)) for s in size)
        lis = tuple(float(rng.uniform(1, s - 1)) for s in size)
        seed_u32 = int(rng.integers(1 << 20, 1 << 32))          # rounds to 24 significant bits in the f32 word
        f = wire.box_job(100 + i, size, walls, src, lis, int(rng.integers(500, 5000)), seed_u32,
                         energy=tuple(float(v) for v in rng.uniform(0.5, 1.5, 3)))
        jobs.append(f)
        dec.append(WO.decode_box_job(f))
    return np.concatenate(jobs), dec


def test_web_box_jobs_equal_single_traces(ctx, oracle):
    O = oracle
    flat, dec = _box_queue()
    echo, ids, rv = wire.trace_web_box_jobs(ctx, flat)
    nb = ctx.cfg.n_bins
    assert list(ids) == [d["id"] for d in dec]
    for k, d in enumerate(dec):
        walls = [Material(tuple(a), s, tuple(t)) for (a, s, t) in d["walls"]]
        bins, dirs = wire.split_echo(echo[k], nb)
        e, r1 = ctx.trace_box(d["size"], walls, d["src"], d["lis"], d["n_rays"], energy=d["energy"], seed=d["seed"])
        assert rv[k].segments == r1.segments, k
        assert rel_bins(bins, e.bins) <= 1e-5, k
        assert np.allclose(dirs, e.dirs, rtol=1e-4, atol=1e-9), k
        if k < 2:
            ob, od, st = O.trace_box(d["size"], [omat(O, m) for m in walls], d["src"], d["lis"], d["n_rays"],
                                     energy=d["energy"], seed=d["seed"], acc64=True)
            assert rv[k].segments == st["segments"]
            assert rel_bins(bins, ob) <= 1e-5


def test_web_world_jobs_equal_single_traces(ctx, oracle):
    O = oracle
    case = W.multiroom(seed=2)
    scene = gpu_scene(ctx, case.recorder)
    om = oracle_mesh(O, case.recorder)
    pan = [(mn, mx, m) for (mn, mx, m) in case.panels]
    seeds = [(0xC6D2 + 0x9E3779B9 * k) & 0xFFFFFFFF for k in range(3)]
    jobs = [wire.world_job(7 + k, case.pairs[k][0], case.pairs[k][1], 2048 + 1024 * k, seeds[k], pan[:20 + 20 * k])
            for k in range(3)]
    echo, ids, rv = wire.trace_web_world_jobs(ctx, scene, np.concatenate(jobs))
    assert list(ids) == [7, 8, 9]
    P = oparams(O, ctx.cfg)
    for k, f in enumerate(jobs):
        d = WO.decode_world_job(f)
        assert len(d["panels"]) == min(20 + 20 * k, len(pan), 64)
        panels = [(tuple(mn), tuple(mx), Material(tuple(ab), sc, tuple(tr))) for (mn, mx, ab, sc, tr) in d["panels"]]
        bins, dirs = wire.split_echo(echo[k], ctx.cfg.n_bins)
        e, r1 = ctx.trace_world(scene, d["src"], d["lis"], d["n_rays"], panels=panels, seed=d["seed"])
        assert rv[k].segments == r1.segments, k
        assert rel_bins(bins, e.bins) <= 1e-5, k
        assert np.allclose(dirs, e.dirs, rtol=1e-4, atol=1e-9), k
        if k == 0:
            opan = [(mn, mx, omat(O, m)) for (mn, mx, m) in panels]
            ob, _, st = O.trace_mesh(om, d["src"], d["lis"], d["n_rays"], P=P, seed=d["seed"], panels=opan,
                                     threads=8, acc64=True)
            assert rv[k].segments == st["segments"]
            assert rel_bins(bins, ob) <= 1e-5
    scene.release()


def test_web_jobs_reject_bad_queues(ctx):
    flat, _ = _box_queue(n=2)
    with pytest.raises(_lib.OmgError):
        wire.trace_web_box_jobs(ctx, flat[:-1])       # not a whole number of jobs
    from omg_audio_gb300 import Context, TraceConfig
    with Context(TraceConfig(n_bands=8)) as c8:
        with pytest.raises(_lib.OmgError):
            wire.trace_web_box_jobs(c8, flat)         # the formats carry 3 bands
