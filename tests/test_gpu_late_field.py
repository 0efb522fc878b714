"""The device late field (omg_late_*) and the sim tick loop over it, against
the oracle: the EMA of the same fresh echograms (traced again through the
one-shot batch call with the same jobs), estimate_reverb and late_direction of
the average, and the gate decisions of Sim::reverb_world (sim.rs:346-398)."""
import numpy as np
import pytest

from oracle import sim_oracle as SO

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(built_lib):
    from omg_audio_gb300 import Context, MeshBuilder, TraceConfig, _lib
    from omg_audio_gb300 import workloads as W
    ctx = Context(TraceConfig(tie_mode=1))
    case = W.multiroom(seed=4, nx=3, ny=2, n_pairs=8)
    mb = MeshBuilder()
    case.recorder.replay(mb)
    scene = ctx.upload_builder(mb, 3, _lib.BVH_SAH)
    yield ctx, scene, case
    ctx.close()


def _fresh(ctx, jobs):
    return [(e.bins.copy(), e.dirs.copy()) for e, _ in ctx.trace_batch(jobs)]


def _check_slot(field, ctx, slot, avg, state, from_s=0.08):
    cfg = ctx.cfg
    e = field.read(slot)
    scale = float(np.abs(avg[0]).max()) + 1e-30
    np.testing.assert_allclose(e.bins, avg[0], rtol=1e-5, atol=1e-6 * scale)
    np.testing.assert_allclose(e.dirs, avg[1], rtol=1e-5, atol=1e-6 * (float(np.abs(avg[1]).max()) + 1e-30))
    # the state is the reverb / direction of the device average itself ...
    rv = ctx.estimate_reverb(e.bins)
    np.testing.assert_array_equal(state.rt60, rv.rt60[:3])
    np.testing.assert_array_equal(state.level, rv.level[:3])
    d, a = SO.O.late_direction(e.bins, e.dirs, cfg.bin_dt, from_s, mid=cfg.dir_band)
    np.testing.assert_allclose(state.dir, d, atol=2e-5)
    assert abs(state.anisotropy - a) <= 2e-5 * max(1.0, a)
    # ... and that of the oracle's average
    rt, lv, _ = SO.O.estimate_reverb(avg[0], cfg.bin_dt)
    np.testing.assert_allclose(state.rt60, rt, rtol=2e-3)
    np.testing.assert_allclose(state.level, lv, rtol=1e-4, atol=1e-7)


def test_late_field_blends_and_estimates_like_the_oracle(world):
    from omg_audio_gb300 import Job, OmgError
    from omg_audio_gb300.sim import LateField
    ctx, scene, case = world
    cfg = ctx.cfg
    n_slots = 5
    field = LateField(ctx, n_slots)
    avg = {s: (np.zeros((cfg.n_bins, 3), np.float32), np.zeros((cfg.n_bins, 3), np.float32)) for s in range(n_slots)}
    updates = {s: 0 for s in range(n_slots)}
    plan = [[0, 2], [1, 2, 4], [2], [0, 3, 4], []]
    seed = 11
    for k, slots in enumerate(plan):
        jobs = []
        for s in slots:
            seed += 1
            src, lis = case.pairs[s]
            jobs.append(Job(src, lis, 2048, seed=seed, scene=scene))
        alpha = [1.0 if updates[s] == 0 else 0.3 for s in slots]
        t = field.submit(slots, jobs, (), alpha)
        assert t == k + 1
        assert field.submit(slots, jobs, (), alpha) is None      # one tick in flight
        with pytest.raises(OmgError):
            field.read(0)                                         # not while pending
        tick, states = field.poll(wait=True)
        assert tick == t
        fresh = _fresh(ctx, jobs) if jobs else []
        for (s, a), f in zip(zip(slots, alpha), fresh):
            avg[s] = (SO.ema(avg[s][0], f[0], a), SO.ema(avg[s][1], f[1], a))
            updates[s] += 1
        for s in range(n_slots):
            st = states[s]
            assert st.version == updates[s]
            if updates[s] == 0:
                assert st.rt60[0] == 0.5 and st.level[0] == 0.0 and st.anisotropy == 0.0
                continue
            if s in slots:
                assert st.updated_tick == t
            _check_slot(field, ctx, s, avg[s], st)
    # a reset slot starts over: its next update replaces the average
    field.reset(2)
    _, states = field.poll()
    assert states[2].version == 0 and states[2].rt60[0] == 0.5
    np.testing.assert_array_equal(field.read(2).bins, 0.0)
    src, lis = case.pairs[2]
    job = Job(src, lis, 2048, seed=99, scene=scene)
    field.submit([2], [job])                                      # default weight: 1 on the first update
    _, states = field.poll(wait=True)
    f = _fresh(ctx, [job])[0]
    _check_slot(field, ctx, 2, f, states[2])
    # bad slots
    with pytest.raises(OmgError):
        field.submit([7], [job])
    with pytest.raises(OmgError):
        field.submit([1, 1], [job, job])
    field.close()


def test_sim_field_follows_reverb_world(world):
    """Eight ticks of moving and resting instances: the same instances fire
    as in the oracle's Sim::reverb_world, and each call's reverb, direction
    and staleness-scaled level match the oracle fed the same echograms."""
    from omg_audio_gb300.sim import SimField
    ctx, scene, case = world
    cfg = ctx.cfg
    n, budget = 6, 3
    sf = SimField(ctx, scene, n, rays=256, budget=budget)
    sims = [SO.SimOracle(cfg.n_bins, 3, cfg.bin_dt, phase=i % 8, max_age=8, from_s=0.08, dir_band=cfg.dir_band)
            for i in range(n)]
    rng = np.random.default_rng(5)
    poses = [list(map(lambda p: (np.array(p[0], np.float32), np.array(p[1], np.float32)), case.pairs[:n]))]
    for t in range(1, 10):
        nxt = []
        for i, (s, l) in enumerate(poses[-1]):
            step = [0.0, 0.05, 0.3, 0.6][i % 4]
            nxt.append((s + rng.normal(0, step, 3).astype(np.float32) * np.array([1, 1, 0], np.float32), l))
        poses.append(nxt)
    landed = {}
    fired_total = 0
    for t, tick in enumerate(poses):
        tick = [(tuple(map(float, s)), tuple(map(float, l))) for s, l in tick]
        out = sf.tick(tick)
        b = [budget]
        fire = []
        for i, (src, lis) in enumerate(tick):
            f, rt, lv, d, a = sims[i].step(landed.get(i), src, lis, b)
            if f:
                fire.append(i)
            rp, dd, aa = out[i]
            if sims[i].updates:
                np.testing.assert_allclose(rp.rt60, rt, rtol=2e-3)
                np.testing.assert_allclose(rp.level, lv, rtol=1e-4, atol=1e-7)
                np.testing.assert_allclose(dd, d, atol=5e-4)
                assert abs(aa - a) <= 5e-4
            else:
                assert rp.rt60[0] == 0.5 and rp.level[0] == 0.0
        assert sf.last_slots == fire, (t, sf.last_slots, fire)
        fired_total += len(fire)
        landed = dict(zip(sf.last_slots, _fresh(ctx, sf.last_jobs))) if sf.last_jobs else {}
    assert fired_total >= n          # every instance traced at least once
    sf.close()
