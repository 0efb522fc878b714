"""The sim's trace gate and tick control flow (sim.rs:32-75, 346-398) against
the oracle's restatement, on the host: a stand-in for the device late field
returns canned states, so no GPU is needed."""
import numpy as np
import pytest

from oracle import sim_oracle as SO


def _walk(rng, n_ticks, n_sims, step):
    poses = []
    cur = [(rng.uniform(1, 9, 3), rng.uniform(1, 9, 3)) for _ in range(n_sims)]
    for _ in range(n_ticks):
        nxt = []
        for i, (s, l) in enumerate(cur):
            mv = step[i % len(step)]
            s = s + rng.normal(0, mv, 3) if mv else s
            l = l + rng.normal(0, mv / 2, 3) if mv else l
            nxt.append((s, l))
        cur = nxt
        poses.append([(tuple(map(float, s)), tuple(map(float, l))) for s, l in cur])
    return poses


@pytest.mark.parametrize("max_age", [1, 3, 8, 64])
def test_trace_gate_matches_the_oracle(max_age):
    from omg_audio_gb300.sim import TraceGate
    rng = np.random.default_rng(max_age)
    poses = _walk(rng, 200, 6, step=[0.0, 0.05, 0.2, 0.4])
    for i in range(6):
        g, o = TraceGate(i % 8, max_age), SO.TraceGate(i % 8, max_age)
        for t, tick in enumerate(poses):
            src, lis = tick[i]
            e = [1.0, 1.0, 1.0] if t % 37 else [1.0, 1.2, 1.0]
            assert g.should_trace(src, lis, e) == o.should_trace(src, lis, e), (i, t)
            assert g.age == o.age


def test_gate_fires_on_motion_age_and_energy():
    from omg_audio_gb300.sim import TraceGate
    g = TraceGate(0, 8)
    assert g.should_trace((1, 1, 1), (2, 2, 2), [1, 1, 1])          # first call: never traced
    assert not g.should_trace((1.1, 1, 1), (2, 2, 2), [1, 1, 1])    # 0.1 m: stays
    assert g.should_trace((1.3, 1, 1), (2, 2, 2), [1, 1, 1])        # 0.3 m from the last trace
    assert g.should_trace((1.3, 1, 1), (2, 2, 2), [1, 1.2, 1])      # an energy moved > 10 %
    for _ in range(7):
        assert not g.should_trace((1.3, 1, 1), (2, 2, 2), [1, 1.2, 1])
    assert g.should_trace((1.3, 1, 1), (2, 2, 2), [1, 1.2, 1])      # the 8th call since: age 8


class _FakeField:
    """Stands in for the device late field: each landed slot's state carries
    a distinct level so the test can follow which result is shown."""

    def __init__(self, n, nb=3):
        from omg_audio_gb300.sim import LateState
        self.LS, self.n, self.nb = LateState, n, nb
        self.pending = False
        self.tick = 0
        self.states = [LateState(np.full(nb, 0.5, np.float32), np.zeros(nb, np.float32),
                                 np.array([1, 0, 0], np.float32), 0.0, 0, 0) for _ in range(n)]
        self.submits = []

    def submit(self, slots, jobs, panels, alpha):
        self.tick += 1
        self.submits.append((list(slots), list(alpha)))
        for s in slots:
            st = self.states[s]
            self.states[s] = self.LS(st.rt60 + 0.01, np.full(self.nb, 0.1 * (s + 1), np.float32), st.dir,
                                     st.anisotropy, st.version + 1, self.tick)
        self.pending = True
        return self.tick

    def poll(self, wait=False):
        self.pending = False
        return self.tick, list(self.states)


def test_tick_control_flow_matches_reverb_world():
    """Which instances fire, in which tick their result shows, the budget, the
    0.3 weight of async landings and the staleness scaling of the level."""
    from omg_audio_gb300 import sim as S
    n, budget = 5, 2
    sf = S.SimField.__new__(S.SimField)
    sf.ctx, sf.scene, sf.n, sf.rays, sf.budget = None, None, n, 4096, budget
    sf.field = _FakeField(n)
    sf.gates = [S.TraceGate(i % 8, 8) for i in range(n)]
    sf.version, sf.rp_dist, sf.seed = [0] * n, [S.F32_MAX] * n, 1
    sf.inflight, sf.states, sf.last_jobs, sf.last_slots = [], sf._empty_states(), [], []
    oracle_gates = [SO.TraceGate(i % 8, 8) for i in range(n)]
    rp = [SO.F32_MAX] * n
    rng = np.random.default_rng(3)
    poses = _walk(rng, 40, n, step=[0.0, 0.1, 0.3, 0.5, 0.05])
    landed_prev = []
    for t, tick in enumerate(poses):
        out = sf.tick(tick)
        # the oracle: results of the previous tick's fires land now
        b = [budget]
        fire = []
        for i, (src, lis) in enumerate(tick):
            traced = i in landed_prev
            if not traced and b[0] > 0 and oracle_gates[i].should_trace(src, lis, [1.0] * 3):
                b[0] -= 1
                fire.append(i)
            if traced:
                rp[i] = SO._dist(src, lis)
            lv = np.full(3, 0.1 * (i + 1), np.float32) if sf.states[i].version else np.zeros(3, np.float32)
            if rp[i] < SO.F32_MAX:
                k = min((np.float32(rp[i]) + np.float32(1)) / (np.float32(SO._dist(src, lis)) + np.float32(1)),
                        np.float32(1))
                lv = (lv * np.float32(k)).astype(np.float32)
            np.testing.assert_array_equal(out[i][0].level, lv)
        assert sf.last_slots == fire, t
        if fire:
            assert sf.field.submits[-1] == (fire, [0.3] * len(fire))
        landed_prev = fire
