"""The reference's acceptance tests on its walkthrough world, run on the GPU path.

World: tests/golden/walkthrough_world.json (rooms, doors and furniture of
crates/omg-scene/src/walkthrough.rs), built by the product's world builder
(world.py, dome.rs:79-258) and uploaded as one scene; every context here uses
the reference's own closest-hit rule (tie_mode 0, mesh.rs:505).

1. The seven dome tests of crates/omg-scene/src/dome.rs:494-654, on
   omg_dome_sample (384 rays, 6 events: the High tier), each assertion as the
   reference states it. Beside each sample, the f32 oracle's fan on the same
   world: per-ray escape flags and per-bin energies equal bit for bit.
2. crates/omg-scene/tests/late_world_gate.rs:
   - mesh_late_field_matches_shoebox (:20-93): omg_trace_world over the
     6 x 4 x 3 m box built as 6 quads against omg_trace_box over the analytic
     shoebox, 16384 rays x 4 seeds: RT60 ratio within [0.8, 1.25], level ratio
     within [0.75, 1.33] per band. The oracle traces the same streams: equal
     segment counts, bins within 1e-5 per bin.
   - doorway_wet_is_measured_directional_and_door_sensitive (:96-144): the
     music source in the living room, a corridor listener at (4.4, 7.5, 1.6),
     omg_trace_world over the world mesh with the late panels of world.rs:384-405
     (door leaves, panes, furniture above FURN_REFLECTOR_MIN_VOL). The wet
     field is split as world.rs:785-797 splits it (anisotropy a from
     late_direction at 80 ms, clamped to 0.9: diffuse level sqrt(1 - a), send
     sqrt(a) when a > 0.05); the average of 4 traces of 16384 rays stands in
     for the sim's EMA over 60 ticks. Asserted as the reference does: open wet
     > 1e-4, send > 0.15 of the wet, 0.15 s < RT60 < 3 s, closing the living
     room door drops the wet below 0.6 of open, reopening restores it above 0.6.
"""
import dataclasses
import os

import numpy as np
import pytest

from omg_audio_gb300 import Context, DomeProbe, MeshBuilder, TraceConfig
from omg_audio_gb300 import materials as M
from omg_audio_gb300.tracer import Echogram
from omg_audio_gb300.world import build_world_mesh, door_panels, late_panels

from walkthrough import furniture_world, leaf_panels, load, oracle_world, product_world
from test_gpu_parity import oparams, rel_bins
from test_oracle_golden import omat

pytestmark = pytest.mark.gpu

N_RAYS, EVENTS = 384, 6   # the High tier (quality.rs: dome rays 384, events 6)
THREADS = os.cpu_count() or 8


@pytest.fixture(scope="module")
def wctx(built_lib):
    c = Context(TraceConfig())     # the reference's constants and closest-hit rule
    yield c
    c.close()


def _doors(opened):
    """Product doors and the oracle's door dicts with openness overrides {index: value}."""
    R, D = product_world()
    D = [dataclasses.replace(d, openness=opened.get(i, d.openness)) for i, d in enumerate(D)]
    _, dd = load()
    dd = [dict(d, openness=opened.get(i, d["openness"])) for i, d in enumerate(dd)]
    return R, D, dd


class DomeCase:
    """The world for one door configuration: the GPU probe and the f32 oracle's."""

    def __init__(self, ctx, O, opened=None):
        R, D, dd = _doors(opened or {})
        self.mb = MeshBuilder()
        glass = build_world_mesh(self.mb, R, D)
        self.scene = ctx.upload_builder(self.mb)
        self.ctx = ctx
        self.glass = glass
        self.leaves = door_panels(D)
        self.oleaves = leaf_panels(dd)
        orooms, odoors = oracle_world(O, dd)
        ob = O.MeshBuilder()
        oglass = O.world_build(ob, orooms, odoors)
        self.O = O
        self.omesh = ob.build("f32")
        self.oglass = oglass

    def sample(self, eye, leaves=False):
        """One fresh probe per sample (its EMA is primed with alpha 1: energy = raw bins)."""
        probe = DomeProbe(self.ctx, self.scene, self.glass, n_fan=N_RAYS)
        g = probe.sample([eye], self.leaves if leaves else (), n_rays=N_RAYS, max_events=EVENTS)
        probe.destroy()
        op = self.O.DomeProbe(self.omesh, self.oglass, n_fan=N_RAYS, nb=3)
        r = op.sample(eye, self.oleaves if leaves else [], n_rays=N_RAYS, max_events=EVENTS)
        assert np.array_equal(g["escape"][0], r["escape"])
        assert np.array_equal(g["raw"][0], r["raw"].astype(np.float32))
        assert np.array_equal(g["dir"][0], r["dir"])
        return dict(energy=g["energy"][0], dir=g["dir"][0])

    def release(self):
        self.scene.release()


def total_mid(r):
    return float(r["energy"][:, 1].sum())


@pytest.fixture(scope="module")
def world(wctx, oracle):
    w = DomeCase(wctx, oracle)
    yield w
    w.release()


def test_open_field_hears_the_dome_and_rooms_hear_slivers(world):
    """dome.rs:494-505."""
    open_ = total_mid(world.sample((18, 8, 1.6)))
    assert 0.4 < open_ < 1.0
    hall = total_mid(world.sample((7, 18, 1.6)))
    assert 1e-4 < hall < 0.25 * open_


def test_indoor_inflow_localizes_the_opening(world):
    """dome.rs:507-522."""
    r = world.sample((7, 18, 1.6))
    best = int(np.argmax(r["energy"][:, 1]))
    assert r["dir"][best][1] > 0.6


def test_interior_room_receives_through_two_doorways(world):
    """dome.rs:524-536."""
    t = total_mid(world.sample((4, 10, 1.6)))
    hall = total_mid(world.sample((7, 18, 1.6)))
    assert 1e-6 < t < hall


def test_leaf_coverage_sweeps_the_inflow(wctx, oracle):
    """dome.rs:538-570."""
    prev, open_t = float("inf"), 0.0
    for step in range(5):
        w = DomeCase(wctx, oracle, {2: 1.0 - step / 4})
        t = total_mid(w.sample((7, 20, 1.6), leaves=True))
        w.release()
        assert t <= prev + 1e-6
        if step == 0:
            open_t = t
        prev = t
    assert prev < 0.2 * open_t
    w = DomeCase(wctx, oracle, {1: 0.0, 2: 0.0})
    r = w.sample((7, 20, 1.6), leaves=True)
    w.release()
    assert r["energy"][:, 0].sum() > 8.0 * r["energy"][:, 2].sum()


def test_walls_beside_you_dampen_their_directions(world):
    """dome.rs:572-605."""
    r = world.sample((27.5, 24.5, 1.6))
    lateral = along = lat_zw = lat_e = 0.0
    for e, d in zip(r["energy"], r["dir"]):
        if d[2] > 0.8:
            continue
        if abs(d[1]) > 0.7:
            lateral += e[1]
            lat_zw += d[2] * e[1]
            lat_e += e[1]
        elif abs(d[0]) > 0.7:
            along += e[1]
    assert lateral < 0.72 * along
    assert lat_zw / max(lat_e, 1e-9) > 0.03


def test_indoor_inflow_is_never_unfiltered(world, wctx, oracle):
    """dome.rs:607-638."""
    r = world.sample((8, 66, 1.6))
    lo, hi = r["energy"][:, 0].sum(), r["energy"][:, 2].sum()
    open_ = total_mid(world.sample((8, 40, 1.6)))
    assert lo + hi < 0.25 * open_
    w = DomeCase(wctx, oracle, {6: 0.0})
    r2 = w.sample((8, 66, 1.6), leaves=True)
    w.release()
    assert r2["energy"][:, 0].sum() > 8.0 * r2["energy"][:, 2].sum()


def test_glass_transmits_with_its_spectrum(world):
    """dome.rs:640-654."""
    r = world.sample((27.5, 19.5, 4.6))
    lo, hi = r["energy"][:, 0].sum(), r["energy"][:, 2].sum()
    assert lo > 1e-5 and lo > 2.0 * hi


# ------------------------------------------------------------ late world gate
def test_mesh_late_field_matches_shoebox(wctx, oracle):
    """late_world_gate.rs:20-93, on omg_trace_world and omg_trace_box."""
    O = oracle
    ctx = wctx
    walls = [M.CONCRETE] * 4 + [M.WOOD_PANEL, M.CONCRETE]
    quads = [
        ([(0, 0, 0), (0, 4, 0), (0, 4, 3), (0, 0, 3)], 0),
        ([(6, 0, 0), (6, 0, 3), (6, 4, 3), (6, 4, 0)], 1),
        ([(0, 0, 0), (0, 0, 3), (6, 0, 3), (6, 0, 0)], 2),
        ([(0, 4, 0), (6, 4, 0), (6, 4, 3), (0, 4, 3)], 3),
        ([(0, 0, 0), (6, 0, 0), (6, 4, 0), (0, 4, 0)], 4),
        ([(0, 0, 3), (0, 4, 3), (6, 4, 3), (6, 0, 3)], 5),
    ]
    mb, ob = MeshBuilder(), O.MeshBuilder()
    for q, wi in quads:
        m = mb.material(walls[wi])
        mb.quad(*[np.float32(v) for v in q], m)
        om = ob.material(omat(O, walls[wi]))
        ob.quad(*[np.float32(v) for v in q], om)
    scene = ctx.upload_builder(mb)
    mesh = ob.build("f32")
    src, lis = (1.5, 1.0, 1.5), (4.5, 3.0, 1.6)
    size = (6.0, 4.0, 3.0)
    P = oparams(O, ctx.cfg)
    rt_box, lv_box, rt_mesh, lv_mesh = (np.zeros(3) for _ in range(4))
    for seed in range(4):
        eb, rb = ctx.trace_box(size, walls, src, lis, 16384, seed=100 + seed)
        em, rm = ctx.trace_world(scene, src, lis, 16384, seed=100 + seed)
        rt_box += rb.rt60[:3] / 4.0
        lv_box += rb.level[:3] / 4.0
        rt_mesh += rm.rt60[:3] / 4.0
        lv_mesh += rm.level[:3] / 4.0
        if seed == 0:
            # the oracle on the same per-ray streams
            b1, _, s1 = O.trace_box(size, [omat(O, w) for w in walls], src, lis, 16384, P=P, seed=100,
                                    threads=THREADS, acc64=True)
            b2, _, s2 = O.trace_mesh(mesh, src, lis, 16384, P=P, seed=100, threads=THREADS, acc64=True)
            assert rb.segments == s1["segments"] and rm.segments == s2["segments"]
            assert rel_bins(eb.bins, b1) <= 1e-5 and rel_bins(em.bins, b2) <= 1e-5
    scene.release()
    for b in range(3):
        r = rt_mesh[b] / rt_box[b]
        assert 0.8 <= r < 1.25, (b, rt_mesh, rt_box)
        lr = lv_mesh[b] / max(lv_box[b], 1e-6)
        assert 0.75 <= lr < 1.33, (b, lv_mesh, lv_box)


def _late_panels(D):
    furn, _ = furniture_world(lambda m: M.Material(tuple(m["absorption"]), m["scattering"],
                                                   tuple(m["transmission"])))
    return late_panels(D) + furn


def _wet(ctx, scene, panels, seeds=4, rays=16384):
    """world.rs:776-797 on the average of `seeds` traces (the sim's EMA at rest)."""
    src, lis = (2.0, 3.0, 1.5), (4.4, 7.5, 1.6)
    acc_b = acc_d = None
    for s in range(seeds):
        e, _ = ctx.trace_world(scene, src, lis, rays, panels=panels, seed=300 + s)
        acc_b = e.bins / seeds if acc_b is None else acc_b + e.bins / seeds
        acc_d = e.dirs / seeds if acc_d is None else acc_d + e.dirs / seeds
    avg = Echogram.wrap(acc_b.astype(np.float32), acc_d.astype(np.float32), ctx.cfg.bin_dt)
    rv = ctx.estimate_reverb(avg.bins)
    _, aniso = avg.late_direction(0.08)
    a = min(max(aniso, 0.0), 0.9)
    level = np.asarray(rv.level[:3], np.float64)
    diffuse = level[1] * np.sqrt(1.0 - a)
    send = level[1] * np.sqrt(a) if (a > 0.05 and level[1] > 1e-5) else 0.0
    return diffuse + send, send, float(rv.rt60[1])


def test_doorway_wet_is_measured_directional_and_door_sensitive(wctx):
    """late_world_gate.rs:96-144 (door 0 joins the living room and the corridor)."""
    ctx = wctx
    results = {}
    for name, opened in (("open", {}), ("closed", {0: 0.0}), ("reopened", {0: 1.0})):
        R, D, _ = _doors(opened)
        mb = MeshBuilder()
        build_world_mesh(mb, R, D)
        scene = ctx.upload_builder(mb)
        panels = _late_panels(D)
        assert len(panels) <= 64
        results[name] = _wet(ctx, scene, panels)
        scene.release()
    open_wet, open_send, rt60 = results["open"]
    assert open_wet > 1e-4, results
    assert open_send > 0.15 * open_wet, results
    assert 0.15 < rt60 < 3.0, results
    assert results["closed"][0] < 0.6 * open_wet, results
    assert results["reopened"][0] > 0.6 * open_wet, results
