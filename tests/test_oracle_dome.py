"""The oracle's dome (dome.rs:293-478) on the reference's walkthrough world,
held to the reference's own dome tests (dome.rs:496-654), and the product's
world builder (world.py) checked against the oracle's (dome.rs:79-258)."""
import copy

import numpy as np
import pytest

from walkthrough import leaf_panels, oracle_world, product_world

N_RAYS, EVENTS = 384, 6   # the High tier (quality.rs: dome rays 384, events 6)


def probe(O, doors=None, real="f32"):
    rooms, odoors = oracle_world(O, doors)
    mb = O.MeshBuilder()
    glass = O.world_build(mb, rooms, odoors)
    mesh = mb.build(real)
    return O.DomeProbe(mesh, glass, n_fan=N_RAYS, nb=3), mesh


def sample(p, eye, leaves=()):
    return p.sample(eye, list(leaves), n_rays=N_RAYS, max_events=EVENTS)


def total_mid(r):
    return float(r["energy"][:, 1].sum())


@pytest.fixture(scope="module")
def default_probe(oracle):
    return probe(oracle)[0]


def test_open_field_hears_the_dome_and_rooms_hear_slivers(oracle):
    """dome.rs:494-505."""
    O = oracle
    open_ = total_mid(sample(probe(O)[0], (18, 8, 1.6)))
    assert 0.4 < open_ < 1.0
    hall = total_mid(sample(probe(O)[0], (7, 18, 1.6)))
    assert hall < 0.25 * open_ and hall > 1e-4


def test_indoor_inflow_localizes_the_opening(oracle):
    """dome.rs:507-522."""
    r = sample(probe(oracle)[0], (7, 18, 1.6))
    best = int(np.argmax(r["energy"][:, 1]))
    assert r["dir"][best][1] > 0.6


def test_interior_room_receives_through_two_doorways(oracle):
    """dome.rs:524-536."""
    t = total_mid(sample(probe(oracle)[0], (4, 10, 1.6)))
    hall = total_mid(sample(probe(oracle)[0], (7, 18, 1.6)))
    assert t > 1e-6 and t < hall


def test_leaf_coverage_sweeps_the_inflow(oracle):
    """dome.rs:538-570."""
    O = oracle
    _, doors = __import__("walkthrough").load()
    prev, open_t = float("inf"), 0.0
    for step in range(5):
        d = copy.deepcopy(doors)
        d[2]["openness"] = 1.0 - step / 4
        t = total_mid(sample(probe(O, d)[0], (7, 20, 1.6), leaf_panels(d)))
        assert t <= prev + 1e-6
        if step == 0:
            open_t = t
        prev = t
    assert prev < 0.2 * open_t
    d = copy.deepcopy(doors)
    d[1]["openness"] = 0.0
    d[2]["openness"] = 0.0
    r = sample(probe(O, d)[0], (7, 20, 1.6), leaf_panels(d))
    lo, hi = r["energy"][:, 0].sum(), r["energy"][:, 2].sum()
    assert lo > 8.0 * hi


def test_walls_beside_you_dampen_their_directions(oracle):
    """dome.rs:572-605."""
    r = sample(probe(oracle)[0], (27.5, 24.5, 1.6))
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


def test_indoor_inflow_is_never_unfiltered(oracle):
    """dome.rs:607-638."""
    O = oracle
    r = sample(probe(O)[0], (8, 66, 1.6))
    lo, hi = r["energy"][:, 0].sum(), r["energy"][:, 2].sum()
    open_ = total_mid(sample(probe(O)[0], (8, 40, 1.6)))
    assert lo + hi < 0.25 * open_
    _, doors = __import__("walkthrough").load()
    d = copy.deepcopy(doors)
    d[6]["openness"] = 0.0
    r2 = sample(probe(O, d)[0], (8, 66, 1.6), leaf_panels(d))
    assert r2["energy"][:, 0].sum() > 8.0 * r2["energy"][:, 2].sum()


def test_glass_transmits_with_its_spectrum(oracle):
    """dome.rs:640-654."""
    r = sample(probe(oracle)[0], (27.5, 19.5, 4.6))
    lo, hi = r["energy"][:, 0].sum(), r["energy"][:, 2].sum()
    assert lo > 1e-5 and lo > 2.0 * hi


def test_product_world_builder_matches_the_oracle(oracle, built_lib):
    """world.py build_world_mesh / subrects produce the oracle's mesh and panes bit for bit."""
    from omg_audio_gb300 import MeshBuilder
    from omg_audio_gb300.world import build_world_mesh
    O = oracle
    R, D = product_world()
    mb = MeshBuilder()
    glass = build_world_mesh(mb, R, D)
    rooms, odoors = oracle_world(O)
    ob = O.MeshBuilder()
    oglass = O.world_build(ob, rooms, odoors)
    a, b = mb.export(), ob.export()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert len(glass) == len(oglass)
    for g, o in zip(glass, oglass):
        assert g.axis == o["axis"] and np.float32(g.plane) == np.float32(o["plane"])
        assert np.allclose(g.lat, o["lat"], rtol=0, atol=0) and np.allclose(g.z, o["z"], rtol=0, atol=0)
