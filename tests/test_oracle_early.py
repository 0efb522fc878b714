"""The oracle's restatement of the world-mesh early reflections (pt_mesh.rs)
pinned by the reference's own gates (crates/omg-scene/tests/pt_mesh_gate.rs):
the mesh solver agrees with the analytic image sources in a box, doorways
thread without portal code on the walkthrough world, and a furniture face
reflects exactly. CPU only."""
import itertools
import json
import os

import numpy as np
import pytest

from omg_audio_gb300 import materials as M
from walkthrough import HERE, oracle_world

NO = 0xFFFF
AIR = np.float32([1.0e-4, 5.0e-4, 3.0e-3])     # material.rs:76


def db(v):
    return 20.0 * np.log10(np.maximum(np.asarray(v, np.float64), 1e-9))


def omat(O, m):
    return O.Material.make(m.absorption, m.scattering, m.transmission)


BOX_QUADS = [([(0, 0, 0), (0, 4, 0), (0, 4, 3), (0, 0, 3)], 0),
             ([(6, 0, 0), (6, 0, 3), (6, 4, 3), (6, 4, 0)], 1),
             ([(0, 0, 0), (0, 0, 3), (6, 0, 3), (6, 0, 0)], 2),
             ([(0, 4, 0), (6, 4, 0), (6, 4, 3), (0, 4, 3)], 3),
             ([(0, 0, 0), (6, 0, 0), (6, 4, 0), (0, 4, 0)], 4),
             ([(0, 0, 3), (0, 4, 3), (6, 4, 3), (6, 0, 3)], 5)]


def box_mesh(O, walls):
    """pt_mesh_gate.rs:26-51: a 6 x 4 x 3 m box, one authored surface per wall."""
    mb = O.MeshBuilder()
    for q, wi in BOX_QUADS:
        m = mb.material(omat(O, walls[wi]))
        mb.begin_surface()
        mb.quad(*[np.float32(p) for p in q], m)
    return mb.build("f32")


def analytic_images(src, walls, size=(6.0, 4.0, 3.0), max_order=3):
    """Image sources of the shoebox up to max_order (wall sequences without an
    immediate repeat): (order, image, reflection amplitude product)."""
    planes = [(0, 0.0), (0, size[0]), (1, 0.0), (1, size[1]), (2, 0.0), (2, size[2])]
    out = [(0, np.float64(src), np.ones(3))]
    for order in range(1, max_order + 1):
        for seq in itertools.product(range(6), repeat=order):
            if any(seq[i] == seq[i + 1] for i in range(order - 1)):
                continue
            p = np.array(src, np.float64)
            g = np.ones(3)
            for w in reversed(seq):
                a, c = planes[w]
                p[a] = 2 * c - p[a]
            for w in seq:
                g *= np.sqrt(np.maximum(1.0 - np.asarray(walls[w].absorption, np.float64), 0.0))
            out.append((order, p, g))
    return out


def record_of(img, g, lis):
    d = float(np.linalg.norm(img - np.asarray(lis, np.float64)))
    dt = max(d, 0.3)
    return d / 343.0, np.exp(-AIR * dt) / dt * g


def test_mesh_solver_matches_analytic_in_a_box(oracle):
    """pt_mesh_gate.rs:24-123: every mesh record matches an analytic image
    (delay <= 0.5 ms, every band within 1 dB); discovery finds >= 80 % of the
    order <= 2 set; the direct path is exact."""
    O = oracle
    walls = [M.CONCRETE] * 4 + [M.WOOD_PANEL, M.CONCRETE]
    mesh = box_mesh(O, walls)
    E = O.Early(mesh)
    src, lis = (1.5, 1.0, 1.5), (4.5, 3.0, 1.6)
    chains = set()
    for rot in range(8):
        chains.update(E.discover(lis, 4096, rot))
    chains = sorted(chains)
    lst = [((NO, NO, NO), 0)] + chains
    out, valid = E.solve([(0, src)], lst, lis)
    recs = [(lst[c][1], out[0, c]) for c in range(len(lst)) if valid[0, c]]
    assert recs and recs[0][0] == 0
    refs = [(o,) + record_of(p, g, lis) for (o, p, g) in analytic_images(src, walls)]

    def match(delay, gains, ref):
        return abs(ref[1] - delay) * 1000 <= 0.5 and np.all(np.abs(db(ref[2]) - db(gains)) <= 1.0)

    for order, r in recs:
        assert any(match(r[0], r[4:7], q) for q in refs), (order, r[0] * 1000)
    low = [q for q in refs if q[0] <= 2]
    found = sum(any(match(r[0], r[4:7], q) for _, r in recs) for q in low)
    assert found * 10 >= len(low) * 8, (found, len(low))
    d = recs[0][1]
    assert abs(d[0] - np.linalg.norm(np.subtract(src, lis)) / 343.0) < 1e-5


def _walkthrough_mesh(O):
    rooms, odoors = oracle_world(O)
    mb = O.MeshBuilder()
    O.world_build(mb, rooms, odoors)
    return mb.build("f32")


def test_doorways_thread_with_zero_portal_code(oracle):
    """pt_mesh_gate.rs:125-185: the piano in the living room reaches a corridor
    listener through the door hole at about free-space level; a listener behind
    masonry gets only mass-law transmission, >= 20 dB lower, bass above treble."""
    O = oracle
    E = O.Early(_walkthrough_mesh(O))
    src, clear, blocked = (2.0, 3.0, 1.5), (4.4, 7.5, 1.6), (1.0, 7.5, 1.6)
    direct = [((NO, NO, NO), 0)]
    out, valid = E.solve([(0, src)], direct, clear)
    assert valid[0, 0], "direct through the door hole"
    free = 1.0 / np.linalg.norm(np.subtract(src, clear))
    assert abs(db(out[0, 0, 5]) - db(free)) < 3.0
    out2, valid2 = E.solve([(0, src)], direct, blocked)
    if valid2[0, 0]:
        assert db(out2[0, 0, 5]) < db(out[0, 0, 5]) - 20.0
        assert db(out2[0, 0, 4]) - db(out2[0, 0, 6]) > 6.0


def test_overlay_face_reflects_exactly(oracle):
    """pt_mesh_gate.rs:191-244: the table-top chain solves to the exact mirror
    across z = 0.8, refuses a listener off the face rect, and discovery finds it."""
    O = oracle
    mesh = box_mesh(O, [M.CONCRETE] * 6)
    mn, mx = (2.0, 1.5, 0.0), (3.0, 2.5, 0.8)
    E = O.Early(mesh, [(mn, mx, omat(O, M.WOOD_PANEL))])
    top = E.base_overlay + 5
    assert E.n_surfaces == E.base_overlay + 6
    src, lis = (1.0, 2.0, 1.5), (4.0, 2.0, 1.6)
    out, valid = E.solve([(0, src)], [((top, NO, NO), 1)], lis)
    assert valid[0, 0], "table-top bounce must solve"
    want = np.linalg.norm(np.subtract((1.0, 2.0, 2 * 0.8 - 1.5), lis)) / 343.0
    assert abs(out[0, 0, 0] - want) < 1e-5
    assert out[0, 0, 5] > 1e-4 and out[0, 0, 3] < -0.1
    _, v_off = E.solve([(0, src)], [((top, NO, NO), 1)], (1.2, 0.3, 1.6))
    assert not v_off[0, 0]
    found = False
    for rot in range(4):
        found |= any(o >= 1 and top in c[:o] for c, o in E.discover(lis, 4096, rot))
    assert found, "discovery must bounce off the table top"


def test_discovery_is_deterministic_and_rotates(oracle):
    """mesh_chains: the same (listener, rot) gives the same list in the same
    order; chains are unique; another rot changes the fan."""
    O = oracle
    E = O.Early(_walkthrough_mesh(O))
    lis = (10.5, 20.5, 1.6)
    a, b, c = E.discover(lis, 768, 3), E.discover(lis, 768, 3), E.discover(lis, 768, 4)
    assert a == b and len(set(a)) == len(a) and a != c
    assert all(1 <= o <= 3 and all(s != NO for s in ch[:o]) and all(s == NO for s in ch[o:]) for ch, o in a)


def test_walkthrough_furniture_fixture():
    """walkthrough.rs:535-672: furniture rows parallel to their materials."""
    with open(os.path.join(HERE, "golden", "walkthrough_world.json")) as fh:
        d = json.load(fh)
    assert d["furn_reflector_min_vol"] == 0.25
    assert sum(len(v) for v in d["furniture"].values()) == 37
    for room, boxes in d["furniture"].items():
        for b in boxes:
            assert all(lo <= hi for lo, hi in zip(b["min"], b["max"]))
            assert b["transmission"] == b["material"]["transmission"]


def test_reference_acceptance_world_is_not_degenerate(oracle):
    """solve_parity.rs:24-61, 183: on the walkthrough world with its furniture
    and two shut leaves, the oracle solves more than 200 of the pairs of three
    listener spots x six sources."""
    from walkthrough import furniture_world
    O = oracle
    furn, extras = furniture_world(lambda m: O.Material.make(m["absorption"], m["scattering"], m["transmission"]))
    assert len(furn) > 10 and len(extras) == 39
    E = O.Early(_walkthrough_mesh(O), furn)
    srcs = [(8, (10.5, 20.5, 1.2)), (16, (2.0, 2.0, 1.0)), (24, (31.5, 18.0, 1.4)), (32, (7.0, 30.0, 1.7)),
            (40, (18.0, 9.0, 2.2)), (48, (4.0, 25.0, 0.8))]
    solved = 0
    for lis in [(10.5, 20.5, 1.6), (4.4, 7.5, 1.6), (7.0, 27.0, 1.6)]:
        cs = set()
        for rot in range(6):
            cs.update(E.discover(lis, 768, rot))
        chains = [((NO, NO, NO), 0)] + sorted(cs)[:399]
        _, valid = E.solve(srcs, chains, lis, extras, threads=8)
        solved += int(valid.sum())
    assert solved > 200, solved
