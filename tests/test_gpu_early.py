"""World early reflections on the GPU (omg_early_*) against the oracle's
restatement of pt_mesh.rs, on the reference's own acceptance world
(crates/omg-gpu/tests/solve_parity.rs: the walkthrough world with its
furniture as reflectors and blockers and two shut door leaves).

Tolerances: the discovered chain lists equal the oracle's, in order; every
(source, chain) pair solves on the GPU exactly when it solves on the oracle
(the reference's own test allows 0.5 % mismatches; here the arithmetic is the
same, so none are expected), with identical delay and direction and gains
within 2e-6 relative (exp of the air attenuation is the only transcendental).
"""
import time

import numpy as np
import pytest

from omg_audio_gb300 import Context, MeshBuilder, TraceConfig, _lib
from omg_audio_gb300 import materials as M
from omg_audio_gb300.early import WorldEarly
from omg_audio_gb300.materials import Material
from omg_audio_gb300.world import build_world_mesh

from test_oracle_early import BOX_QUADS, box_mesh, omat
from walkthrough import furniture_world, oracle_world, product_world

pytestmark = pytest.mark.gpu

NO = 0xFFFF
SPOTS = [(10.5, 20.5, 1.6), (4.4, 7.5, 1.6), (7.0, 27.0, 1.6)]     # solve_parity.rs:99-103
SOURCES = [(8, (10.5, 20.5, 1.2)), (16, (2.0, 2.0, 1.0)), (24, (31.5, 18.0, 1.4)),
           (32, (7.0, 30.0, 1.7)), (40, (18.0, 9.0, 2.2)), (48, (4.0, 25.0, 0.8))]   # :106-113


@pytest.fixture(scope="module")
def world(oracle):
    O = oracle
    ctx = Context(TraceConfig())
    R, D = product_world()
    mb = MeshBuilder()
    build_world_mesh(mb, R, D)
    scene = ctx.upload_builder(mb, 3, _lib.BVH_SAH)
    furn_g, extras = furniture_world(lambda m: Material(tuple(m["absorption"]), m["scattering"],
                                                         tuple(m["transmission"])))
    furn_o, _ = furniture_world(lambda m: O.Material.make(m["absorption"], m["scattering"], m["transmission"]))
    early = WorldEarly(ctx, scene, furn_g)
    rooms, odoors = oracle_world(O)
    ob = O.MeshBuilder()
    O.world_build(ob, rooms, odoors)
    om = ob.build("f32")
    oe = O.Early(om, furn_o)
    yield ctx, early, oe, extras
    early.close()
    scene.release()
    ctx.close()


def test_surface_table_matches(world):
    ctx, early, oe, _ = world
    assert early.base_overlay == oe.base_overlay
    assert early.n_surfaces == oe.n_surfaces


@pytest.mark.parametrize("spot", range(3))
def test_discovery_matches_the_oracle(world, spot):
    ctx, early, oe, _ = world
    for rot in (0, 1, 7):
        for use_boxes in (True, False):
            g = early.discover(SPOTS[spot], 768, rot, use_boxes)
            o = oe.discover(SPOTS[spot], 768, rot, use_boxes)
            assert g == o, (rot, use_boxes, len(g), len(o))
            assert len(g) > 20


def _chain_list(oe, lis, cap=400):
    """solve_parity.rs:64-79: direct first, then 6 rotations' chains sorted."""
    cs = set()
    for rot in range(6):
        cs.update(oe.discover(lis, 768, rot))
    return [((NO, NO, NO), 0)] + sorted(cs)[:cap - 1]


def test_batched_solve_matches_the_oracle(world):
    ctx, early, oe, extras = world
    total = solved = 0
    for lis in SPOTS:
        chains = _chain_list(oe, lis)
        rec = early.solve(SOURCES, chains, lis, extras)
        ref, valid = oe.solve(SOURCES, chains, lis, extras, threads=8)
        assert rec.shape == valid.shape
        gv = rec["valid"].astype(bool)
        assert np.array_equal(gv, valid), np.argwhere(gv != valid)[:5]
        total += valid.size
        solved += int(valid.sum())
        r = rec[gv]
        o = ref[valid]
        assert np.array_equal(r["delay_s"], o[:, 0])
        assert np.array_equal(r["dir"], o[:, 1:4])
        assert np.all(np.abs(r["gains"] - o[:, 4:7]) <= 2e-6 * np.abs(o[:, 4:7]) + 1e-30)
        # records carry their source, chain and key (pt_mesh.rs:123-134)
        for si, (sid, _) in enumerate(SOURCES):
            assert np.all(rec["source"][si] == sid)
        for c, (ch, order) in enumerate(chains):
            assert np.all(rec["order"][:, c] == order)
        k = rec[gv]
        for row in k[:50]:
            h = (0x811C9DC5 ^ int(row["source"])) & 0xFFFFFFFF
            for q in range(int(row["order"])):
                h = ((h ^ int(row["chain"][q])) * 16777619) & 0xFFFFFFFF
            assert int(row["key"]) == ((h ^ 0xA5) * 16777619) & 0xFFFFFFFF
    print(f"batched solve parity: {total} pairs, {solved} solved")
    assert solved > 200                          # solve_parity.rs:183 (the world is not degenerate)


def test_hundred_source_batch(world):
    """solve_parity.rs:192-265: 100 sources against the full chain list in one
    launch, far under what the CPU pays per source."""
    ctx, early, oe, extras = world
    lis = (7.0, 27.0, 1.6)
    chains = _chain_list(oe, lis)
    srcs = [(i * 8, (2.0 + (i * 0.83) % 38.0, 2.0 + (i * 1.37) % 30.0, 0.8 + (i * 0.11) % 2.0)) for i in range(100)]
    rec = early.solve(srcs, chains, lis, extras)
    assert int(rec["valid"].sum()) > 100
    t0 = time.perf_counter()
    for _ in range(10):
        early.solve(srcs, chains, lis, extras)
    gpu_ms = (time.perf_counter() - t0) * 100.0
    t1 = time.perf_counter()
    oe.solve(srcs[1:2], chains, lis, extras)
    cpu_one_ms = (time.perf_counter() - t1) * 1000.0
    print(f"100 sources x {len(chains)} chains: {gpu_ms:.2f} ms per call; oracle {cpu_one_ms:.2f} ms per source")
    assert gpu_ms < max(cpu_one_ms * 8.0, 10.0)


def test_box_and_table_top_on_the_gpu(oracle):
    """pt_mesh_gate.rs box world and overlay face through the GPU entry points,
    equal to the oracle."""
    O = oracle
    with Context(TraceConfig()) as ctx:
        mb = MeshBuilder()
        mat = mb.material(M.CONCRETE)
        for q, _ in BOX_QUADS:
            mb.begin_surface()
            mb.quad(*[np.float32(p) for p in q], mat)
        scene = ctx.upload_builder(mb, 3, _lib.BVH_SAH)
        mn, mx = (2.0, 1.5, 0.0), (3.0, 2.5, 0.8)
        early = WorldEarly(ctx, scene, [(mn, mx, M.WOOD_PANEL)])
        oe = O.Early(box_mesh(O, [M.CONCRETE] * 6), [(mn, mx, omat(O, M.WOOD_PANEL))])
        lis, src = (4.0, 2.0, 1.6), (1.0, 2.0, 1.5)
        for rot in range(4):
            assert early.discover(lis, 4096, rot) == oe.discover(lis, 4096, rot)
        top = early.base_overlay + 5
        rec = early.solve([(0, src)], [((top, NO, NO), 1)], lis)
        assert rec["valid"][0, 0]
        want = np.linalg.norm(np.subtract((1.0, 2.0, 2 * 0.8 - 1.5), lis)) / 343.0
        assert abs(float(rec["delay_s"][0, 0]) - want) < 1e-5
        off = early.solve([(0, src)], [((top, NO, NO), 1)], (1.2, 0.3, 1.6))
        assert not off["valid"][0, 0]
        early.close()
        scene.release()
