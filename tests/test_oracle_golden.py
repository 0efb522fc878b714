"""The oracle pinned against the reference's own known-answer tests.

Golden vectors: crates/omg-core/tests/trace_golden.rs:51-108 (three shoeboxes,
[rt60 x3, late level dB x3, anisotropy]); tolerances :33-40 and :145-171;
averaging of 4 traces with the running-mean EMA :125-143. The oracle runs the
reference's own xorshift64* stream (rng.rs) with the reference's seeds, and the
per-ray PCG stream with the reference GPU parity test's seeds
(crates/omg-gpu/tests/parity.rs:30). Other known answers: lib.rs:57-101,
mesh.rs:697-784, tracer.rs:270-311.
"""
import numpy as np
import pytest

from omg_audio_gb300 import materials as M

GOLDEN_RAYS = 4096
GOLDEN_AVG = 4
GOLDEN_SEED = 0xC0FFEE
GOLDEN_LATE_S = 0.05
RT60_REL_TOL = 0.12
LEVEL_DB_TOL = 1.0
ANISO_TOL = 0.06
ANISO_LEVEL_FLOOR_DB = -40.0

GOLDEN = [
    ("live-room", (6.0, 4.0, 3.0), [M.CONCRETE] * 4 + [M.WOOD_PANEL, M.CONCRETE], (1.5, 1.0, 1.5), (4.5, 3.0, 1.6),
     [1.19, 1.05, 1.05, -6.8, -3.4, -4.7, 0.010]),
    ("dead-room", (12.0, 9.0, 4.0), [M.ACOUSTIC_TILE] * 4 + [M.CARPET, M.ACOUSTIC_TILE], (3.0, 2.0, 1.5),
     (9.0, 7.0, 1.6), [0.49, 0.20, 0.16, -26.6, -42.9, -50.5, 0.187]),
    ("hall", (16.0, 3.5, 3.0), [M.DRYWALL] * 4 + [M.WOOD_PANEL, M.CONCRETE], (1.5, 1.75, 1.5), (14.0, 1.75, 1.6),
     [0.75, 1.32, 1.46, -19.8, -10.3, -8.4, 0.014]),
]


def omat(O, m):
    return O.Material.make(m.absorption, m.scattering, m.transmission)


def metrics_of(O, bins, dirs, bin_dt=0.010):
    """trace_golden.rs:113-123."""
    rt, lv, _ = O.estimate_reverb(bins, bin_dt)
    _, an = O.late_direction(bins, dirs, bin_dt, GOLDEN_LATE_S)
    return list(rt) + [20 * np.log10(max(float(v), 1e-9)) for v in lv] + [an]


def assert_golden(name, got, expect):
    """trace_golden.rs:145-179."""
    for b in range(3):
        rel = abs(got[b] - expect[b]) / expect[b]
        assert rel <= RT60_REL_TOL, f"{name}: rt60[{b}] {got[b]:.3f} vs {expect[b]} ({rel:.1%})"
        tol = 4.0 if expect[3 + b] < ANISO_LEVEL_FLOOR_DB else LEVEL_DB_TOL
        assert abs(got[3 + b] - expect[3 + b]) <= tol, f"{name}: level[{b}] {got[3 + b]:.2f} vs {expect[3 + b]}"
    if expect[4] > ANISO_LEVEL_FLOOR_DB:
        assert abs(got[6] - expect[6]) <= ANISO_TOL, f"{name}: aniso {got[6]:.3f} vs {expect[6]}"


def run_avg(trace_one, k_seeds):
    """Running mean of GOLDEN_AVG traces in f32 (trace_golden.rs:125-143)."""
    avg = avgd = None
    for k, seed in enumerate(k_seeds):
        b, d = trace_one(seed)
        b, d = b.astype(np.float32), d.astype(np.float32)
        if avg is None:
            avg, avgd = np.zeros_like(b), np.zeros_like(d)
        a = np.float32(1.0 / (k + 1))
        avg += a * (b - avg)
        avgd += a * (d - avgd)
    return avg, avgd


@pytest.mark.parametrize("seed", [GOLDEN_SEED, 0x5EED_5EED])
@pytest.mark.parametrize("cfg", GOLDEN, ids=[c[0] for c in GOLDEN])
def test_oracle_xorshift_within_goldens(oracle, cfg, seed):
    """cpu_tracer_within_goldens (trace_golden.rs:202-210): the reference's stream and seeds."""
    O = oracle
    name, size, walls, src, lis, expect = cfg
    w = [omat(O, m) for m in walls]
    seeds = [(seed + k * 0x9E3779B97F4A7C15) % (1 << 64) for k in range(GOLDEN_AVG)]
    avg, avgd = run_avg(lambda s: O.trace_box(size, w, src, lis, GOLDEN_RAYS, rng="xorshift", seed=s)[:2], seeds)
    assert_golden(name, metrics_of(O, avg, avgd), expect)


GPU_SEEDS = [(0xD15EA5E ^ ((k * 0x85EBCA6B) & 0xFFFFFFFF)) for k in range(GOLDEN_AVG)]  # parity.rs:30


@pytest.mark.parametrize("real", ["f32", "f64"])
@pytest.mark.parametrize("cfg", GOLDEN, ids=[c[0] for c in GOLDEN])
def test_oracle_pcg_within_goldens(oracle, cfg, real):
    """The per-ray stream the GPU uses lands in the same tolerances (parity.rs:15-42 seeds)."""
    O = oracle
    name, size, walls, src, lis, expect = cfg
    w = [omat(O, m) for m in walls]
    avg, avgd = run_avg(lambda s: O.trace_box(size, w, src, lis, GOLDEN_RAYS, real=real, rng="pcg", seed=s)[:2],
                        GPU_SEEDS)
    assert_golden(name, metrics_of(O, avg, avgd), expect)


def test_xorshift_stream_known_values(oracle):
    """rng.rs:9-21 restated: first draws of Rng::new(1), computed by hand here."""
    x = 1
    want = []
    for _ in range(4):
        x ^= x >> 12
        x ^= (x << 25) & 0xFFFFFFFFFFFFFFFF
        x ^= x >> 27
        want.append((x * 0x2545F4914F6CDD1D) & 0xFFFFFFFFFFFFFFFF)
    assert list(oracle.xorshift_draws(1, 4)) == want
    # Rng::new(0) clamps to 1 (rng.rs:5-7)
    assert list(oracle.xorshift_draws(0, 4)) == want


def test_pcg_stream_known_values(oracle):
    """trace_mesh.wgsl:90-94, 211-213 restated in Python integers."""
    def draws(seed, ray, n):
        s = ((seed ^ ((ray * 0x9E3779B9) & 0xFFFFFFFF)) + 1) & 0xFFFFFFFF
        out = []
        for i in range(n + 2):
            s = (s * 747796405 + 2891336453) & 0xFFFFFFFF
            w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
            out.append((w >> 22) ^ w)
        return out[2:]
    for seed, ray in [(1, 0), (0xD15EA5E, 7), (0xFFFFFFFF, 123456)]:
        assert list(oracle.pcg_draws(seed, ray, 6)) == draws(seed, ray, 6)


def test_rt60_tracks_absorption(oracle):
    """lib.rs:169-190: concrete > 2x tile; drywall Sabine in (0.8, 3.0)."""
    O = oracle

    def rt(mat):
        b, d, _ = O.trace_box((8, 6, 3), [omat(O, mat)] * 6, (2, 2, 1.5), (5, 4, 1.5), 20000, rng="xorshift", seed=7)
        return O.estimate_reverb(b, 0.010)[0][1]

    live, dead = rt(M.CONCRETE), rt(M.ACOUSTIC_TILE)
    assert live > 2 * dead
    assert 0.8 < rt(M.DRYWALL) < 3.0


def test_late_level_distance_independent(oracle):
    """lib.rs:192-213."""
    O = oracle
    w = [omat(O, M.DRYWALL)] * 6

    def level(lis, seed):
        b, _, _ = O.trace_box((10, 8, 4), w, (2, 4, 1.5), lis, 40000, rng="xorshift", seed=seed)
        return O.estimate_reverb(b, 0.010)[1][1]

    ratio = level((3, 4, 1.5), 11) / max(level((8, 4, 1.5), 12), 1e-6)
    assert 0.5 <= ratio < 2.0


def test_bvh_matches_brute_force(oracle):
    """mesh.rs:696-735: 200-tri soup, 500 rays, |dt| < 1e-4, same hit/miss."""
    O = oracle
    rng = np.random.default_rng(7)
    mb = O.MeshBuilder()
    m = mb.material(omat(O, M.CONCRETE))
    for _ in range(200):
        base = rng.uniform(0, 20, 3)
        u = rng.normal(size=(2, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        mb.tri(base, base + 2 * u[0], base + 2 * u[1], m)
    mesh = mb.build("f32")
    o = rng.uniform(0, 20, (500, 3)).astype(np.float32)
    d = rng.normal(size=(500, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tb, _, _ = mesh.raycast(o, d)
    tr, _, _ = mesh.raycast(o, d, brute=True)
    assert np.array_equal(tb < 0, tr < 0)
    hit = tb >= 0
    assert np.all(np.abs(tb[hit] - tr[hit]) < 1e-4)


def test_box_mesh_traces_like_shoebox(oracle):
    """mesh.rs:737-768: 8192 rays; RT60 ratio in [0.8, 1.25), level ratio in [0.7, 1.4)."""
    O = oracle
    mb = O.MeshBuilder()
    mb.abox((0, 0, 0), (8, 6, 3), mb.material(omat(O, M.CONCRETE)))
    mesh = mb.build("f32")
    w = [omat(O, M.CONCRETE)] * 6
    bb, _, _ = O.trace_box((8, 6, 3), w, (2, 3, 1.5), (6, 2, 1.6), 8192, rng="xorshift", seed=42)
    bm, _, _ = O.trace_mesh(mesh, (2, 3, 1.5), (6, 2, 1.6), 8192, rng="xorshift", seed=42)
    rb, lb, _ = O.estimate_reverb(bb, 0.010)
    rm, lm, _ = O.estimate_reverb(bm, 0.010)
    for b in range(3):
        assert 0.8 <= rm[b] / rb[b] < 1.25
        assert 0.7 <= lm[b] / max(lb[b], 1e-9) < 1.4


def test_segment_hits_counts_wall_crossings(oracle):
    """mesh.rs:770-784."""
    O = oracle
    mb = O.MeshBuilder()
    mb.abox((0, 0, 0), (4, 4, 3), mb.material(omat(O, M.CONCRETE)))
    mesh = mb.build("f32")
    t, _, _ = mesh.segment_hits((-2, 2, 1.5), (6, 2, 1.5))
    assert len(t) == 2 and t[0] < t[1]
    assert len(mesh.segment_hits((-2, 2, 1.5), (2, 2, 1.5))[0]) == 1
    assert len(mesh.segment_hits((1, 2, 1.5), (3, 2, 1.5))[0]) == 0


def holed_room(O):
    """tracer.rs:272-285 / mesh_parity.rs:16-29: shell with a doorway in x=8."""
    mb = O.MeshBuilder()
    m = mb.material(omat(O, M.CONCRETE))
    v = lambda x, y, z: (x, y, z)
    mb.quad(v(0, 0, 0), v(0, 6, 0), v(0, 6, 3), v(0, 0, 3), m)
    mb.quad(v(0, 0, 0), v(8, 0, 0), v(8, 0, 3), v(0, 0, 3), m)
    mb.quad(v(0, 6, 0), v(8, 6, 0), v(8, 6, 3), v(0, 6, 3), m)
    mb.quad(v(0, 0, 0), v(8, 0, 0), v(8, 6, 0), v(0, 6, 0), m)
    mb.quad(v(0, 0, 3), v(8, 0, 3), v(8, 6, 3), v(0, 6, 3), m)
    mb.quad(v(8, 0, 0), v(8, 2.5, 0), v(8, 2.5, 3), v(8, 0, 3), m)
    mb.quad(v(8, 3.5, 0), v(8, 6, 0), v(8, 6, 3), v(8, 3.5, 3), m)
    mb.quad(v(8, 2.5, 2.1), v(8, 3.5, 2.1), v(8, 3.5, 3), v(8, 2.5, 3), m)
    return mb


def test_reverb_through_a_hole_reports_the_hole_direction(oracle):
    """tracer.rs:270-299."""
    O = oracle
    mesh = holed_room(O).build("f32")
    lis = np.array([12.0, 3.0, 1.6])
    b, d, _ = O.trace_mesh(mesh, (2, 3, 1.5), lis, 16384, rng="xorshift", seed=21)
    dirv, an = O.late_direction(b, d, 0.010, 0.05)
    to_hole = np.array([8.0, 3.0, 1.05]) - lis
    to_hole /= np.linalg.norm(to_hole)
    assert float(np.dot(dirv, to_hole)) > 0.85
    assert an > 0.5


def test_closed_room_late_field_is_diffuse(oracle):
    """tracer.rs:301-311."""
    O = oracle
    b, d, _ = O.trace_box((8, 6, 3), [omat(O, M.DRYWALL)] * 6, (2, 3, 1.5), (6, 2, 1.6), 16384, rng="xorshift",
                          seed=5)
    _, an = O.late_direction(b, d, 0.010, 0.15)
    assert an < 0.35


def test_f32_and_f64_oracles_agree_on_the_stream(oracle):
    """Same per-ray stream: the f32 and FP64 restatements give RT60 within 1%."""
    O = oracle
    w = [omat(O, m) for m in GOLDEN[0][2]]
    b32, _, s32 = O.trace_box((6, 4, 3), w, (1.5, 1, 1.5), (4.5, 3, 1.6), 8192, real="f32", seed=99)
    b64, _, s64 = O.trace_box((6, 4, 3), w, (1.5, 1, 1.5), (4.5, 3, 1.6), 8192, real="f64", seed=99)
    r32 = O.estimate_reverb(b32, 0.010, level_f32=False)[0]
    r64 = O.estimate_reverb(b64, 0.010, level_f32=False)[0]
    assert np.all(np.abs(r32 / r64 - 1) < 0.01)
    assert abs(s32["segments"] - s64["segments"]) < 0.001 * s64["segments"]


def test_f32_sincos_error_bound(oracle):
    """The f32 sin/cos both sides use for ray directions (Cody-Waite + Taylor)
    stays within 3 ulp of the true values on [0, 2*pi]."""
    phi = (np.float32(6.2831855) * np.arange(1 << 18, dtype=np.float64) / (1 << 18)).astype(np.float32)
    s, c = oracle.sincos_f32(phi)
    S, Cc = np.sin(phi.astype(np.float64)), np.cos(phi.astype(np.float64))
    for got, want in ((s, S), (c, Cc)):
        big = np.abs(want) > 1e-3
        ulp = np.spacing(np.abs(want[big]).astype(np.float32)).astype(np.float64)
        assert np.max(np.abs(got[big] - want[big]) / ulp) <= 3.0
        assert np.max(np.abs(got - want)) < 2e-7
