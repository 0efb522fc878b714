"""Edge cases of the tracer against the oracle (exact segment counts,
histograms within 1e-5 per bin on bins holding >= 1e-6 of the band total):

- a mesh scene with no triangles: every ray misses at its first segment and
  only direct passes through the receiver sphere are recorded (tracer.rs:103-130:
  the receiver test runs before the miss ends the ray);
- a scene of one triangle (the tree is a single leaf) and a scene whose
  triangles include zero-area ones (Möller–Trumbore's |det| < 1e-9 rejects them);
- a shoebox job whose source lies outside the box (the ray is transmitted out:
  scene.rs:41-47 returns no hit);
- a listener at the source;
- invalid requests (a job without rays, alone or in a batch; bin counts above
  the reverb estimate's bound) rejected with OMG_E_INVALID, the context still
  usable afterwards;
- a host wait that runs out (OMG_E_TIMEOUT) while the batch keeps running, and a
  later read of the finished batch.
"""
import numpy as np
import pytest

from omg_audio_gb300 import Context, Job, MeshBuilder, TraceConfig, _lib
from omg_audio_gb300 import materials as M

from test_gpu_parity import oparams, rel_bins
from test_oracle_golden import omat

pytestmark = pytest.mark.gpu


def _pair(ctx, O, build, src, lis, n_rays=4096, seed=9):
    mb = MeshBuilder()
    ob = O.MeshBuilder()
    build(mb, ob)
    scene = ctx.upload_builder(mb, 3)
    e, rv = ctx.trace_world(scene, src, lis, n_rays, seed=seed)
    P = oparams(O, ctx.cfg)
    b, _, st = O.trace_mesh(ob.build("f32"), src, lis, n_rays, P=P, seed=seed, acc64=True)
    scene.release()
    return e, rv, b, st


@pytest.mark.parametrize("tie", [0, 1], ids=["first-found", "near-tie"])
def test_empty_mesh(oracle, tie):
    O = oracle
    with Context(TraceConfig(tie_mode=tie)) as ctx:
        e, rv, b, st = _pair(ctx, O, lambda mb, ob: None, (1.0, 1.0, 1.0), (1.3, 1.0, 1.0))
    assert rv.segments == st["segments"] == 4096
    assert rel_bins(e.bins, b) <= 1e-5
    assert e.bins.sum() > 0          # a few rays pass through the receiver sphere on their way out


@pytest.mark.parametrize("tie", [0, 1], ids=["first-found", "near-tie"])
def test_single_triangle_and_degenerate_triangles(oracle, tie):
    O = oracle

    def one(mb, ob):
        for b in (mb, ob):
            m = b.material(M.CONCRETE if b is mb else omat(O, M.CONCRETE))
            b.tri(np.float32([-5, -5, 0]), np.float32([5, -5, 0]), np.float32([0, 5, 0]), m)

    def degenerate(mb, ob):
        for b in (mb, ob):
            m = b.material(M.CONCRETE if b is mb else omat(O, M.CONCRETE))
            b.abox(np.float32([0, 0, 0]), np.float32([6, 4, 3]), m)
            # zero-area slivers inside the room: collinear corners and a repeated vertex
            b.tri(np.float32([1, 1, 1]), np.float32([2, 2, 2]), np.float32([3, 3, 3]), m)
            b.tri(np.float32([4, 1, 1]), np.float32([4, 1, 1]), np.float32([5, 2, 1]), m)

    with Context(TraceConfig(tie_mode=tie)) as ctx:
        for build, src, lis in ((one, (0.0, 0.0, 1.0), (0.5, 0.0, 1.5)), (degenerate, (1.5, 1.2, 1.4), (4.2, 2.6, 1.7))):
            e, rv, b, st = _pair(ctx, O, build, src, lis)
            assert rv.segments == st["segments"], build.__name__
            assert rel_bins(e.bins, b) <= 1e-5, build.__name__


def test_box_source_outside_and_listener_at_source(ctx, oracle):
    O = oracle
    walls = [M.CONCRETE] * 4 + [M.WOOD_PANEL, M.CONCRETE]
    for src, lis in (((7.0, 2.0, 1.5), (3.0, 2.0, 1.5)), ((2.0, 2.0, 1.5), (2.0, 2.0, 1.5))):
        e, rv = ctx.trace_box((6, 4, 3), walls, src, lis, 4096, seed=5)
        b, _, st = O.trace_box((6, 4, 3), [omat(O, m) for m in walls], src, lis, 4096, seed=5, acc64=True)
        assert rv.segments == st["segments"], src
        assert rel_bins(e.bins, b) <= 1e-5, src
    # a source outside: every ray leaves after one segment (heard only when it
    # passes the receiver sphere on its way)
    e, rv = ctx.trace_box((6, 4, 3), walls, (7.0, 2.0, 1.5), (3.0, 2.0, 1.5), 1024, seed=5)
    assert rv.segments == 1024


def test_invalid_requests_are_rejected(ctx):
    walls = [M.CONCRETE] * 6
    with pytest.raises(_lib.OmgError) as ex:
        ctx.trace_box((6, 4, 3), walls, (1, 1, 1), (2, 2, 2), 0)
    assert ex.value.status == _lib.E_INVALID
    with pytest.raises(_lib.OmgError):
        ctx.trace_batch([Job((1, 1, 1), (2, 2, 2), 64, box_size=(6, 4, 3), box_walls=walls),
                         Job((1, 1, 1), (2, 2, 2), 0, box_size=(6, 4, 3), box_walls=walls)])
    e, rv = ctx.trace_box((6, 4, 3), walls, (1, 1, 1), (2, 2, 2), 256, seed=1)   # still usable
    assert rv.segments >= 256 and np.isfinite(e.bins).all()


def test_bin_counts_above_the_reverb_bound_are_refused(ctx):
    """A bin count above 19,370 (the reverb estimate holds one band's curve in
    a block's 227 KB of shared memory) is refused up front: omg_create returns
    NULL, a job and an omg_estimate_reverb call get OMG_E_INVALID. The bound
    itself works, and the context stays usable."""
    with pytest.raises(Exception):
        Context(TraceConfig(n_bins=19371))
    walls = [M.CONCRETE] * 6
    with pytest.raises(_lib.OmgError) as ex:
        ctx.trace_batch([Job((1, 1, 1), (2, 2, 2), 64, box_size=(6, 4, 3), box_walls=walls, n_bins=19371)])
    assert ex.value.status == _lib.E_INVALID
    with pytest.raises(_lib.OmgError) as ex:
        ctx.estimate_reverb(np.ones((19371, 3), np.float32))
    assert ex.value.status == _lib.E_INVALID
    bins = np.exp(-np.arange(19370, dtype=np.float64) / 2000.0)[:, None].repeat(3, 1).astype(np.float32)
    rv = ctx.estimate_reverb(bins, bin_dt=0.001)
    assert np.all(np.isfinite(rv.rt60)) and np.all(rv.rt60 > 0)
    e, rv2 = ctx.trace_box((6, 4, 3), walls, (1, 1, 1), (2, 2, 2), 256, seed=1)   # still usable
    assert rv2.segments >= 256


def test_host_wait_times_out_and_the_context_stays_usable(oracle):
    """The host's bounded wait (timeout_ms = 1) gives up on a batch that runs
    ~10 ms and returns OMG_E_TIMEOUT; nothing on the device is interrupted.
    A later read of the same batch, once it has finished, returns the same
    result as a context with the default wait."""
    import time
    from omg_audio_gb300 import workloads as W
    case = W.multiroom(seed=2, n_pairs=64)
    cfg = dict(n_bands=3, n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200, energy_floor=1e-6, tie_mode=1)
    out = []
    for timeout in (1, 60000):
        with Context(TraceConfig(timeout_ms=timeout, **cfg)) as ctx:
            mb = MeshBuilder()
            case.recorder.replay(mb)
            scene = ctx.upload_builder(mb, 3, _lib.BVH_SAH3)
            jobs = [Job(src, lis, 4096, seed=1000 + p, scene=scene, panel_offset=0, n_panels=len(case.panels))
                    for p, (src, lis) in enumerate(case.pairs)]
            b = ctx.batch(jobs, case.panels)
            b.launch()
            if timeout == 1:
                with pytest.raises(_lib.OmgError) as ex:
                    b.read()
                assert ex.value.status == _lib.E_TIMEOUT
                time.sleep(1.0)                       # the batch finishes on its own
            res = seg = None
            for _ in range(50):                       # a read's own copies may still outlast a 1 ms wait
                try:
                    res = res or b.read()
                    seg = b.segments()
                    break
                except _lib.OmgError as e:
                    assert e.status == _lib.E_TIMEOUT
                    time.sleep(0.1)
            assert res is not None and seg is not None
            out.append((seg, res))
            b.destroy()
            scene.release()
    (s1, r1), (s2, r2) = out
    assert s1 == s2
    for (e1, v1), (e2, v2) in zip(r1, r2):
        assert v1.segments == v2.segments
        assert rel_bins(e1.bins, e2.bins) <= 1e-5
