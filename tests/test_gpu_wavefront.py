"""Wavefront rounds (a traversal kernel and a shading kernel over a queue of
live rays, the persistent kernel finishing the tail from the saved ray state)
and persistent-kernel epochs (rays parked between two segments and resumed in
full warps by the next launch) against the oracle, for hand-set launch shapes
and for the autotuner's pick.

Every shape traces the same rays with the same operations, so per job:
  - the segment count equals the f32-trajectory oracle's exactly;
  - the compensated FP32 histogram is within 1e-5 (relative, bins holding
    >= 1e-6 of the band total) of the oracle's f32 trajectories summed in FP64.
Shapes cover the three persistent kernels (per-lane state machine, warp-local
wavefront, cooperative 4-lane walks) alone and in epochs, on the binary and
the 4-wide tree, a hand-over after a few rounds, a hand-over at a live-ray
threshold, and rounds to the last ray.
"""
import dataclasses

import numpy as np
import pytest

from omg_audio_gb300 import Context, Job, MeshBuilder, TraceConfig, _lib
from omg_audio_gb300 import workloads as W

from test_gpu_parity import gpu_scene, oparams, rel_bins
from test_oracle_golden import GOLDEN, omat

pytestmark = pytest.mark.gpu

SHAPES = [dict(mode=0, wf_rounds=0, wf_tail=0, epochs=0),
          dict(mode=0, wf_rounds=3, wf_tail=0, epochs=0),
          dict(mode=0, wf_rounds=40, wf_tail=2000, epochs=0),
          dict(mode=0, wf_rounds=400, wf_tail=0, epochs=0),
          dict(mode=0, wf_rounds=0, wf_tail=0, epochs=6, park_pct=50),
          dict(mode=0, wf_rounds=0, wf_tail=0, epochs=32, park_pct=95),
          dict(mode=0, wf_rounds=5, wf_tail=0, epochs=4, park_pct=60),
          dict(mode=1, wf_rounds=0, wf_tail=0, epochs=0, walk_steps=8),
          dict(mode=1, wf_rounds=0, wf_tail=0, epochs=0, walk_steps=0),
          dict(mode=1, wf_rounds=0, wf_tail=0, epochs=6, park_pct=50, walk_steps=4),
          dict(mode=1, wf_rounds=0, wf_tail=0, epochs=32, park_pct=95, walk_steps=16),
          dict(mode=1, wf_rounds=5, wf_tail=0, epochs=4, park_pct=60, walk_steps=8),
          dict(mode=0, wf_rounds=0, wf_tail=0, epochs=0, walk_steps=8, wide=1),
          dict(mode=1, wf_rounds=0, wf_tail=0, epochs=3, park_pct=50, walk_steps=4, wide=1),
          dict(mode=2, wf_rounds=0, wf_tail=0, epochs=0, walk_steps=0),
          dict(mode=2, wf_rounds=0, wf_tail=0, epochs=0, walk_steps=3),
          dict(mode=2, wf_rounds=0, wf_tail=0, epochs=6, park_pct=50, walk_steps=0),
          dict(mode=2, wf_rounds=4, wf_tail=0, epochs=3, park_pct=60, walk_steps=8),
          dict(mode=0, tail_mode=2, wf_rounds=0, wf_tail=0, epochs=2, park_pct=30, walk_steps=0),
          dict(mode=0, tail_mode=2, wf_rounds=0, wf_tail=0, epochs=2, park_pct=30, walk_steps=0, wl_shade_min=1),
          dict(mode=1, wf_rounds=0, wf_tail=0, epochs=3, park_pct=50, walk_steps=0, wl_shade_min=4),
          dict(mode=2, wf_rounds=0, wf_tail=0, epochs=0, walk_steps=0, wl_shade_min=8)]
for _s in SHAPES:
    _s.setdefault("wide", 0)
    _s.setdefault("tail_mode", _s["mode"])
    _s.setdefault("wl_shade_min", 32)


def _launches(shape):
    """omg_batch_kernel_count for a shape: finalize, reverb, one persistent
    launch per epoch, and init + 2 per round + hand-over for wavefront rounds."""
    r, ep = shape.get("wf_rounds", 0), shape.get("epochs", 0)
    return 2 + max(ep, 1) + (2 + 2 * r if r else 0)


def _oracle_mesh(O, rec):
    ob = O.MeshBuilder()
    rec.replay(ob, lambda m: omat(O, m))
    return ob.build("f32")


@pytest.fixture(scope="module")
def mixed(oracle):
    """Two pairs of the 49k-primitive multiroom scene with its panes as panels,
    a 12-triangle shoebox mesh and an analytic shoebox, with their oracle
    results (3 bands, near-tie rule)."""
    O = oracle
    cfg = TraceConfig(tie_mode=1)
    ctx = Context(cfg)
    case = W.multiroom(seed=2)
    big = gpu_scene(ctx, case.recorder)
    box12 = W.shoebox12(seed=4)
    small = gpu_scene(ctx, box12.recorder)
    _, size, walls, bsrc, blis, _ = GOLDEN[0]
    jobs = [Job(case.pairs[0][0], case.pairs[0][1], 4096, seed=21, scene=big, panel_offset=0,
                n_panels=len(case.panels)),
            Job(box12.src, box12.lis, 3000, seed=22, scene=small),
            Job(case.pairs[5][0], case.pairs[5][1], 2048, seed=23, scene=big, panel_offset=0,
                n_panels=len(case.panels)),
            Job(bsrc, blis, 2500, seed=24, box_size=size, box_walls=walls)]
    P = oparams(O, cfg)
    om_big, om_small = _oracle_mesh(O, case.recorder), _oracle_mesh(O, box12.recorder)
    pan = [(mn, mx, omat(O, m)) for (mn, mx, m) in case.panels]
    ref = []
    for j in jobs:
        if j.box_size is not None:
            b, _, st = O.trace_box(j.box_size, [omat(O, m) for m in j.box_walls], j.src, j.lis, j.n_rays, P=P,
                                   seed=j.seed, threads=8, acc64=True)
        else:
            m = om_big if j.scene is big else om_small
            b, _, st = O.trace_mesh(m, j.src, j.lis, j.n_rays, P=P, seed=j.seed, threads=8, acc64=True,
                                    panels=pan if j.n_panels else ())
        ref.append((b, st["segments"]))
    yield ctx, jobs, case.panels, ref
    big.release()
    small.release()
    ctx.close()


@pytest.mark.parametrize("shape", SHAPES,
                         ids=[f"m{s['mode']}-r{s['wf_rounds']}-t{s['wf_tail']}-e{s['epochs']}-w{s.get('walk_steps', '')}"
                              f"{'-wide' if s['wide'] else ''}-t{s['tail_mode']}" for s in SHAPES])
def test_wavefront_shapes_match_the_oracle(mixed, shape):
    ctx, jobs, panels, ref = mixed
    b = ctx.batch(jobs, panels)
    b.set_shape(**shape)
    got = b.shape()
    assert all(got[k] == v for k, v in shape.items())
    assert b.kernel_count() == _launches(shape)
    for _ in range(2):          # the second launch reuses the recorded graph
        b.launch()
        res = b.read()
        for k, ((e, rv), (ob, segs)) in enumerate(zip(res, ref)):
            assert rv.segments == segs, (k, rv.segments, segs)
            assert rel_bins(e.bins, ob) <= 1e-5, k
    b.destroy()


def test_wavefront_eight_bands(oracle):
    """Batches with more than 3 bands run the 8-band kernels (two energy
    records per ray in the wavefront state)."""
    O = oracle
    cfg = TraceConfig(tie_mode=1)
    rooms = W.room_batch(seed=5, n_rooms=5, tri_median=400, tri_hi=2000, ray_lo=512, ray_hi=4096)
    with Context(cfg) as ctx:
        scenes, jobs = [], []
        for k, r in enumerate(rooms):
            mb = MeshBuilder()
            r.recorder.replay(mb)
            sc = ctx.upload_builder(mb, r.n_bands)
            scenes.append(sc)
            jobs.append(Job(r.src, r.lis, r.n_rays, seed=300 + k, scene=sc, n_bands=r.n_bands, n_bins=r.n_bins,
                            max_time=r.max_time))
        assert max(r.n_bands for r in rooms) == 8
        b = ctx.batch(jobs)
        for shape in (SHAPES[1], SHAPES[3], SHAPES[5], SHAPES[7], SHAPES[10], SHAPES[12], SHAPES[13], SHAPES[14],
                      SHAPES[16], SHAPES[18]):
            b.set_shape(**shape)
            b.launch()
            res = b.read()
            for k, (r, (e, rv)) in enumerate(zip(rooms, res)):
                P = oparams(O, cfg)
                P.n_bands, P.n_bins, P.max_time = r.n_bands, r.n_bins, r.max_time
                ob, _, st = O.trace_mesh(_oracle_mesh(O, r.recorder), r.src, r.lis, r.n_rays,
                                         energy=[1.0] * r.n_bands, P=P, seed=300 + k, threads=8, acc64=True)
                assert rv.segments == st["segments"], (shape, k)
                assert rel_bins(e.bins, ob) <= 1e-5, (shape, k)
        b.destroy()
        for sc in scenes:
            sc.release()


def test_autotuned_shape_keeps_the_result(mixed):
    ctx, jobs, panels, ref = mixed
    b = ctx.batch(jobs, panels)
    best = b.autotune(reps=1)
    assert best["ms"] > 0 and best == {**b.shape(), "ms": best["ms"]}
    b.launch()
    for (e, rv), (ob, segs) in zip(b.read(), ref):
        assert rv.segments == segs
        assert rel_bins(e.bins, ob) <= 1e-5
    b.destroy()


@pytest.mark.parametrize("shape", [SHAPES[0], SHAPES[8], SHAPES[13], SHAPES[14], SHAPES[18]],
                         ids=["m0", "m1", "m1-wide", "m2", "m0-tail2"])
def test_three_axis_sah_tree_keeps_the_result(mixed, shape):
    """The same jobs over the three-axis binned-SAH tree (OMG_BVH_SAH3): under
    the near-tie rule the closest hit does not depend on the tree, so segment
    counts and histograms equal the oracle's as on the reference's tree."""
    ctx, jobs, panels, ref = mixed
    case = W.multiroom(seed=2)
    big3 = gpu_scene(ctx, case.recorder, _lib.BVH_SAH3)
    big = jobs[0].scene
    jobs3 = [dataclasses.replace(j, scene=big3) if j.scene is big else j for j in jobs]
    b = ctx.batch(jobs3, panels)
    b.set_shape(**shape)
    b.launch()
    for k, ((e, rv), (ob, segs)) in enumerate(zip(b.read(), ref)):
        assert rv.segments == segs, (k, rv.segments, segs)
        assert rel_bins(e.bins, ob) <= 1e-5, k
    b.destroy()
    big3.release()
