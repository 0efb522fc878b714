"""Device-side limits driven to their error status, on the GPU, without a fault.

Every walk carries a node budget (flag 4) and every persistent trace kernel a
per-warp loop guard (flag 8). Both end the kernel's work early and let it
return, so a test can make them run out on purpose: omg_set_limits makes them
tiny, the call returns OMG_E_OVERFLOW with the flag in omg_last_flags, and
after the limits are put back the SAME context traces the same job exactly as
the oracle does (segment count equal, bins within 1e-5 per bin on bins holding
>= 1e-6 of the band total). The no-alloc entry point reports the same flags
through its device flag word.
"""
import ctypes as C

import numpy as np
import pytest

from omg_audio_gb300 import Context, MeshBuilder, TraceConfig, _lib
from omg_audio_gb300 import materials as M
from omg_audio_gb300 import workloads as W

from test_gpu_parity import oparams, rel_bins
from test_oracle_golden import omat

pytestmark = pytest.mark.gpu

CFG = dict(n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200, energy_floor=1e-6)


def _scene_pair(ctx, O):
    case = W.shoebox12(seed=1)
    mb = MeshBuilder()
    case.recorder.replay(mb)
    scene = ctx.upload_builder(mb)
    ob = O.MeshBuilder()
    case.recorder.replay(ob, lambda m: omat(O, m))
    return case, scene, ob.build("f32")


def _expect_overflow(fn, ctx, flag):
    with pytest.raises(_lib.OmgError) as ei:
        fn()
    assert ei.value.status == _lib.E_OVERFLOW, ei.value
    assert ctx.last_flags() & flag, ctx.last_flags()


@pytest.mark.parametrize("tie", [0, 1], ids=["first-found", "near-tie"])
@pytest.mark.parametrize("limit", ["walk_budget", "loop_guard"])
def test_limit_runs_out_then_the_context_traces_correctly(oracle, tie, limit):
    O = oracle
    with Context(TraceConfig(tie_mode=tie, **CFG)) as ctx:
        case, scene, mesh = _scene_pair(ctx, O)
        # a clean run first: no flags
        ctx.trace_world(scene, case.src, case.lis, 4096, seed=5)
        assert ctx.last_flags() == 0
        if limit == "walk_budget":
            ctx.set_limits(walk_budget=3)
            flag = 4
        else:
            ctx.set_limits(loop_guard=50)
            flag = 8
        _expect_overflow(lambda: ctx.trace_world(scene, case.src, case.lis, 4096, seed=5), ctx, flag)
        # the same context, limits back to their defaults
        ctx.set_limits(0, 0)
        e, rv = ctx.trace_world(scene, case.src, case.lis, 4096, seed=5)
        assert ctx.last_flags() == 0
        P = oparams(O, ctx.cfg)
        b, _, st = O.trace_mesh(mesh, case.src, case.lis, 4096, P=P, seed=5, acc64=True)
        assert rv.segments == st["segments"]
        assert rel_bins(e.bins, b) <= 1e-5
        scene.release()


def test_limits_apply_to_a_batch_created_before_them(oracle):
    """omg_set_limits re-records the graphs of batches that already exist."""
    from omg_audio_gb300 import Job
    with Context(TraceConfig(tie_mode=1, **CFG)) as ctx:
        case, scene, _ = _scene_pair(ctx, oracle)
        batch = ctx.batch([Job(case.src, case.lis, 4096, seed=k, scene=scene) for k in range(4)])
        batch.launch()
        ref = batch.read()
        ctx.set_limits(loop_guard=50)
        batch.launch()
        _expect_overflow(batch.read, ctx, 8)
        ctx.set_limits(0, 0)
        batch.launch()
        got = batch.read()
        for (e0, r0), (e1, r1) in zip(ref, got):
            assert r0.segments == r1.segments
            assert rel_bins(e1.bins, e0.bins) <= 1e-5
        scene.release()


def test_noalloc_reports_the_loop_guard_flag(built_lib):
    """omg_trace_box_noalloc writes the kernels' flag word to the caller's device
    word: the loop guard's flag when it runs out, then 0 on the next call, whose
    echogram equals the allocating entry point's."""
    import torch
    torch.cuda.set_device(0)
    cfg = TraceConfig(**CFG)
    walls = [M.CONCRETE] * 4 + [M.WOOD_PANEL, M.CONCRETE]
    size, src, lis = (6.0, 4.0, 3.0), (1.5, 1.0, 1.5), (4.5, 3.0, 1.6)
    job = _lib.omg_box_job()
    for k in range(3):
        job.size[k], job.src[k], job.lis[k] = size[k], src[k], lis[k]
    for w in range(6):
        job.walls[w] = walls[w].to_c()
    job.n_rays = 4096
    for b in range(cfg.n_bands):
        job.energy[b] = 1.0
    job.seed = 21
    bins = torch.empty(cfg.n_bins * cfg.n_bands, dtype=torch.float32, device="cuda")
    dirs = torch.empty(cfg.n_bins * 3, dtype=torch.float32, device="cuda")
    flags = torch.full((1,), 0xFFFF, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()

    def call(prm):
        rc = built_lib.omg_trace_box_noalloc(C.byref(job), C.byref(prm), C.c_void_p(bins.data_ptr()),
                                             C.c_void_p(dirs.data_ptr()), C.c_void_p(flags.data_ptr()),
                                             C.c_void_p(stream.cuda_stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        return int(flags.item())

    cut = TraceConfig(loop_guard=50, **CFG).to_c()
    assert call(cut) & 8
    assert call(cfg.to_c()) == 0
    with Context(cfg) as ctx:
        ref, _ = ctx.trace_box(size, walls, src, lis, 4096, seed=21)
    got = bins.cpu().numpy().reshape(cfg.n_bins, cfg.n_bands)
    assert rel_bins(got, ref.bins) <= 1e-5
