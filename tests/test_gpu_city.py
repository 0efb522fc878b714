"""The stress configuration's scene (procedural city: subdivided buildings
with floor slabs and window holes, jittered vertices) on the GPU.

- A 12-building city (about 60k triangles, 8 bands, 4 s at 1 ms): one source
  x 4096 rays against the f32-trajectory oracle (near-tie rule): identical
  segment count, compensated histogram within 1e-5 per bin (bins holding
  >= 1e-6 of the band total).
- The full 1 M-triangle city built on the device (LBVH): 4 sources x 16k
  rays trace without error into finite, non-negative echograms.
"""
import numpy as np
import pytest

from omg_audio_gb300 import Context, Job, MeshBuilder, TraceConfig, _lib
from omg_audio_gb300 import workloads as W

from test_gpu_parity import oparams, rel_bins
from test_oracle_golden import omat

pytestmark = pytest.mark.gpu


def test_small_city_matches_the_oracle(oracle):
    O = oracle
    case = W.city(seed=7, nx=4, ny=3, n_dome=16)
    cfg = TraceConfig(tie_mode=1, n_bands=8, n_bins=4000, bin_dt=0.001, max_time=4.0, max_bounces=200,
                      energy_floor=1e-6, timeout_ms=60000)
    with Context(cfg) as ctx:
        mb = MeshBuilder()
        case.recorder.replay(mb)
        scene = ctx.upload_builder(mb, 8)
        src, lis = case.sources[0], case.listeners[0]
        e, rv = ctx.trace_batch([Job(tuple(src), tuple(lis), 4096, seed=31, scene=scene)])[0]
        ob = O.MeshBuilder()
        case.recorder.replay(ob, lambda m: omat(O, m))
        m32 = ob.build("f32")
        P = oparams(O, cfg)
        b32, _, st = O.trace_mesh(m32, tuple(src), tuple(lis), 4096, energy=[1.0] * 8, P=P, seed=31, threads=8,
                                  acc64=True)
        assert rv.segments == st["segments"]
        assert rel_bins(e.bins, b32) <= 1e-5
        scene.release()


def test_full_city_on_the_device_lbvh():
    case = W.city(seed=5, n_dome=16)
    assert case.recorder.n_tris > 1_000_000
    cfg = TraceConfig(tie_mode=1, n_bands=8, n_bins=4000, bin_dt=0.001, max_time=4.0, max_bounces=200,
                      energy_floor=1e-6, timeout_ms=120000)
    with Context(cfg) as ctx:
        mb = MeshBuilder()
        case.recorder.replay(mb)
        scene = ctx.upload_builder(mb, 8, _lib.BVH_LBVH)
        assert scene.info()["prims"] > 1_000_000
        # listeners 8 m down the street from their sources
        jobs = [Job(tuple(s), tuple(s + np.array([0.0, 8.0, 0.0], np.float32)), 16384, seed=90 + k, scene=scene)
                for k, s in enumerate(case.sources[:4])]
        res = ctx.trace_batch(jobs)
        for e, rv in res:
            assert rv.segments > 16384
            assert np.all(np.isfinite(e.bins)) and np.all(e.bins >= 0)
        assert any(e.bins.sum() > 0 for e, _ in res)
        scene.release()
