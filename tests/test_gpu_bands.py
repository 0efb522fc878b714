"""Every band count from 1 to 8 against the f32 oracle (exact segment counts,
histograms within 1e-5 per bin on bins holding >= 1e-6 of the band total).

The kernels are compiled for 3 and 8 bands and run any smaller count in the
larger form, so band counts 1, 2 and 4-7 are ragged cases of those two. The
scene is two rooms joined by a transmissive wall whose strongest band is the
last one (the transmission probability is the maximum of T^2 over the job's
bands, tracer.rs:150-158), with a pane as a panel; the shoebox job uses the
same materials.
"""
import numpy as np
import pytest

from omg_audio_gb300 import Context, Job, MeshBuilder, TraceConfig, _lib
from omg_audio_gb300.materials import Material

from test_gpu_parity import oparams, rel_bins
from test_oracle_golden import omat

pytestmark = pytest.mark.gpu

CFG = dict(n_bins=1500, bin_dt=0.001, max_time=1.5, max_bounces=120, energy_floor=1e-6, tie_mode=1)


def _materials(nb, seed):
    rng = np.random.default_rng(seed)
    wall = Material(tuple(float(v) for v in rng.uniform(0.02, 0.3, nb)), 0.15, tuple([0.0] * nb))
    t = [float(v) for v in rng.uniform(0.05, 0.2, nb)]
    t[-1] = 0.45                                  # the strongest band is the last one
    party = Material(tuple(float(v) for v in rng.uniform(0.05, 0.2, nb)), 0.3, tuple(t))
    pane = Material(tuple(float(v) for v in rng.uniform(0.02, 0.1, nb)), 0.0,
                    tuple(float(v) for v in rng.uniform(0.1, 0.4, nb)))
    return wall, party, pane


def _build(b, wall, party):
    """Two 5 x 4 x 3 m rooms side by side; the shared wall at x = 5 is its own surface."""
    f = np.float32
    w = b.material(wall)
    p = b.material(party)
    b.begin_surface()
    b.quad(f([0, 0, 0]), f([10, 0, 0]), f([10, 4, 0]), f([0, 4, 0]), w)      # floor
    b.begin_surface()
    b.quad(f([0, 0, 3]), f([0, 4, 3]), f([10, 4, 3]), f([10, 0, 3]), w)      # ceiling
    b.begin_surface()
    b.quad(f([0, 0, 0]), f([0, 0, 3]), f([10, 0, 3]), f([10, 0, 0]), w)      # y = 0
    b.begin_surface()
    b.quad(f([0, 4, 0]), f([10, 4, 0]), f([10, 4, 3]), f([0, 4, 3]), w)      # y = 4
    b.begin_surface()
    b.quad(f([0, 0, 0]), f([0, 4, 0]), f([0, 4, 3]), f([0, 0, 3]), w)        # x = 0
    b.begin_surface()
    b.quad(f([10, 0, 0]), f([10, 0, 3]), f([10, 4, 3]), f([10, 4, 0]), w)    # x = 10
    b.begin_surface()
    b.quad(f([5, 0, 0]), f([5, 4, 0]), f([5, 4, 3]), f([5, 0, 3]), p)        # the party wall


@pytest.mark.parametrize("nb", [1, 2, 4, 5, 7])
def test_band_counts_match_the_oracle(oracle, nb):
    O = oracle
    wall, party, pane = _materials(nb, seed=40 + nb)
    src, lis = (1.5, 1.2, 1.4), (7.8, 2.9, 1.6)
    panels = [((2.0, 3.0, 0.5), (3.0, 3.2, 2.5), pane)]
    with Context(TraceConfig(n_bands=nb, dir_band=min(1, nb - 1), **CFG)) as ctx:
        mb = MeshBuilder()
        _build(mb, wall, party)
        scene = ctx.upload_builder(mb, nb, _lib.BVH_SAH3)
        jobs = [Job(src, lis, 4096, seed=70 + nb, scene=scene, panel_offset=0, n_panels=1),
                Job(src, (3.9, 2.5, 1.1), 4096, seed=80 + nb, box_size=(5.0, 4.0, 3.0),
                    box_walls=[wall] * 5 + [party])]
        res = ctx.trace_batch(jobs, panels)
        scene.release()
    assert res[0][0].bins.shape == (CFG["n_bins"], nb)
    P = oparams(O, ctx.cfg)
    ob = O.MeshBuilder()
    _build(ob, omat(O, wall), omat(O, party))
    pan = [((2.0, 3.0, 0.5), (3.0, 3.2, 2.5), omat(O, pane))]
    bm, _, sm = O.trace_mesh(ob.build("f32"), src, lis, 4096, energy=[1.0] * nb, P=P, seed=70 + nb, panels=pan,
                             acc64=True)
    bb, _, sb = O.trace_box((5.0, 4.0, 3.0), [omat(O, wall)] * 5 + [omat(O, party)], src, (3.9, 2.5, 1.1), 4096,
                            energy=[1.0] * nb, P=P, seed=80 + nb, acc64=True)
    (em, rm), (eb, rb) = res
    assert rm.segments == sm["segments"] and rb.segments == sb["segments"]
    assert rel_bins(em.bins, bm) <= 1e-5 and rel_bins(eb.bins, bb) <= 1e-5
    assert em.bins[:, -1].sum() > 0           # the listener behind the wall hears the last band
