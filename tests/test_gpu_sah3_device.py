"""The three-axis binned-SAH tree built on the GPU (OMG_BVH_SAH3, sah3.cu)
against the same tree built on the host (OMG_BVH_SAH3_HOST, scene.cpp).

Every split of the builder depends only on the set of primitives in a node and
on f32 operations the device repeats exactly, so the two trees must be equal:
  - node arrays (build_sah3's form and numbering): child links and leaf
    ranges identical, boxes equal as floats;
  - each leaf holds the same primitives (the order inside a leaf may differ);
  - traces over the two trees under the near-tie rule: identical segment
    counts and bit-identical echograms.
Scenes: the 12-triangle shoebox (one block builds the whole tree), the
40-room scene (large-node levels, then blocks), the 1 M-triangle city (1.94 M
primitives, 13 large-node levels), a random triangle soup, and
a degenerate scene whose 6000 triangles share (or nearly share, within 4e-7)
one centre, so that nodes of more than 2048 and of fewer primitives fall back
to object-median splits (host: nth_element by centre and index).
"""
import numpy as np
import pytest

from omg_audio_gb300 import Context, Job, MeshBuilder, TraceConfig
from omg_audio_gb300 import _lib
from omg_audio_gb300 import materials as M
from omg_audio_gb300 import workloads as W

pytestmark = pytest.mark.gpu

LEAF = np.uint32(0x80000000)
CFG = dict(n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200, energy_floor=1e-6, tie_mode=1)


def _soup(n, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 30.0, (n, 1, 3))
    d = rng.normal(size=(n, 3, 3)) * rng.uniform(0.05, 3.0, (n, 1, 1))
    return (c + d).reshape(-1, 3).astype(np.float32)


def _coincident(n_same, n_jit, n_other, seed):
    rng = np.random.default_rng(seed)
    base = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.0, 0.5, 0.25]], np.float32)
    same = np.tile(base, (n_same, 1, 1))
    jit = np.tile(base, (n_jit, 1, 1)) + rng.uniform(-2e-7, 2e-7, (n_jit, 1, 3)).astype(np.float32)
    other = rng.uniform(-5.0, 5.0, (n_other, 1, 3)) + rng.normal(size=(n_other, 3, 3)) * 0.3
    return np.concatenate([same, jit, other]).reshape(-1, 3).astype(np.float32)


def _upload(ctx, scene, kind):
    if scene[0] == "recorder":
        mb = MeshBuilder()
        scene[1].replay(mb)
        return ctx.upload_builder(mb, 3, kind)
    pos = scene[1]
    idx = np.arange(len(pos), dtype=np.uint32).reshape(-1, 3)
    tm = np.zeros(len(idx), np.uint16)
    return ctx.upload_mesh(pos, idx, tm, [M.CONCRETE], n_bands=3, bvh=kind)


def _rows_by_leaf(ex):
    """Primitive rows (geometry bits, triangle, material) sorted inside each leaf."""
    ab = ex["node_ab"]
    leaf = (ab[:, 0] & LEAF) != 0
    start = (ab[leaf, 0] & ~LEAF).astype(np.int64)
    cnt = ab[leaf, 1].astype(np.int64)
    n = len(ex["prim_tri"])
    owner = np.full(n, -1, np.int64)
    for k, (s, c) in enumerate(zip(start, cnt)):
        owner[s:s + c] = k
    assert (owner >= 0).all()
    rows = np.concatenate([owner[:, None].astype(np.uint64),
                           ex["prim_geo"].view(np.uint32).astype(np.uint64),
                           ex["prim_tri"][:, None].astype(np.uint64),
                           ex["prim_mat"][:, None].astype(np.uint64)], axis=1)
    order = np.lexsort(rows.T[::-1])
    return rows[order]


SCENES = {
    "shoebox12": lambda: ("recorder", W.shoebox12(seed=1).recorder),
    "multiroom": lambda: ("recorder", W.multiroom().recorder),
    "city": lambda: ("recorder", W.city(seed=5).recorder),
    "soup": lambda: ("mesh", _soup(20000, 1)),
    "coincident": lambda: ("mesh", _coincident(3000, 3000, 500, 2)),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_device_tree_equals_host_tree(built_lib, name):
    scene = SCENES[name]()
    with Context(TraceConfig(**CFG)) as ctx:
        dev = _upload(ctx, scene, _lib.BVH_SAH3)
        host = _upload(ctx, scene, _lib.BVH_SAH3_HOST)
        ed, eh = dev.export_bvh(), host.export_bvh()
        assert ed["node_ab"].shape == eh["node_ab"].shape
        assert np.array_equal(ed["node_ab"], eh["node_ab"])
        assert np.array_equal(ed["node_boxes"], eh["node_boxes"])
        assert np.array_equal(_rows_by_leaf(ed), _rows_by_leaf(eh))
        dev.release()
        host.release()


def test_median_splits_are_exercised(built_lib):
    """The degenerate scene has nodes above and below 2048 primitives whose
    centres span at most 1e-6 on every axis (the object-median fallback)."""
    pos = _coincident(3000, 3000, 500, 2)
    with Context(TraceConfig(**CFG)) as ctx:
        sc = _upload(ctx, ("mesh", pos), _lib.BVH_SAH3)
        ex = sc.export_bvh()
        sc.release()
    ab, geo = ex["node_ab"], ex["prim_geo"].reshape(-1, 3, 3)
    v = np.stack([geo[:, 0], geo[:, 0] + geo[:, 1], geo[:, 0] + geo[:, 2]], axis=1)
    cen = (v.min(axis=1) + v.max(axis=1)) * 0.5
    sizes, degenerate = {}, []

    def walk(i):
        if ab[i, 0] & LEAF:
            s, c = int(ab[i, 0] & ~LEAF), int(ab[i, 1])
            sizes[i] = (s, s + c)
        else:
            walk(int(ab[i, 0]))
            walk(int(ab[i, 1]))
            sizes[i] = (sizes[int(ab[i, 0])][0], sizes[int(ab[i, 1])][1])
        s, e = sizes[i]
        if e - s > 4 and (np.ptp(cen[s:e], axis=0) <= 1e-6).all():
            degenerate.append(e - s)

    walk(0)
    assert max(degenerate) > 2048 and min(degenerate) <= 2048, degenerate[:8]


@pytest.mark.parametrize("name", ["multiroom", "soup"])
def test_traces_over_both_trees_are_identical(built_lib, name):
    scene = SCENES[name]()
    with Context(TraceConfig(**CFG)) as ctx:
        dev = _upload(ctx, scene, _lib.BVH_SAH3)
        host = _upload(ctx, scene, _lib.BVH_SAH3_HOST)
        if name == "multiroom":
            pairs = W.multiroom().pairs[:8]
        else:
            pairs = [((15.0, 15.0, 15.0), (10.0, 12.0, 14.0)), ((5.0, 25.0, 10.0), (20.0, 5.0, 20.0))]
        out = []
        for sc in (dev, host):
            res = ctx.trace_batch([Job(s, l, 4096, seed=7 + k, scene=sc) for k, (s, l) in enumerate(pairs)])
            out.append(res)
        for (e0, r0), (e1, r1) in zip(*out):
            assert r0.segments == r1.segments
            assert np.array_equal(e0.bins, e1.bins)
        dev.release()
        host.release()
