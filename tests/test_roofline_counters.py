"""The traversal counters behind the roofline's bytes per segment (CPU only).

bench.py's B_seg = 32 N_node + 48 N_prim + 4 (NB + 3) h comes from the f32
oracle's counters of the reference's ordered walk (mesh.rs:484-541). These
tests pin what the counters mean:
  - on meshes small enough to count by hand: a one-leaf mesh, and two leaves
    along a ray whose far leaf is culled by the first hit (the root record, both
    child records, the near leaf's 4 primitives);
  - on a trace of the 40-room scene: every segment is one closest-hit query,
    every processed internal node reads both child boxes, the distinct records
    are the root plus the child boxes, and bench.bytes_per_segment follows the
    formula it prints.
"""
import numpy as np

import bench
from oracle import oracle as O

MAT = dict(absorption=(0.1, 0.1, 0.1), scattering=0.1, transmission=(0.0, 0.0, 0.0))


def _mesh(tris):
    mb = O.MeshBuilder()
    m = mb.material(O.Material.make(**MAT))
    mb.begin_surface()
    for a, b, c in tris:
        mb.tri(a, b, c, m)
    return mb.build("f32")


def _wall(x, y0, z0):
    """Two triangles of a 0.5 m square in the plane x, corner (y0, z0)."""
    a, b, c, d = (x, y0, z0), (x, y0 + 0.5, z0), (x, y0 + 0.5, z0 + 0.5), (x, y0, z0 + 0.5)
    return [(a, b, c), (a, c, d)]


def test_one_leaf():
    mesh = _mesh(_wall(0.0, -0.25, -0.25))
    assert mesh.info()["nodes"] == 1
    t, tri, st = mesh.raycast([[-1.0, 0.1, 0.05]], [[1.0, 0.0, 0.0]])
    assert t[0] == 1.0
    assert st == dict(node_reads=1, prim_tests=2, queries=1, internal_visits=0, leaf_visits=1, child_boxes=0,
                      unique_nodes=1)


def test_two_leaves_far_one_culled():
    near = _wall(0.0, -0.25, -0.25) + _wall(0.2, -0.25, -0.25)
    far = _wall(10.0, -0.25, -0.25) + _wall(10.2, -0.25, -0.25)
    mesh = _mesh(near + far)
    assert mesh.info()["nodes"] == 3   # the root and two leaves of 4
    t, tri, st = mesh.raycast([[-1.0, 0.1, 0.05]], [[1.0, 0.0, 0.0]])
    assert t[0] == 1.0
    # the root, both child records, the near leaf; the far leaf's entry (t = 11)
    # is beyond the first hit and is never read again
    assert st == dict(node_reads=4, prim_tests=4, queries=1, internal_visits=1, leaf_visits=1, child_boxes=2,
                      unique_nodes=3)
    b_query = 32 * st["unique_nodes"] + 48 * st["prim_tests"]
    assert b_query == 288


def test_trace_counters_follow_the_counting_rule():
    case = bench.build_case()
    mesh = bench.oracle_mesh(case)
    P = O.params(tie_mode=0, **bench.CFG)
    pan = [(mn, mx, O.Material.make(m.absorption, m.scattering, m.transmission)) for (mn, mx, m) in case.panels]
    src, lis = case.pairs[0]
    _, _, st = O.trace_mesh(mesh, src, lis, 4096, P=P, seed=1000, panels=pan, ray_end=256)
    assert st["segments"] > 1000
    assert st["queries"] == st["segments"]
    assert st["child_boxes"] == 2 * st["internal_visits"]
    assert st["unique_nodes"] == st["queries"] + st["child_boxes"]
    assert st["node_reads"] == st["internal_visits"] + st["leaf_visits"] + st["child_boxes"]
    b_seg, parts = bench.bytes_per_segment(st, nb=3)
    s = st["segments"]
    want = (32.0 * st["unique_nodes"] + 48.0 * st["prim_tests"] + 4.0 * 6 * st["receiver_hits"]) / s
    assert np.isclose(b_seg, want, rtol=1e-12)
    assert np.isclose(parts["n_node"], st["unique_nodes"] / s)
    # the 40-room scene's figure (2018 B over the 64 pairs), within the spread of a 256-ray sample
    assert 1700.0 < b_seg < 2400.0, b_seg
