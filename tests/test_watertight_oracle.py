"""The watertight checker (oracle/watertight_oracle.py) on the CPU.

A closed triangle mesh (a subdivided icosahedron of radius 3 m, vertices
shared by index) surrounds an origin, so every ray from the origin must hit
it. Rays aimed exactly at its vertices (each shared by 5 or 6 triangles) and
at the midpoints of its edges all hit under the watertight test, also with
the mesh moved 10^3 m from the coordinate origin. The same rays through the
reference's epsilon Moller-Trumbore (restated here in f32) are only counted.
"""
import numpy as np

from oracle import watertight_oracle as WT

F = np.float32


def icosphere(level, radius=3.0, center=(0.0, 0.0, 0.0)):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    v = [np.asarray(p, np.float64) / np.linalg.norm(p) for p in v]
    for _ in range(level):
        cache, nf = {}, []

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[k] = len(v) - 1
            return cache[k]
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    pos = (np.asarray(v) * radius + np.asarray(center)).astype(F)
    return pos, np.asarray(f, np.uint32)


def aimed_rays(pos, idx, origin):
    """Rays from origin toward every vertex and every edge midpoint (f32)."""
    o = np.asarray(origin, F)
    edges = {tuple(sorted((int(a), int(b)))) for tri in idx for a, b in ((tri[0], tri[1]), (tri[1], tri[2]),
                                                                           (tri[2], tri[0]))}
    targets = [pos]
    targets.append(np.asarray([((pos[a] + pos[b]) * F(0.5)).astype(F) for a, b in sorted(edges)], F))
    tg = np.concatenate(targets)
    d = (tg - o).astype(F)
    return np.repeat(o[None], len(d), 0), d


def mt_reference_hits(o, d, A, B, C):
    """The reference's Moller-Trumbore (mesh.rs:437-456) in f32: any hit per ray."""
    e1, e2 = (B - A).astype(F), (C - A).astype(F)
    out = np.zeros(len(o), bool)
    for r in range(len(o)):
        dx, dy, dz = d[r]
        p = np.stack([dy * e2[:, 2] - dz * e2[:, 1], dz * e2[:, 0] - dx * e2[:, 2], dx * e2[:, 1] - dy * e2[:, 0]],
                     1).astype(F)
        det = (e1 * p).sum(1, dtype=F)
        ok = np.abs(det) >= F(1e-9)
        inv = np.where(ok, F(1.0) / np.where(ok, det, F(1)), F(0)).astype(F)
        s = (o[r] - A).astype(F)
        u = ((s * p).sum(1, dtype=F) * inv).astype(F)
        q = np.stack([s[:, 1] * e1[:, 2] - s[:, 2] * e1[:, 1], s[:, 2] * e1[:, 0] - s[:, 0] * e1[:, 2],
                      s[:, 0] * e1[:, 1] - s[:, 1] * e1[:, 0]], 1).astype(F)
        v = ((d[r] * q).sum(1, dtype=F) * inv).astype(F)
        t = ((e2 * q).sum(1, dtype=F) * inv).astype(F)
        one = F(1.0) + F(1e-6)
        hit = ok & (u >= F(-1e-6)) & (u <= one) & (v >= F(-1e-6)) & ((u + v) <= one) & (t > F(1e-5))
        out[r] = hit.any()
    return out


def test_rays_through_shared_vertices_and_edges_never_escape():
    for center in [(0.0, 0.0, 0.0), (1000.25, -730.5, 412.75)]:
        pos, idx = icosphere(2, 3.0, center)
        A, B, C = pos[idx[:, 0]], pos[idx[:, 1]], pos[idx[:, 2]]
        for off in [(0.0, 0.0, 0.0), (0.37, -0.81, 0.23)]:
            origin = (np.asarray(center) + np.asarray(off)).astype(F)
            o, d = aimed_rays(pos, idx, origin)
            hit, _ = WT.intersect(o, d, A, B, C)
            assert hit.any(axis=1).all(), (center, off, int((~hit.any(axis=1)).sum()))
            mt = mt_reference_hits(o, d, A, B, C)
            print(f"center {center} offset {off}: {len(o)} rays, watertight misses 0, "
                  f"reference test misses {int((~mt).sum())}")


def test_shared_edge_hits_one_side_with_opposite_edge_signs():
    """Two triangles sharing an edge; a ray through the edge's midpoint hits at
    least one, and the closest hit is the lower triangle id (near-tie rule)."""
    A = np.asarray([[0, 0, 0], [0, 0, 0]], F)
    B = np.asarray([[1, 0, 0], [0, 1, 0]], F)
    C = np.asarray([[0, 1, 0], [-1, 0, 0]], F)
    o = np.asarray([[0.0, 0.5, 1.0]], F)
    d = np.asarray([[0.0, 0.0, -1.0]], F)
    hit, t = WT.intersect(o, d, A, B, C)
    assert hit.any()
    tt, tri = WT.closest(o, d, A, B, C, np.asarray([7, 3], np.uint32))
    assert tri[0] == 3 and tt[0] == F(1.0)
