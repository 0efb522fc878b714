"""Seeded synthetic scenes with the shapes of the benchmark configurations.

The reference has no datasets; these generators stand in for its scenes:
  shoebox12   - a 10 x 7 x 4 m room as 12 f32 triangles, per-surface
                absorption U[0.02, 0.4] per band, 3 bands, scattering 0.10,
                no transmission;
  multiroom   - 40 box rooms on an 8 x 5 grid (sides U[4, 20] m, heights
                U[3, 12] m) sharing walls, 1 x 2.1 m door holes, glass panes
                (transmission U[0.05, 0.3] per band) over window holes, on a
                ground plane; 64 source/listener pairs;
  room_batch  - independent furnished rooms with lognormal triangle counts,
                ray budgets, band counts and histogram lengths.
A `Recorder` captures the builder calls of a scene so the same scene can be
replayed into the library's MeshBuilder and into any other builder with the
same methods (the tests replay it into the oracle's).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

import numpy as np

from . import materials as M
from .materials import Material
from .world import Door, RoomDef, build_world_mesh, late_panels


class Recorder:
    """Records material / begin_surface / coarse / quad calls in order."""

    def __init__(self):
        self.materials: List[Material] = []
        self.quads: List[np.ndarray] = []
        self.mats: List[int] = []
        self.new_surface: List[int] = []
        self.max_edge: List[float] = []
        self._pending_surf = 0
        self._coarse = 0.0

    def material(self, m: Material) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def begin_surface(self):
        self._pending_surf += 1

    def coarse(self, e: float):
        self._coarse = float(e)

    def quad(self, a, b, c, d, m: int):
        self.quads.append(np.array([a, b, c, d], np.float32).reshape(12))
        self.mats.append(m)
        self.new_surface.append(self._pending_surf)
        self.max_edge.append(self._coarse)
        self._pending_surf = 0

    def add_quads(self, q, mats, new_surface, max_edge: float):
        """Many quads at once: q (n, 12) corner coordinates, per-quad material,
        begin_surface counts before each quad, one tessellation limit."""
        q = np.asarray(q, np.float32).reshape(-1, 12)
        self.quads.extend(list(q))
        self.mats.extend(int(m) for m in np.broadcast_to(np.asarray(mats), (len(q),)))
        ns = np.asarray(new_surface).astype(int)
        if self._pending_surf and len(ns):
            ns = ns.copy()
            ns[0] += self._pending_surf
            self._pending_surf = 0
        self.new_surface.extend(ns.tolist())
        self.max_edge.extend([float(max_edge)] * len(q))

    @property
    def n_tris(self) -> int:
        return 2 * len(self.quads)

    def replay(self, mb, material_of=lambda m: m):
        """Replay into a builder with material/quads(q, mat, new_surface, max_edge)."""
        for m in self.materials:
            mb.material(material_of(m))
        if self.quads:
            mb.quads(np.stack(self.quads), np.array(self.mats, np.uint16), np.array(self.new_surface, np.uint8),
                     np.array(self.max_edge, np.float32))
        return mb


def _uniform_material(rng, nb: int, lo=0.02, hi=0.4, scattering=0.10) -> Material:
    return Material(tuple(float(v) for v in rng.uniform(lo, hi, nb)), scattering, tuple([0.0] * nb))


def _interior_point(rng, mn, mx, margin=1.0):
    return tuple(float(rng.uniform(mn[k] + margin, mx[k] - margin)) for k in range(3))


# ------------------------------------------------------------------ config 1
@dataclass
class ShoeboxCase:
    recorder: Recorder
    size: Tuple[float, float, float]
    walls: List[Material]
    src: Tuple[float, float, float]
    lis: Tuple[float, float, float]


def shoebox12(seed: int = 1, size=(10.0, 7.0, 4.0), nb: int = 3) -> ShoeboxCase:
    """A 10 x 7 x 4 m room as 12 triangles (one surface and material per face)."""
    rng = np.random.default_rng(seed)
    walls = [_uniform_material(rng, nb) for _ in range(6)]
    rec = Recorder()
    a, b = (0.0, 0.0, 0.0), size
    ax, ay, az = a
    bx, by, bz = b
    ids = [rec.material(w) for w in walls]
    # Shoebox wall order x-, x+, y-, y+, z-, z+ (scene.rs:23-26); windings as MeshBuilder::abox
    faces = [
        ((ax, ay, az), (ax, by, az), (ax, by, bz), (ax, ay, bz)),
        ((bx, ay, az), (bx, ay, bz), (bx, by, bz), (bx, by, az)),
        ((ax, ay, az), (ax, ay, bz), (bx, ay, bz), (bx, ay, az)),
        ((ax, by, az), (bx, by, az), (bx, by, bz), (ax, by, bz)),
        ((ax, ay, az), (bx, ay, az), (bx, by, az), (ax, by, az)),
        ((ax, ay, bz), (ax, by, bz), (bx, by, bz), (bx, ay, bz)),
    ]
    for f, m in zip(faces, ids):
        rec.begin_surface()
        rec.quad(*f, m)
    src = _interior_point(rng, a, b)
    lis = _interior_point(rng, a, b)
    return ShoeboxCase(rec, tuple(size), walls, src, lis)


# ------------------------------------------------------------------ config 2
@dataclass
class MultiroomCase:
    recorder: Recorder
    rooms: List[RoomDef]
    doors: List[Door]
    glass: list                     # dome panels (panes)
    panels: list                    # late-tracer panel boxes (panes)
    pairs: List[Tuple[tuple, tuple]]
    listeners: np.ndarray
    extent: Tuple[float, float]


def pane_material(d: Door) -> Material:
    """A pane in the late field: hard glass with the door's transmission."""
    return Material((0.04, 0.03, 0.02), 0.05, tuple(d.trans))


def multiroom(seed: int = 2, nx: int = 8, ny: int = 5, n_pairs: int = 64, wall_max_edge: float = 2.3,
              max_windows: int = 48) -> MultiroomCase:
    rng = np.random.default_rng(seed)
    widths = rng.uniform(4.0, 20.0, nx)
    depths = rng.uniform(4.0, 20.0, ny)
    xs = np.concatenate([[0.0], np.cumsum(widths)]).astype(np.float32)
    ys = np.concatenate([[0.0], np.cumsum(depths)]).astype(np.float32)
    presets = [M.CONCRETE, M.BRICK, M.DRYWALL, M.WOOD_PANEL]
    rooms: List[RoomDef] = []
    idx = {}
    for i in range(nx):
        for j in range(ny):
            h = float(rng.uniform(3.0, 12.0))
            wm = presets[int(rng.integers(len(presets)))]
            floor = [M.CARPET, M.CONCRETE, M.WOOD_PANEL][int(rng.integers(3))]
            ceil = [M.ACOUSTIC_TILE, M.CONCRETE, M.DRYWALL][int(rng.integers(3))]
            idx[(i, j)] = len(rooms)
            rooms.append(RoomDef(f"r{i}_{j}", (float(xs[i]), float(ys[j])), (float(xs[i + 1]), float(ys[j + 1])), h, h,
                                 0.0, [wm, wm, wm, wm, floor, ceil], float(rng.uniform(0.12, 0.3))))
    W, D = float(xs[-1]), float(ys[-1])
    outside = len(rooms)
    rooms.append(RoomDef("Outside", (-60.0, -60.0), (W + 60.0, D + 60.0), 30.0, 30.0, 0.0, [M.GRASS] * 6, 0.15,
                         outdoor=True))
    doors: List[Door] = []

    def place(lo, hi, half):
        return float(rng.uniform(lo + half + 0.3, hi - half - 0.3))

    # interior doors (1 x 2.1 m): every x-neighbour pair, 70% of y-neighbour pairs
    for i in range(nx - 1):
        for j in range(ny):
            doors.append(Door((idx[(i, j)], idx[(i + 1, j)]), (float(xs[i + 1]), place(ys[j], ys[j + 1], 0.5)), 0,
                              0.5, 2.1, 1.05))
    for i in range(nx):
        for j in range(ny - 1):
            if rng.random() < 0.7:
                doors.append(Door((idx[(i, j)], idx[(i, j + 1)]), (place(xs[i], xs[i + 1], 0.5), float(ys[j + 1])),
                                  1, 0.5, 2.1, 1.05))
    # exterior: a few doors to the outside, windows (panes) on the facades
    boundary = [(i, j) for i in range(nx) for j in range(ny) if i in (0, nx - 1) or j in (0, ny - 1)]
    rng.shuffle(boundary)
    n_win = 0
    for k, (i, j) in enumerate(boundary):
        r = idx[(i, j)]
        if j == 0:
            plane, axis, lo, hi = float(ys[0]), 1, xs[i], xs[i + 1]
        elif j == ny - 1:
            plane, axis, lo, hi = float(ys[-1]), 1, xs[i], xs[i + 1]
        elif i == 0:
            plane, axis, lo, hi = float(xs[0]), 0, ys[j], ys[j + 1]
        else:
            plane, axis, lo, hi = float(xs[-1]), 0, ys[j], ys[j + 1]
        if k < 6:
            lat = place(lo, hi, 0.5)
            pos = (plane, lat) if axis == 0 else (lat, plane)
            doors.append(Door((r, outside), pos, axis, 0.5, 2.1, 1.05))
        if n_win < max_windows and hi - lo > 4.0:
            lat = place(lo, hi, 0.8) if k >= 6 else (float(lo) + 1.0 + 0.8 if hi - lo > 6 else place(lo, hi, 0.8))
            pos = (plane, lat) if axis == 0 else (lat, plane)
            trans = tuple(float(v) for v in rng.uniform(0.05, 0.3, 3))
            doors.append(Door((r, outside), pos, axis, 0.8, 1.2, 1.6, glass=True, trans=trans))
            n_win += 1
    rec = Recorder()
    town = (float(ys[0]) - 40.0, float(ys[-1]) + 40.0)
    # walls and slabs pack at wall_max_edge (the reference's coarse() lever)
    glass = _build(rec, rooms, doors, town, wall_max_edge)
    panels = late_panels([d for d in doors if d.glass], pane_material=pane_material)
    pairs = []
    inner = [r for r in rooms if not r.outdoor]
    for p in range(n_pairs):
        rs = inner[int(rng.integers(len(inner)))]
        rl = rs if p % 2 == 0 else inner[int(rng.integers(len(inner)))]
        src = _interior_point(rng, (rs.min[0], rs.min[1], 0.0), (rs.max[0], rs.max[1], rs.height))
        lis = _interior_point(rng, (rl.min[0], rl.min[1], 0.0), (rl.max[0], rl.max[1], rl.height))
        pairs.append((src, lis))
    listeners = np.array([p[1] for p in pairs], np.float32)
    return MultiroomCase(rec, rooms, doors, glass, panels, pairs, listeners, (W, D))


def _build(rec: Recorder, rooms, doors, town, wall_max_edge):
    """build_world_mesh with the non-ground surfaces packed at wall_max_edge."""
    class _Coarse:
        def __init__(self, inner):
            self.inner = inner
            self.ground_done = False

        def material(self, m):
            return self.inner.material(m)

        def begin_surface(self):
            self.inner.begin_surface()

        def coarse(self, e):
            # the ground bands set their own limits; everything after uses wall_max_edge
            if e == 0.0:
                self.ground_done = True
                self.inner.coarse(wall_max_edge)
            else:
                self.inner.coarse(e)

        def quad(self, *a):
            self.inner.quad(*a)

    return build_world_mesh(_Coarse(rec), rooms, doors, town=town)


# ------------------------------------------------------------------ config 3
@dataclass
class BatchRoom:
    recorder: Recorder
    size: Tuple[float, float, float]
    src: tuple
    lis: tuple
    n_rays: int
    n_bands: int
    n_bins: int
    max_time: float


def room_batch(seed: int = 3, n_rooms: int = 256, tri_median: float = 2000.0, tri_lo: int = 12,
               tri_hi: int = 20000, ray_lo: int = 512, ray_hi: int = 65536) -> List[BatchRoom]:
    """Independent furnished rooms: lognormal triangle counts (median 2k, clipped
    [12, 20k]), lognormal rays ([512, 65536]), 3 or 8 bands, 0.5-4 s at 1 ms."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_rooms):
        n_tri = int(np.clip(rng.lognormal(np.log(tri_median), 1.0), tri_lo, tri_hi))
        n_rays = int(np.clip(rng.lognormal(np.log(4096), 1.0), ray_lo, ray_hi))
        nb = 3 if rng.random() < 0.5 else 8
        tmax = float(rng.uniform(0.5, 4.0))
        size = tuple(float(v) for v in (rng.uniform(4, 20), rng.uniform(4, 20), rng.uniform(3, 12)))
        rec = Recorder()
        walls = [_uniform_material(rng, nb) for _ in range(6)]
        ids = [rec.material(w) for w in walls]
        ax = ay = az = 0.0
        bx, by, bz = size
        faces = [
            ((ax, ay, az), (ax, by, az), (ax, by, bz), (ax, ay, bz)),
            ((bx, ay, az), (bx, ay, bz), (bx, by, bz), (bx, by, az)),
            ((ax, ay, az), (ax, ay, bz), (bx, ay, bz), (bx, ay, az)),
            ((ax, by, az), (bx, by, az), (bx, by, bz), (ax, by, bz)),
            ((ax, ay, az), (bx, ay, az), (bx, by, az), (ax, by, az)),
            ((ax, ay, bz), (ax, by, bz), (bx, by, bz), (bx, ay, bz)),
        ]
        rec.coarse(1e9)  # keep the shell as 12 triangles: the count is the furniture's
        for f, m in zip(faces, ids):
            rec.begin_surface()
            rec.quad(*f, m)
        furn = rec.material(Material(tuple(float(v) for v in rng.uniform(0.05, 0.5, nb)), 0.3, tuple([0.0] * nb)))
        n_boxes = max(0, (n_tri - 12) // 12)
        for _ in range(n_boxes):
            c = np.array([rng.uniform(0.5, bx - 0.5), rng.uniform(0.5, by - 0.5), rng.uniform(0.2, bz - 0.5)])
            hs = rng.uniform(0.05, 0.4, 3)
            mn, mx = (c - hs).astype(np.float32), (c + hs).astype(np.float32)
            rec.begin_surface()
            _abox(rec, mn, mx, furn)
        src = _interior_point(rng, (0, 0, 0), size)
        lis = _interior_point(rng, (0, 0, 0), size)
        n_bins = int(round(tmax / 0.001))
        out.append(BatchRoom(rec, size, src, lis, n_rays, nb, n_bins, tmax))
    return out


def _abox(rec, mn, mx, m):
    """MeshBuilder::abox (mesh.rs:144-153) windings."""
    ax, ay, az = (float(v) for v in mn)
    bx, by, bz = (float(v) for v in mx)
    rec.quad((ax, ay, az), (ax, by, az), (ax, by, bz), (ax, ay, bz), m)
    rec.quad((bx, ay, az), (bx, ay, bz), (bx, by, bz), (bx, by, az), m)
    rec.quad((ax, ay, az), (ax, ay, bz), (bx, ay, bz), (bx, ay, az), m)
    rec.quad((ax, by, az), (bx, by, az), (bx, by, bz), (ax, by, bz), m)
    rec.quad((ax, ay, az), (bx, ay, az), (bx, by, az), (ax, by, az), m)
    rec.quad((ax, ay, bz), (ax, by, bz), (bx, by, bz), (bx, ay, bz), m)


# ------------------------------------------------------------------ config 5
@dataclass
class CityCase:
    recorder: Recorder
    sources: np.ndarray          # (16, 3)
    listeners: np.ndarray        # (16, 3), one per source
    dome_eyes: np.ndarray        # (n_eyes, 3)
    buildings: np.ndarray        # (n, 6): footprint min x, y, size x, y, height, floor height
    n_bands: int
    absorption: dict = None      # per-band absorption of the "facade", "slab" and "ground" materials
    window_frac: float = 0.4     # share of facade cells left open


def _grid_quads(p0, u, v, nu, nv):
    """nu x nv cells of the parallelogram p0 + [0,1] u + [0,1] v: (nu nv, 4, 3)
    corners (p, p + u/nu, p + u/nu + v/nv, p + v/nv)."""
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    i, j = i.reshape(-1, 1), j.reshape(-1, 1)
    du, dv = np.asarray(u) / nu, np.asarray(v) / nv
    a = np.asarray(p0) + i * du + j * dv
    return np.stack([a, a + du, a + du + dv, a + dv], axis=1)


def city(seed: int = 5, nx: int = 20, ny: int = 10, pitch: float = 60.0, cell: float = 1.5, slab_cell: float = 3.0,
         floors=(5, 28), window_frac: float = 0.4, n_bands: int = 8, n_sources: int = 16,
         n_dome: int = 1024, jitter: float = 0.01) -> CityCase:
    """Procedural city: nx x ny buildings (subdivided boxes: facades in
    `cell`-wide panels with a `window_frac` share left open as aperture holes,
    floor slabs and a roof in `slab_cell` cells) on a subdivided ground plane;
    every vertex jittered N(0, jitter) m. 20 x 10 buildings give about 1 M
    triangles. Sources, their listeners and the dome eyes stand in the streets
    at 1.5 m."""
    rng = np.random.default_rng(seed)
    rec = Recorder()
    alpha = {"facade": tuple(float(v) for v in rng.uniform(0.02, 0.1, n_bands))}
    facade = rec.material(Material(alpha["facade"], 0.2, tuple([0.0] * n_bands)))
    alpha["slab"] = tuple(float(v) for v in rng.uniform(0.01, 0.05, n_bands))
    slab = rec.material(Material(alpha["slab"], 0.1, tuple([0.0] * n_bands)))
    alpha["ground"] = tuple(float(v) for v in rng.uniform(0.02, 0.15, n_bands))
    ground = rec.material(Material(alpha["ground"], 0.3, tuple([0.0] * n_bands)))
    blocks = []
    quads, mats, surf = [], [], []

    def add(q, m):
        n = len(q)
        quads.append(q.reshape(n, 12))
        mats.append(np.full(n, m))
        s_ = np.zeros(n, int)
        s_[0] = 1
        surf.append(s_)

    for bx in range(nx):
        for by in range(ny):
            w, d = rng.uniform(15.0, 45.0, 2)
            x0 = bx * pitch + (pitch - w) / 2
            y0 = by * pitch + (pitch - d) / 2
            nf = int(rng.integers(floors[0], floors[1] + 1))
            fh = 3.5
            h = nf * fh
            blocks.append((x0, y0, w, d, h, fh))
            corners = [(x0, y0), (x0 + w, y0), (x0 + w, y0 + d), (x0, y0 + d)]
            for k in range(4):
                (ax, ay), (cx, cy) = corners[k], corners[(k + 1) % 4]
                length = float(np.hypot(cx - ax, cy - ay))
                nu = max(1, int(round(length / cell)))
                q = _grid_quads((ax, ay, 0.0), (cx - ax, cy - ay, 0.0), (0.0, 0.0, h), nu, nf)
                keep = rng.random(len(q)) >= window_frac   # open cells are aperture holes
                add(q[keep], facade)
            for f in range(1, nf + 1):
                z = f * fh
                nu, nv = max(1, int(round(w / slab_cell))), max(1, int(round(d / slab_cell)))
                add(_grid_quads((x0, y0, z), (w, 0.0, 0.0), (0.0, d, 0.0), nu, nv), slab)
    gx, gy = nx * pitch, ny * pitch
    add(_grid_quads((0.0, 0.0, 0.0), (gx, 0.0, 0.0), (0.0, gy, 0.0), int(gx / 10), int(gy / 10)), ground)
    q = np.concatenate(quads)
    q = q + rng.normal(0.0, jitter, q.shape).astype(np.float32)
    rec.add_quads(q, np.concatenate(mats), np.concatenate(surf), 4.0)

    def street_points(n):
        # on the street lines between blocks, 1.5 m up
        i = rng.integers(0, nx, n)
        j = rng.integers(0, ny, n)
        along = rng.random(n)
        xs = np.where(rng.random(n) < 0.5, i * pitch + along * pitch, i * pitch + 1.0)
        ys = np.where(xs == i * pitch + 1.0, j * pitch + along * pitch, j * pitch + 1.0)
        return np.stack([xs, ys, np.full(n, 1.5)], 1).astype(np.float32)

    src = street_points(n_sources)
    lis = street_points(n_sources)
    eyes = street_points(n_dome)
    return CityCase(rec, src, lis, eyes, np.array(blocks, np.float32), n_bands, alpha, window_frac)
