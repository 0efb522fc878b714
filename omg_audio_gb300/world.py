"""World construction for the mesh tracer and the dome
(crates/omg-scene/src/dome.rs:79-291, world.rs:108-140).

Rooms are axis-aligned boxes on the ground; walls are authored per room with
true holes for their apertures, ceilings with holes for vertical portals, and
one ground surface (far field packed coarse). Glass panes come back as dome
panels; door leaves are panels whose coverage follows their openness. All
coordinates are computed in f32 as in the reference.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

import numpy as np

from .materials import (DOOR_PANEL_TRANSMISSION, HEAVY_PANEL_TRANSMISSION, CONCRETE, WOOD_PANEL, Material,
                        glass_transmission)

f32 = np.float32


@dataclass
class RoomDef:
    """walkthrough.rs:29-42."""
    name: str
    min: Tuple[float, float]
    max: Tuple[float, float]
    height: float
    barrier_height: float
    floor_z: float
    walls: Sequence[Material]
    wall_thickness: float
    outdoor: bool = False


@dataclass
class Door:
    """walkthrough.rs:228-249; `trans` overrides the pane transmission."""
    rooms: Tuple[int, int]
    pos: Tuple[float, float]
    axis: int
    half: float
    height: float
    zc: float
    glass: bool = False
    openness: float = 1.0
    heavy: bool = False
    trans: Tuple[float, ...] = ()

    def pane_transmission(self):
        return tuple(self.trans) if self.trans else glass_transmission(self.heavy)


@dataclass
class DomePanel:
    """dome.rs:41-69 with its per-band amplitude transmission."""
    axis: int
    plane: float
    lat: Tuple[float, float]
    z: Tuple[float, float]
    glass: bool
    trans: Tuple[float, ...]

    def as_dict(self):
        return dict(axis=self.axis, plane=self.plane, lat=self.lat, z=self.z, glass=self.glass, trans=self.trans)


def subrects(r, holes):
    """dome.rs:79-119: rectangle (u0,u1,v0,v1) minus holes, as sub-rectangles."""
    r = tuple(f32(v) for v in r)
    cuts = [r[0], r[1]]
    for h in holes:
        cuts.append(min(max(f32(h[0]), r[0]), r[1]))
        cuts.append(min(max(f32(h[1]), r[0]), r[1]))
    cuts.sort()
    ded = []
    for c in cuts:  # Vec::dedup_by keeps the first of each run
        if ded and abs(f32(c - ded[-1])) < f32(1e-4):
            continue
        ded.append(c)
    out = []
    for u0, u1 in zip(ded[:-1], ded[1:]):
        if f32(u1 - u0) < f32(1e-3):
            continue
        um = f32(f32(0.5) * f32(u0 + u1))
        vh = []
        for h in holes:
            if f32(h[0]) <= um <= f32(h[1]):
                a, b = max(f32(h[2]), r[2]), min(f32(h[3]), r[3])
                if b > a:
                    vh.append((a, b))
        vh.sort(key=lambda x: x[0])
        v = r[2]
        for h0, h1 in vh:
            if f32(h0 - v) > f32(1e-3):
                out.append((u0, u1, v, h0))
            v = max(v, h1)
        if f32(r[3] - v) > f32(1e-3):
            out.append((u0, u1, v, r[3]))
    return out


def _thick_material(m: Material, thickness: float) -> Material:
    return m.with_transmission(m.transmission_at(thickness))


def build_world_mesh(mb, rooms: Sequence[RoomDef], doors: Sequence[Door], town=(-40.0, 120.0)):
    """dome.rs:121-258 into a MeshBuilder (the library's, engine.MeshBuilder).
    Returns the glass panes as dome panels."""
    glass: List[DomePanel] = []
    outdoor = next(r for r in rooms if r.outdoor)
    ground = mb.material(outdoor.walls[4])
    mb.begin_surface()
    shafts = [(f32(d.pos[0]) - f32(1.5), f32(d.pos[0]) + f32(0.8), f32(d.pos[1]) - f32(d.half),
               f32(d.pos[1]) + f32(d.half)) for d in doors if d.zc < 0.0]
    t0, t1 = f32(town[0]), f32(town[1])
    for (u0, u1, v0, v1) in subrects((outdoor.min[0], outdoor.max[0], outdoor.min[1], outdoor.max[1]), shafts):
        bands = []
        n0, n1 = max(v0, t0), min(v1, t1)
        if v0 < t0:
            bands.append((v0, min(v1, t0), 64.0))
        if n1 > n0:
            bands.append((n0, n1, 0.0))
        if v1 > t1:
            bands.append((max(v0, t1), v1, 64.0))
        for (y0, y1, coarse) in bands:
            mb.coarse(coarse)
            mb.quad((u0, y0, 0.0), (u1, y0, 0.0), (u1, y1, 0.0), (u0, y1, 0.0), ground)
        mb.coarse(0.0)
    for ri, r in enumerate(rooms):
        if r.outdoor:
            continue
        z0, z1 = f32(r.floor_z), f32(f32(r.floor_z) + f32(r.height))
        above = None
        for n in rooms:
            if (not n.outdoor and f32(n.floor_z) >= f32(z1 - f32(0.05)) and f32(n.floor_z) <= f32(z1 + f32(0.8))
                    and abs(f32(n.min[0]) - f32(r.min[0])) < 2.0 and abs(f32(n.min[1]) - f32(r.min[1])) < 2.0):
                above = n
                break
        wall_top = f32(above.floor_z) if above is not None else max(f32(r.barrier_height), z1)
        sides = [(0, r.min[0], r.min[1], r.max[1], 0), (1, r.max[0], r.min[1], r.max[1], 0),
                 (2, r.min[1], r.min[0], r.max[0], 1), (3, r.max[1], r.min[0], r.max[0], 1)]
        for (wi, plane, lo, hi, axis) in sides:
            mat = mb.material(_thick_material(r.walls[wi], r.wall_thickness))
            mb.begin_surface()
            holes = []
            for d in doors:
                if d.axis != axis or (d.rooms[0] != ri and d.rooms[1] != ri):
                    continue
                dp = f32(d.pos[0] if axis == 0 else d.pos[1])
                dl = f32(d.pos[1] if axis == 0 else d.pos[0])
                if abs(f32(dp - f32(plane))) > f32(0.1):
                    continue
                hz0 = f32(f32(d.zc) - f32(f32(0.5) * f32(d.height)))
                hz1 = f32(f32(d.zc) + f32(f32(0.5) * f32(d.height)))
                holes.append((dl - f32(d.half), dl + f32(d.half), hz0, hz1))
                if d.glass:
                    glass.append(DomePanel(axis, float(plane), (float(dl - f32(d.half)), float(dl + f32(d.half))),
                                           (float(hz0), float(hz1)), True, d.pane_transmission()))
            for (u0, u1, v0, v1) in subrects((lo, hi, z0, wall_top), holes):
                if axis == 0:
                    p = lambda u, v: (plane, u, v)
                else:
                    p = lambda u, v: (u, plane, v)
                mb.quad(p(u0, v0), p(u1, v0), p(u1, v1), p(u0, v1), mat)
        mat = mb.material(_thick_material(r.walls[5], r.wall_thickness))
        mb.begin_surface()
        holes = []
        for d in doors:
            vertical = abs(f32(f32(d.zc) - z1)) < f32(0.6)
            if vertical and (d.rooms[0] == ri or d.rooms[1] == ri) and not d.glass:
                holes.append((f32(d.pos[0]) - f32(d.half), f32(d.pos[0]) + f32(d.half),
                              f32(d.pos[1]) - f32(d.half), f32(d.pos[1]) + f32(d.half)))
        for (u0, u1, v0, v1) in subrects((r.min[0], r.max[0], r.min[1], r.max[1]), holes):
            mb.quad((u0, v0, z1), (u1, v0, z1), (u1, v1, z1), (u0, v1, z1), mat)
    return glass


def door_panels(doors: Sequence[Door]) -> List[DomePanel]:
    """dome.rs:269-291: leaves covering (1 - openness) of their aperture."""
    out = []
    for d in doors:
        if d.glass or not (d.openness < 0.999):
            continue
        lat_c, plane = (d.pos[1], d.pos[0]) if d.axis == 0 else (d.pos[0], d.pos[1])
        covered = f32(f32(f32(1.0) - f32(d.openness)) * f32(2.0)) * f32(d.half)
        lo = f32(f32(lat_c) - f32(d.half))
        hz0 = f32(f32(d.zc) - f32(f32(0.5) * f32(d.height)))
        hz1 = f32(f32(d.zc) + f32(f32(0.5) * f32(d.height)))
        t = HEAVY_PANEL_TRANSMISSION if d.heavy else DOOR_PANEL_TRANSMISSION
        out.append(DomePanel(d.axis, float(plane), (float(lo), float(f32(lo + covered))), (float(hz0), float(hz1)),
                             False, t))
    return out


def late_panels(doors: Sequence[Door], pane_material=None):
    """world.rs:108-140, 384-392: aperture boxes for the late tracer (panes and
    closed leaves, 4 cm either side of the wall plane)."""
    out = []
    for d in doors:
        lat_c, plane = (d.pos[1], d.pos[0]) if d.axis == 0 else (d.pos[0], d.pos[1])
        if d.glass:
            lat0, lat1 = f32(lat_c) - f32(d.half), f32(lat_c) + f32(d.half)
            m = pane_material(d) if pane_material else CONCRETE
        else:
            if d.openness >= 0.999:
                continue
            covered = f32(f32(f32(1.0) - f32(d.openness)) * f32(2.0)) * f32(d.half)
            lat0 = f32(lat_c) - f32(d.half)
            lat1 = lat0 + covered
            m = WOOD_PANEL
        z0 = f32(d.zc) - f32(0.5) * f32(d.height)
        z1 = f32(d.zc) + f32(0.5) * f32(d.height)
        if d.axis == 0:
            mn, mx = (plane - 0.04, float(lat0), float(z0)), (plane + 0.04, float(lat1), float(z1))
        else:
            mn, mx = (float(lat0), plane - 0.04, float(z0)), (float(lat1), plane + 0.04, float(z1))
        out.append((mn, mx, m))
    return out
