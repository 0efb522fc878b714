"""The reference's walkthrough world (tests/golden/walkthrough_world.json,
extracted from crates/omg-scene/src/walkthrough.rs) for the dome tests."""
import json
import os

from omg_audio_gb300 import materials as M
from omg_audio_gb300.world import Door, RoomDef

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with open(os.path.join(HERE, "golden", "walkthrough_world.json")) as fh:
        d = json.load(fh)
    return d["rooms"], d["doors"]


def product_world():
    rooms, doors = load()
    R = [RoomDef(r["name"], tuple(r["min"]), tuple(r["max"]), r["height"], r["barrier_height"], r["floor_z"],
                 [M.PRESETS[w] for w in r["walls"]], r["wall_thickness"], r["outdoor"]) for r in rooms]
    D = [Door(tuple(d["rooms"]), tuple(d["pos"]), d["axis"], d["half"], d["height"], d["zc"], d["glass"],
              d["openness"], d["heavy"]) for d in doors]
    return R, D


def oracle_world(O, doors_override=None):
    """rooms/doors dicts with oracle materials and pane transmissions."""
    rooms, doors = load()
    if doors_override is not None:
        doors = doors_override
    mats = {k: O.Material.make(v.absorption, v.scattering, v.transmission) for k, v in M.PRESETS.items()}
    orooms = [dict(r, walls=[mats[w] for w in r["walls"]]) for r in rooms]
    odoors = [dict(d, pane_trans=M.glass_transmission(d["heavy"])) for d in doors]
    return orooms, odoors


def leaf_panels(doors):
    """dome.rs:269-291 door_panels, as dicts (leaf seep = door/heavy constants)."""
    import numpy as np
    f32 = np.float32
    out = []
    for d in doors:
        if d["glass"] or not (d["openness"] < 0.999):
            continue
        lat_c, plane = (d["pos"][1], d["pos"][0]) if d["axis"] == 0 else (d["pos"][0], d["pos"][1])
        covered = f32(f32(f32(1.0) - f32(d["openness"])) * f32(2.0)) * f32(d["half"])
        lo = f32(f32(lat_c) - f32(d["half"]))
        z0 = f32(f32(d["zc"]) - f32(0.5) * f32(d["height"]))
        z1 = f32(f32(d["zc"]) + f32(0.5) * f32(d["height"]))
        t = M.HEAVY_PANEL_TRANSMISSION if d["heavy"] else M.DOOR_PANEL_TRANSMISSION
        out.append(dict(axis=d["axis"], plane=float(plane), lat=(float(lo), float(lo + covered)),
                        z=(float(z0), float(z1)), glass=False, trans=t))
    return out


def furniture_world(materials_of):
    """The reference's solve_parity.rs world (solve_parity.rs:24-61): every
    furniture box in world coordinates as an extras blocker, the pieces above
    FURN_REFLECTOR_MIN_VOL as reflector boxes with their materials, and two
    shut wood leaves. materials_of(dict) -> the caller's material object.
    Returns (furniture [(min, max, material)], extras [(min, max, transmission)])."""
    import numpy as np
    f32 = np.float32
    with open(os.path.join(HERE, "golden", "walkthrough_world.json")) as fh:
        d = json.load(fh)
    rooms = d["rooms"]
    furn, extras = [], []
    for ri, r in enumerate(rooms):
        o = (f32(r["min"][0]), f32(r["min"][1]), f32(r["floor_z"]))
        for b in d["furniture"].get(str(ri), []):
            mn = tuple(float(f32(b["min"][k]) + o[k]) for k in range(3))
            mx = tuple(float(f32(b["max"][k]) + o[k]) for k in range(3))
            extras.append((mn, mx, tuple(b["transmission"])))
            dd = [f32(f32(b["max"][k]) - f32(b["min"][k])) for k in range(3)]
            if f32(f32(dd[0] * dd[1]) * dd[2]) > f32(d["furn_reflector_min_vol"]):
                furn.append((mn, mx, materials_of(b["material"])))
    leaf = M.WOOD_PANEL.transmission
    extras.append(((6.9, 24.9, 0.0), (7.5, 25.1, 2.1), leaf))
    extras.append(((3.9, 7.9, 0.0), (4.9, 8.1, 2.1), leaf))
    return furn, extras
