"""Extract the reference's walkthrough world (rooms, doors, furniture) as JSON data.

Reads crates/omg-scene/src/walkthrough.rs of the reference checkout (text
only, nothing is executed) and writes tests/golden/walkthrough_world.json:
the room table of `rooms()` (walkthrough.rs:44-226), the door table of
`doors()` (walkthrough.rs:275-307), with wall materials by preset name, and
the furniture of `furniture(room)` / `furniture_mats(room)` with
FURN_REFLECTOR_MIN_VOL (walkthrough.rs:535-672). The dome tests of
dome.rs:496-654 and the world early-reflection tests (the reference's
solve_parity.rs world) run on this world.

    python tests/golden/make_walkthrough_fixture.py /path/to/reference
"""
import json
import os
import re
import sys


def parse(src: str):
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"pub const (\w+): usize = (\d+);", src)}
    body = src[src.index("pub fn rooms()"):src.index("pub const LIVING")]
    rooms = []
    for blk in re.findall(r"RoomDef \{(.*?)\n        \}", body, re.S):
        def f(key):
            return re.search(rf"\b{key}: ([^,\n]+),", blk).group(1).strip()

        def pair(key):
            a, b = re.search(rf"\b{key}: \(([-\d.]+), ([-\d.]+)\)", blk).groups()
            return [float(a), float(b)]

        w = re.search(r"walls: \[(.*?)\],", blk, re.S).group(1)
        rep = re.match(r"\s*(?:Material::)?(\w+); 6\s*$", w)
        walls = [rep.group(1)] * 6 if rep else [x.strip().replace("Material::", "") for x in w.split(",") if x.strip()]
        rooms.append(dict(name=re.search(r'name: "([^"]+)"', blk).group(1), min=pair("min"), max=pair("max"),
                          height=float(f("height")), barrier_height=float(f("barrier_height")),
                          floor_z=float(f("floor_z")), walls=walls, wall_thickness=float(f("wall_thickness")),
                          outdoor=f("outdoor") == "true"))
    dbody = src[src.index("pub fn doors()"):src.index("pub const DOOR_HALF_WIDTH")]
    doors = []
    for blk in re.findall(r"Door \{ (rooms:.*?) \}", dbody):
        a, b = re.search(r"rooms: \((\w+), (\w+)\)", blk).groups()
        px, py = re.search(r"pos: \(([-\d.]+), ([-\d.]+)\)", blk).groups()
        g = lambda k: re.search(rf"\b{k}: ([\w.\-]+)", blk).group(1)
        doors.append(dict(rooms=[consts[a], consts[b]], pos=[float(px), float(py)], axis=int(g("axis")),
                          half=float(g("half")), height=float(g("height")), zc=float(g("zc")),
                          glass=g("glass") == "true", openness=float(g("openness")), heavy=g("heavy") == "true"))
    return rooms, doors


def parse_furniture(src: str):
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"pub const (\w+): usize = (\d+);", src)}
    fb = src[src.index("pub fn furniture(room: usize)"):src.index("pub const FURN_REFLECTOR_MIN_VOL")]
    num = r"(-?[\d.]+)"
    tconst = {m.group(1): [float(v) for v in m.group(2).split(",")]
              for m in re.finditer(r"const (\w+): \[f32; 3\] = \[([^\]]+)\];", fb)}
    tables = {}
    for m in re.finditer(r"static (\w+): \[omg_core::pt::Aabb; \d+\] = \[(.*?)\];", fb, re.S):
        boxes = []
        for b in re.finditer(r"boxy\(" + r",\s*".join([num] * 6) + r",\s*(\w+)\)", m.group(2)):
            v = [float(b.group(i)) for i in range(1, 7)]
            boxes.append(dict(min=v[:3], max=v[3:], transmission=tconst[b.group(7)]))
        tables[m.group(1)] = boxes
    rooms_f = {consts[a]: tables[b] for a, b in re.findall(r"(\w+) => &(\w+_F),", fb)}
    mb = src[src.index("pub fn furniture_mats(room: usize)"):]
    mb = mb[:mb.index("\n}\n") + 3]
    mconst = {}
    for m in re.finditer(r"const (\w+): Material = Material \{\s*absorption: \[([^\]]+)\],\s*scattering: ([\d.]+),"
                         r"\s*transmission: \[([^\]]+)\],\s*\};", mb):
        mconst[m.group(1)] = dict(absorption=[float(v) for v in m.group(2).split(",")], scattering=float(m.group(3)),
                                  transmission=[float(v) for v in m.group(4).split(",")])
    mtables = {}
    for m in re.finditer(r"static (\w+): \[Material; (\d+)\] =\s*\[(.*?)\];", mb, re.S):
        body = re.sub(r"//[^\n]*", "", m.group(3))
        rep = re.match(r"\s*(\w+); (\d+)\s*$", body)
        names = [rep.group(1)] * int(rep.group(2)) if rep else [x.strip() for x in body.split(",") if x.strip()]
        assert len(names) == int(m.group(2)), m.group(1)
        mtables[m.group(1)] = [mconst[n] for n in names]
    rooms_m = {consts[a]: mtables[b] for a, b in re.findall(r"(\w+) => &(\w+_M),", mb)}
    out = {}
    for r, boxes in rooms_f.items():
        mats = rooms_m[r]
        assert len(mats) == len(boxes), r
        out[str(r)] = [dict(b, material=m) for b, m in zip(boxes, mats)]
    vol = float(re.search(r"pub const FURN_REFLECTOR_MIN_VOL: f32 = ([\d.]+);", src).group(1))
    return out, vol


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_walkthrough_fixture.py <path of the reference checkout>")
    ref = sys.argv[1]
    src = open(os.path.join(ref, "crates/omg-scene/src/walkthrough.rs")).read()
    rooms, doors = parse(src)
    furniture, min_vol = parse_furniture(src)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "walkthrough_world.json")
    with open(out, "w") as fh:
        json.dump({"source": "crates/omg-scene/src/walkthrough.rs rooms(), doors(), furniture(), furniture_mats()",
                   "rooms": rooms, "doors": doors, "furniture": furniture,
                   "furn_reflector_min_vol": min_vol}, fh, indent=1)
    print(out, len(rooms), "rooms", len(doors), "doors", sum(len(v) for v in furniture.values()), "furniture")


if __name__ == "__main__":
    main()
