"""Extract the reference's walkthrough world (rooms and doors) as JSON data.

Reads crates/omg-scene/src/walkthrough.rs of the reference checkout (text
only, nothing is executed) and writes tests/golden/walkthrough_world.json:
the room table of `rooms()` (walkthrough.rs:44-226) and the door table of
`doors()` (walkthrough.rs:275-307), with wall materials by preset name. The
dome tests of dome.rs:496-654 run on this world.

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


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    src = open(os.path.join(ref, "crates/omg-scene/src/walkthrough.rs")).read()
    rooms, doors = parse(src)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "walkthrough_world.json")
    with open(out, "w") as fh:
        json.dump({"source": "crates/omg-scene/src/walkthrough.rs rooms() and doors()", "rooms": rooms,
                   "doors": doors}, fh, indent=1)
    print(out, len(rooms), "rooms", len(doors), "doors")


if __name__ == "__main__":
    main()
