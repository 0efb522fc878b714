"""ctypes wrapper of the CPU oracle (liboracle.so) — TEST INFRASTRUCTURE.

The oracle restates omg-audio's CPU tracer (crates/omg-core/src/tracer.rs,
scene.rs, mesh.rs, rng.rs) and ambient dome (crates/omg-scene/src/dome.rs) in
C++, templated on f32 (the reference's own arithmetic) and f64 (the FP64
oracle). Only the tests, the smoke check and the benchmark's CPU-baseline leg
import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
MAXB = 8

# -ffp-contract=off: no fused multiply-add, so f32 arithmetic rounds exactly as
# the reference's Rust code does. No -march flags: it builds the same on x86 and Arm.
BUILD_CMD = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
             os.path.join(HERE, "omg_oracle.cpp"), "-o", LIB_PATH]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "omg_oracle.cpp")
    hdrs = [os.path.join(HERE, f) for f in ("omg_oracle.hpp", "omg_oracle_early.hpp")]
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in hdrs])):
        return LIB_PATH
    subprocess.check_call(BUILD_CMD)
    return LIB_PATH


class Material(C.Structure):
    """crates/omg-core/src/material.rs:7-16 with a runtime band count (<= 8)."""
    _fields_ = [("absorption", C.c_float * MAXB), ("scattering", C.c_float),
                ("transmission", C.c_float * MAXB)]

    @staticmethod
    def make(absorption, scattering, transmission):
        m = Material()
        for i, v in enumerate(absorption):
            m.absorption[i] = v
        m.scattering = scattering
        for i, v in enumerate(transmission):
            m.transmission[i] = v
        return m


class BoxC(C.Structure):
    _fields_ = [("size", C.c_float * 3), ("walls", Material * 6)]


class BoxPanelC(C.Structure):
    _fields_ = [("mn", C.c_float * 3), ("mx", C.c_float * 3), ("m", Material)]


class TraceParams(C.Structure):
    _fields_ = [("n_bands", C.c_uint32), ("n_bins", C.c_uint32), ("bin_dt", C.c_float),
                ("max_time", C.c_float), ("max_bounces", C.c_uint32), ("energy_floor", C.c_float),
                ("receiver_radius", C.c_float), ("wall_eps", C.c_float), ("speed_of_sound", C.c_float),
                ("dir_band", C.c_uint32), ("tie_mode", C.c_uint32)]


class DomePanel(C.Structure):
    _fields_ = [("axis", C.c_int), ("plane", C.c_float), ("lat0", C.c_float), ("lat1", C.c_float),
                ("z0", C.c_float), ("z1", C.c_float), ("glass", C.c_int), ("trans", C.c_float * MAXB)]


def params(n_bands=3, n_bins=300, bin_dt=0.010, max_time=3.0, max_bounces=64, energy_floor=1e-7,
           receiver_radius=0.5, wall_eps=1e-3, speed_of_sound=343.0, dir_band=1, tie_mode=0) -> TraceParams:
    """Defaults are the reference constants (tracer.rs:12-16, 103, 163; lib.rs:18-22)."""
    return TraceParams(n_bands, n_bins, bin_dt, max_time, max_bounces, energy_floor, receiver_radius,
                       wall_eps, speed_of_sound, dir_band, tie_mode)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, U32, U64, F, I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int
        fp = C.POINTER(C.c_float)
        L.orc_mb_new.restype = P
        L.orc_mb_free.argtypes = [P]
        L.orc_mb_material.argtypes = [P, C.POINTER(Material)]
        L.orc_mb_material.restype = U32
        L.orc_mb_begin_surface.argtypes = [P]
        L.orc_mb_begin_surface.restype = U32
        L.orc_mb_coarse.argtypes = [P, F]
        L.orc_mb_tri.argtypes = [P, fp, fp, fp, U32]
        L.orc_mb_quads.argtypes = [P, P, P, P, P, U32]
        L.orc_mb_abox.argtypes = [P, fp, fp, U32]
        L.orc_mb_counts.argtypes = [P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]
        L.orc_mb_export.argtypes = [P, P, P, P, P, P]
        L.orc_mesh_new.argtypes = [I, P]
        L.orc_mesh_new.restype = P
        L.orc_mesh_free.argtypes = [P]
        L.orc_mesh_info.argtypes = [P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]
        L.orc_mesh_export_bvh.argtypes = [P, P, P, P, P, P]
        L.orc_mesh_raycast.argtypes = [P, P, P, U32, I, P, P, P]
        L.orc_mesh_segment_hits.argtypes = [P, P, P, P, P, P, U32]
        L.orc_mesh_segment_hits.restype = U32
        L.orc_trace_box.argtypes = [I, C.POINTER(BoxC), P, U32, C.POINTER(TraceParams), P, P, U32, P, I, U64,
                                    U32, U32, I, P, P, P]
        L.orc_trace_mesh.argtypes = [I, P, P, U32, C.POINTER(TraceParams), P, P, U32, P, I, U64, U32, U32, I,
                                     P, P, P]
        L.orc_trace_mesh_log.argtypes = [I, P, C.POINTER(TraceParams), P, P, U32, P, U32, U32, U32, P, P, U32]
        L.orc_trace_mesh_log.restype = U32
        L.orc_estimate_reverb.argtypes = [P, U32, U32, F, I, P, P, P]
        L.orc_late_direction.argtypes = [P, P, U32, U32, U32, F, F, I, P, P]
        L.orc_dome_new.argtypes = [P, P, U32, U32, U32, I]
        L.orc_dome_new.restype = P
        L.orc_dome_free.argtypes = [P]
        L.orc_dome_sample.argtypes = [P, P, P, U32, U32, U32, U32, F, P, P, P, P, P, P]
        L.orc_dome_fan.argtypes = [U32, I, P]
        L.orc_pcg_draws.argtypes = [U32, U32, U32, P]
        L.orc_xorshift_draws.argtypes = [U64, U32, P]
        L.orc_early_new.argtypes = [P, P, U32]
        L.orc_early_new.restype = P
        L.orc_early_free.argtypes = [P]
        L.orc_early_base_overlay.argtypes = [P]
        L.orc_early_base_overlay.restype = U32
        L.orc_early_n_surfaces.argtypes = [P]
        L.orc_early_n_surfaces.restype = U32
        L.orc_early_discover.argtypes = [P, P, U32, U32, I, P, P, U32]
        L.orc_early_discover.restype = U32
        L.orc_early_solve.argtypes = [P, P, P, U32, P, P, U32, P, P, U32, P, P, I]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


TRAV_KEYS = ("node_reads", "prim_tests", "queries", "internal_visits", "leaf_visits", "child_boxes",
             "unique_nodes")


def _trav(st) -> dict:
    """The traversal counters (omg_oracle.hpp TraversalStats) by name."""
    return {k: int(v) for k, v in zip(TRAV_KEYS, st)}


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(3))


# ---------------------------------------------------------------- builders
class MeshBuilder:
    """crates/omg-core/src/mesh.rs:70-165."""

    def __init__(self):
        self.h = lib().orc_mb_new()

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mb_free(self.h)
            self.h = None

    def material(self, m: Material) -> int:
        return lib().orc_mb_material(self.h, C.byref(m))

    def begin_surface(self) -> int:
        return lib().orc_mb_begin_surface(self.h)

    def coarse(self, e: float):
        lib().orc_mb_coarse(self.h, e)

    def tri(self, a, b, c, m: int):
        fa, fb, fc = _f3(a), _f3(b), _f3(c)
        fp = C.POINTER(C.c_float)
        lib().orc_mb_tri(self.h, fa.ctypes.data_as(fp), fb.ctypes.data_as(fp), fc.ctypes.data_as(fp), m)

    def quad(self, a, b, c, d, m: int):
        self.tri(a, b, c, m)
        self.tri(a, c, d, m)

    def quads(self, q: np.ndarray, mat: np.ndarray, new_surface: np.ndarray, max_edge: np.ndarray):
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, 12)
        mat = np.ascontiguousarray(mat, dtype=np.uint16)
        ns = np.ascontiguousarray(new_surface, dtype=np.uint8)
        me = np.ascontiguousarray(max_edge, dtype=np.float32)
        lib().orc_mb_quads(self.h, _p(q), _p(mat), _p(ns), _p(me), len(q))

    def abox(self, mn, mx, m: int):
        fa, fb = _f3(mn), _f3(mx)
        fp = C.POINTER(C.c_float)
        lib().orc_mb_abox(self.h, fa.ctypes.data_as(fp), fb.ctypes.data_as(fp), m)

    def export(self):
        nv, nt, nm = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib().orc_mb_counts(self.h, C.byref(nv), C.byref(nt), C.byref(nm))
        pos = np.zeros((nv.value, 3), np.float32)
        idx = np.zeros((nt.value, 3), np.uint32)
        tm = np.zeros(nt.value, np.uint16)
        ts = np.zeros(nt.value, np.uint16)
        te = np.zeros(nt.value, np.float32)
        lib().orc_mb_export(self.h, _p(pos), _p(idx), _p(tm), _p(ts), _p(te))
        return dict(positions=pos, indices=idx, tri_material=tm, tri_surface=ts, tri_max_edge=te)

    def build(self, real: str = "f32") -> "Mesh":
        return Mesh(lib().orc_mesh_new(0 if real == "f32" else 1, self.h), real)


class Mesh:
    """crates/omg-core/src/mesh.rs:19-38, 167-620 (BVH built on construction)."""

    def __init__(self, h, real):
        self.h = h
        self.real = real

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_free(self.h)
            self.h = None

    def info(self):
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib().orc_mesh_info(self.h, C.byref(a), C.byref(b), C.byref(c))
        return dict(nodes=a.value, prims=b.value, tris=c.value)

    def export_bvh(self):
        inf = self.info()
        nb = np.zeros((inf["nodes"], 6), np.float32)
        nab = np.zeros((inf["nodes"], 2), np.uint32)
        pg = np.zeros((inf["prims"], 9), np.float32)
        pt = np.zeros(inf["prims"], np.uint32)
        pm = np.zeros(inf["prims"], np.uint16)
        rc = lib().orc_mesh_export_bvh(self.h, _p(nb), _p(nab), _p(pg), _p(pt), _p(pm))
        assert rc == 0
        return dict(node_boxes=nb, node_ab=nab, prim_geo=pg, prim_tri=pt, prim_mat=pm)

    def raycast(self, o: np.ndarray, d: np.ndarray, brute: bool = False, tie: bool = False):
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        n = len(o)
        t = np.zeros(n, np.float64)
        tri = np.zeros(n, np.uint32)
        st = np.zeros(7, np.uint64)
        lib().orc_mesh_raycast(self.h, _p(o), _p(d), n, int(brute) | (2 if tie else 0), _p(t), _p(tri), _p(st))
        return t, tri, _trav(st)

    def segment_hits(self, a, b, cap: int = 256):
        fa, fb = _f3(a), _f3(b)
        t = np.zeros(cap, np.float64)
        tri = np.zeros(cap, np.uint32)
        mat = np.zeros(cap, np.uint16)
        n = lib().orc_mesh_segment_hits(self.h, _p(fa), _p(fb), _p(t), _p(tri), _p(mat), cap)
        n = min(n, cap)
        return t[:n], tri[:n], mat[:n]


# ------------------------------------------------------------------ tracer
def _panels_arr(panels):
    if not panels:
        return None, 0
    arr = (BoxPanelC * len(panels))()
    for i, (mn, mx, m) in enumerate(panels):
        for k in range(3):
            arr[i].mn[k] = mn[k]
            arr[i].mx[k] = mx[k]
        arr[i].m = m
    return arr, len(panels)


def _trace_common(fn, first, real, panels, P, src, lis, n_rays, energy, rng, seed, ray_begin, ray_end,
                  threads, acc64=False):
    nb = P.n_bands
    bins = np.zeros((P.n_bins, nb), np.float64)
    dirs = np.zeros((P.n_bins, 3), np.float64)
    st = np.zeros(2 + 7, np.uint64)
    e = np.zeros(MAXB, np.float32)
    e[:nb] = np.asarray(energy, np.float32)[:nb]
    parr, np_ = _panels_arr(panels)
    ray_end = n_rays if ray_end is None else ray_end
    rc = fn(0 if real == "f32" else 1, first, C.cast(parr, C.c_void_p) if parr is not None else None, np_,
            C.byref(P), _p(_f3(src)), _p(_f3(lis)), n_rays, _p(e), (0 if rng == "xorshift" else 1) | (0x10 if acc64 else 0), seed,
            ray_begin, ray_end, threads, _p(bins), _p(dirs), _p(st))
    assert rc == 0, rc
    return bins, dirs, dict(segments=int(st[0]), receiver_hits=int(st[1]), **_trav(st[2:]))


def trace_box(size, walls, src, lis, n_rays, energy=(1, 1, 1), P=None, *, real="f32", rng="pcg", seed=1,
              panels=(), ray_begin=0, ray_end=None, threads=1, acc64=False):
    """tracer.rs:80-202 over Shoebox (scene.rs:27-88) [+ WithPanels]. acc64: f32
    trajectories with double histogram sums."""
    P = P or params()
    box = BoxC()
    for k in range(3):
        box.size[k] = size[k]
    for i in range(6):
        box.walls[i] = walls[i]
    return _trace_common(lib().orc_trace_box, C.byref(box), real, panels, P, src, lis, n_rays, energy, rng,
                         seed, ray_begin, ray_end, threads, acc64)


def trace_mesh(mesh: Mesh, src, lis, n_rays, energy=(1, 1, 1), P=None, *, rng="pcg", seed=1, panels=(),
               ray_begin=0, ray_end=None, threads=1, acc64=False):
    """tracer.rs:80-202 over Mesh (mesh.rs:607-620) [+ WithPanels]."""
    P = P or params()
    return _trace_common(lib().orc_trace_mesh, mesh.h, mesh.real, panels, P, src, lis, n_rays, energy, rng,
                         seed, ray_begin, ray_end, threads, acc64)


def trace_mesh_log(mesh: Mesh, src, lis, n_rays, seed, ray_begin, ray_end, energy=(1, 1, 1), P=None,
                   cap=1 << 20):
    """Per-segment (origin, dir, closest original tri) log of rays [ray_begin, ray_end)."""
    P = P or params()
    e = np.zeros(MAXB, np.float32)
    e[:P.n_bands] = np.asarray(energy, np.float32)[:P.n_bands]
    seg = np.zeros((cap, 6), np.float32)
    tri = np.zeros(cap, np.uint32)
    n = lib().orc_trace_mesh_log(0 if mesh.real == "f32" else 1, mesh.h, C.byref(P), _p(_f3(src)),
                                 _p(_f3(lis)), n_rays, _p(e), seed, ray_begin, ray_end, _p(seg), _p(tri), cap)
    n = min(n, cap)
    return seg[:n], tri[:n]


def estimate_reverb(bins: np.ndarray, bin_dt: float, level_f32: bool = True):
    """tracer.rs:204-257. Returns (rt60[nb], level[nb], rt60_lsq[nb])."""
    bins = np.ascontiguousarray(bins, np.float64)
    nbins, nb = bins.shape
    rt = np.zeros(nb, np.float32)
    lv = np.zeros(nb, np.float32)
    fit = np.zeros(nb, np.float64)
    lib().orc_estimate_reverb(_p(bins), nbins, nb, bin_dt, int(level_f32), _p(rt), _p(lv), _p(fit))
    return rt, lv, fit


def late_direction(bins, dirs, bin_dt, from_s, mid=1, f32=True):
    """tracer.rs:62-77. Returns (unit dir[3], anisotropy)."""
    bins = np.ascontiguousarray(bins, np.float64)
    dirs = np.ascontiguousarray(dirs, np.float64)
    d = np.zeros(3, np.float32)
    a = np.zeros(1, np.float32)
    lib().orc_late_direction(_p(bins), _p(dirs), bins.shape[0], bins.shape[1], mid, bin_dt, from_s, int(f32),
                             _p(d), _p(a))
    return d, float(a[0])


# -------------------------------------------------------------------- dome
def dome_panels(panels):
    """panels: list of dicts(axis, plane, lat=(a,b), z=(a,b), glass, trans=[...])."""
    if not panels:
        return None, 0
    arr = (DomePanel * len(panels))()
    for i, p in enumerate(panels):
        arr[i].axis = int(p["axis"])
        arr[i].plane = p["plane"]
        arr[i].lat0, arr[i].lat1 = p["lat"]
        arr[i].z0, arr[i].z1 = p["z"]
        arr[i].glass = int(p["glass"])
        for b, v in enumerate(p["trans"]):
            arr[i].trans[b] = v
    return arr, len(panels)


class DomeProbe:
    """crates/omg-scene/src/dome.rs:293-478 over a prebuilt world mesh."""

    def __init__(self, mesh: Mesh, glass=(), n_fan=384, nb=3, tie=False):
        arr, n = dome_panels(list(glass))
        self._glass = arr
        self.mesh = mesh
        self.nb = nb
        self.h = lib().orc_dome_new(mesh.h, C.cast(arr, C.c_void_p) if arr is not None else None, n, n_fan, nb,
                                    int(tie))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_dome_free(self.h)
            self.h = None

    def sample(self, eye, leaves=(), n_rays=384, max_events=6, ema=0.35):
        arr, n = dome_panels(list(leaves))
        nb = self.nb
        out_dir = np.zeros((9, 3), np.float32)
        out_e = np.zeros((9, nb), np.float32)
        raw = np.zeros((9, nb), np.float64)
        esc = np.zeros(n_rays, np.uint8)
        tp = np.zeros((n_rays, nb), np.float32)
        st = np.zeros(2 + 7, np.uint64)
        rc = lib().orc_dome_sample(self.h, _p(_f3(eye)), C.cast(arr, C.c_void_p) if arr is not None else None,
                                   n, n_rays, max_events, nb, ema, _p(out_dir), _p(out_e), _p(raw), _p(esc),
                                   _p(tp), _p(st))
        assert rc == 0, rc
        return dict(dir=out_dir, energy=out_e, raw=raw, escape=esc, ray_tp=tp,
                    stats=dict(escape_events=int(st[0]), through_calls=int(st[1]), **_trav(st[2:])))


def dome_fan(n: int, real: str = "f32") -> np.ndarray:
    out = np.zeros((n, 3), np.float64)
    lib().orc_dome_fan(n, 0 if real == "f32" else 1, _p(out))
    return out


def pcg_draws(seed: int, ray: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_pcg_draws(seed, ray, n, _p(out))
    return out


def xorshift_draws(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint64)
    lib().orc_xorshift_draws(seed, n, _p(out))
    return out


# ------------------------------------------------------------- world build
class RoomC(C.Structure):
    """walkthrough.rs:29-42."""
    _fields_ = [("min", C.c_float * 2), ("max", C.c_float * 2), ("height", C.c_float),
                ("barrier_height", C.c_float), ("floor_z", C.c_float), ("wall_thickness", C.c_float),
                ("outdoor", C.c_int), ("walls", Material * 6)]


class DoorC(C.Structure):
    """walkthrough.rs:228-249 with the pane's amplitude transmission."""
    _fields_ = [("rooms", C.c_int * 2), ("pos", C.c_float * 2), ("axis", C.c_int), ("half", C.c_float),
                ("height", C.c_float), ("zc", C.c_float), ("glass", C.c_int), ("openness", C.c_float),
                ("heavy", C.c_int), ("pane_trans", C.c_float * MAXB)]


def world_build(mb: MeshBuilder, rooms, doors, town=(-40.0, 120.0), wall_max_edge=0.0, nb=3):
    """dome.rs:121-258 into an oracle MeshBuilder. rooms/doors: dicts with the
    walkthrough fields; room walls are oracle Materials; door 'pane_trans' is
    the pane's amplitude transmission. Returns the glass panes as dicts."""
    L = lib()
    L.orc_world_build.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_float, C.c_float,
                                  C.c_float, C.c_uint32, C.c_void_p, C.c_uint32]
    L.orc_world_build.restype = C.c_uint32
    ra = (RoomC * len(rooms))()
    for i, r in enumerate(rooms):
        ra[i].min[0], ra[i].min[1] = r["min"]
        ra[i].max[0], ra[i].max[1] = r["max"]
        ra[i].height, ra[i].barrier_height = r["height"], r["barrier_height"]
        ra[i].floor_z, ra[i].wall_thickness = r["floor_z"], r["wall_thickness"]
        ra[i].outdoor = int(r["outdoor"])
        for w in range(6):
            ra[i].walls[w] = r["walls"][w]
    da = (DoorC * max(1, len(doors)))()
    for i, d in enumerate(doors):
        da[i].rooms[0], da[i].rooms[1] = d["rooms"]
        da[i].pos[0], da[i].pos[1] = d["pos"]
        da[i].axis, da[i].half, da[i].height, da[i].zc = d["axis"], d["half"], d["height"], d["zc"]
        da[i].glass, da[i].openness, da[i].heavy = int(d["glass"]), d["openness"], int(d["heavy"])
        for b, v in enumerate(d.get("pane_trans", ())):
            da[i].pane_trans[b] = v
    cap = 256
    ga = (DomePanel * cap)()
    n = L.orc_world_build(mb.h, C.cast(ra, C.c_void_p), len(rooms), C.cast(da, C.c_void_p), len(doors), town[0],
                          town[1], wall_max_edge, nb, C.cast(ga, C.c_void_p), cap)
    out = []
    for i in range(min(n, cap)):
        g = ga[i]
        out.append(dict(axis=g.axis, plane=g.plane, lat=(g.lat0, g.lat1), z=(g.z0, g.z1), glass=bool(g.glass),
                        trans=tuple(g.trans[:nb])))
    return out


def sincos_f32(phi: np.ndarray):
    """The f32 sin/cos both the oracle and the kernel use for ray directions."""
    phi = np.ascontiguousarray(phi, np.float32)
    s = np.zeros_like(phi)
    c = np.zeros_like(phi)
    L = lib()
    L.orc_sincos_f32.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    L.orc_sincos_f32(_p(phi), len(phi), _p(s), _p(c))
    return s, c


# ----------------------------------------------------- world early reflections
class AabbC(C.Structure):
    """crates/omg-core/src/pt.rs:31-35."""
    _fields_ = [("mn", C.c_float * 3), ("mx", C.c_float * 3), ("transmission", C.c_float * 3)]


def aabbs(extras):
    """(min, max, transmission3) triples -> a ctypes array (or None)."""
    if not extras:
        return None
    arr = (AabbC * len(extras))()
    for i, (mn, mx, tr) in enumerate(extras):
        for k in range(3):
            arr[i].mn[k] = mn[k]
            arr[i].mx[k] = mx[k]
            arr[i].transmission[k] = tr[k]
    return arr


class Early:
    """pt_mesh.rs over an f32 oracle mesh: SurfaceTable (+ furniture faces),
    mesh_chains discovery, mesh_record solves."""

    def __init__(self, mesh: "Mesh", furniture=()):
        assert mesh.real == "f32"
        self.mesh = mesh      # keeps the mesh alive
        parr, n = _panels_arr(list(furniture))
        self.h = lib().orc_early_new(mesh.h, C.cast(parr, C.c_void_p) if parr is not None else None, n)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_early_free(self.h)
            self.h = None

    @property
    def base_overlay(self) -> int:
        return int(lib().orc_early_base_overlay(self.h))

    @property
    def n_surfaces(self) -> int:
        return int(lib().orc_early_n_surfaces(self.h))

    def discover(self, listener, n_rays=768, rot=0, use_boxes=True, cap=1 << 16):
        """mesh_chains: list of (chain tuple, order) in first-found order."""
        ch = np.zeros((cap, 3), np.uint16)
        od = np.zeros(cap, np.uint8)
        n = lib().orc_early_discover(self.h, _p(_f3(listener)), n_rays, rot, int(use_boxes), _p(ch), _p(od), cap)
        n = min(n, cap)
        return [(tuple(int(v) for v in ch[i]), int(od[i])) for i in range(n)]

    def solve(self, sources, chains, listener, extras=(), threads=1):
        """mesh_record for every (source, chain) pair, source-major.
        sources: (id, pos) pairs; chains: (chain3, order) pairs.
        Returns (records (n_src, n_chain, 7) = delay, dir3, gains3; valid bool (n_src, n_chain))."""
        ns, nc = len(sources), len(chains)
        ids = np.array([s[0] for s in sources], np.uint16)
        pos = np.array([s[1] for s in sources], np.float32).reshape(-1, 3)
        ch = np.array([c[0] for c in chains], np.uint16).reshape(-1, 3)
        od = np.array([c[1] for c in chains], np.uint8)
        out = np.zeros((ns, nc, 7), np.float32)
        valid = np.zeros((ns, nc), np.uint8)
        ex = aabbs(list(extras))
        lib().orc_early_solve(self.h, _p(ids), _p(pos), ns, _p(ch), _p(od), nc, _p(_f3(listener)),
                              C.cast(ex, C.c_void_p) if ex is not None else None, len(extras), _p(out), _p(valid),
                              threads)
        return out, valid.astype(bool)
