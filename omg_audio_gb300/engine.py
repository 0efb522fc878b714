"""Python face of the C ABI: a device context with scenes, traces, batches,
closest-hit queries, reverb estimation and dome probes.

Every call goes to libomg_cuda.so; nothing here computes a trace on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check, lib
from .materials import Material
from .tracer import Echogram, ReverbParams


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f3(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))


@dataclass
class TraceConfig:
    """Tracer constants as runtime values; defaults are the reference's
    (tracer.rs:12-16, 103, 163; lib.rs:18-22)."""
    n_bands: int = 3
    n_bins: int = 300
    bin_dt: float = 0.010
    max_time: float = 3.0
    max_bounces: int = 64
    energy_floor: float = 1e-7
    receiver_radius: float = 0.5
    wall_eps: float = 1e-3
    speed_of_sound: float = 343.0
    dir_band: int = 1
    device: int = 0
    timeout_ms: int = 20000
    tie_mode: int = 0          # 0: reference first-found; 1: lowest surface id among near-ties
    walk_budget: int = 0       # visits of one closest-hit walk before it stops (flag 4); 0: structural bound
    loop_guard: int = 0        # per-warp loop iterations of a persistent trace kernel (flag 8); 0: 2^22
    tri_test: int = 0          # 0: the reference's Moller-Trumbore; 1: watertight (needs tie_mode 1)

    def to_c(self) -> _lib.omg_params:
        p = _lib.omg_params()
        for k in ("n_bands", "n_bins", "bin_dt", "max_time", "max_bounces", "energy_floor", "receiver_radius",
                  "wall_eps", "speed_of_sound", "dir_band", "device", "timeout_ms", "tie_mode", "walk_budget",
                  "loop_guard", "tri_test"):
            setattr(p, k, getattr(self, k))
        return p


Panel = tuple  # (mn[3], mx[3], Material): late.rs:88


def panels_to_c(panels: Sequence[Panel]):
    arr = (_lib.omg_panel * max(1, len(panels)))()
    for i, (mn, mx, m) in enumerate(panels):
        for k in range(3):
            arr[i].mn[k] = mn[k]
            arr[i].mx[k] = mx[k]
        arr[i].material = m.to_c()
    return arr


def _reverb_of(r: _lib.omg_reverb, nb: int) -> ReverbParams:
    return ReverbParams(np.array(r.rt60[:nb], np.float32), np.array(r.level[:nb], np.float32),
                        np.array(r.rt60_fit[:nb], np.float32), int(r.segments))


# omg_reverb as a numpy record: rt60[8], level[8], rt60_fit[8] f32, segments u64 (104 bytes)
_REVERB_DTYPE = np.dtype([("rt60", np.float32, 8), ("level", np.float32, 8), ("rt60_fit", np.float32, 8),
                          ("segments", np.uint64)])


def _reverbs_of(rv, n: int):
    """All n omg_reverb records of a ctypes array as (rt60, level, rt60_fit, segments) arrays, one copy."""
    rec = np.frombuffer(rv, _REVERB_DTYPE, count=n).copy()
    return rec["rt60"], rec["level"], rec["rt60_fit"], rec["segments"].tolist()


class Context:
    """omg_create / omg_destroy. Raises when no CUDA device is usable."""

    def __init__(self, cfg: Optional[TraceConfig] = None):
        self.cfg = cfg or TraceConfig()
        prm = self.cfg.to_c()
        self.h = lib().omg_create(C.byref(prm))
        if not self.h:
            raise _lib.OmgError(_lib.E_NO_DEVICE, "omg_create")

    def close(self):
        if getattr(self, "h", None):
            lib().omg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def last_error(self) -> str:
        return lib().omg_last_error(self.h).decode()

    def set_limits(self, walk_budget: int = 0, loop_guard: int = 0) -> None:
        """Device-side limits for later calls (omg_set_limits; 0 = default)."""
        self._check(lib().omg_set_limits(self.h, walk_budget, loop_guard), "omg_set_limits")
        self.cfg.walk_budget, self.cfg.loop_guard = walk_budget, loop_guard

    def last_flags(self) -> int:
        """Kernel flag word of the last trace or dome call (omg_last_flags):
        1 stack overflow, 2 crossing list overflow, 4 walk budget, 8 loop guard."""
        return int(lib().omg_last_flags(self.h))

    def _check(self, rc: int, what: str):
        if rc < 0:
            raise _lib.OmgError(rc, f"{what} ({self.last_error()})")
        return rc

    def set_stream(self, cuda_stream: int):
        self._check(lib().omg_set_stream(self.h, C.c_void_p(cuda_stream)), "omg_set_stream")

    def io_bytes(self):
        """(host->device, device->host) bytes of the last one-shot trace call."""
        a, b = C.c_uint64(), C.c_uint64()
        self._check(lib().omg_io_bytes(self.h, C.byref(a), C.byref(b)), "omg_io_bytes")
        return a.value, b.value

    # ------------------------------------------------------------- scenes
    def upload_builder(self, mb: "MeshBuilder", n_bands: int = 3, bvh: int = _lib.BVH_SAH) -> "Scene":
        sid = C.c_uint32()
        self._check(lib().omg_scene_from_builder(self.h, mb.h, n_bands, bvh, C.byref(sid)), "omg_scene_from_builder")
        return Scene(self, sid.value, n_bands)

    def upload_mesh(self, positions, indices, tri_material, materials: Sequence[Material], tri_max_edge=None,
                    n_bands: int = 3, bvh: int = _lib.BVH_SAH) -> "Scene":
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        tm = np.ascontiguousarray(tri_material, np.uint16)
        mats = (_lib.omg_material * max(1, len(materials)))(*[m.to_c() for m in materials])
        te = None if tri_max_edge is None else np.ascontiguousarray(tri_max_edge, np.float32)
        sid = C.c_uint32()
        rc = lib().omg_scene_upload(self.h, _p(pos), len(pos), _p(idx), len(idx), _p(tm),
                                    _p(te) if te is not None else None, mats, len(materials), n_bands, bvh,
                                    C.byref(sid))
        self._check(rc, "omg_scene_upload")
        return Scene(self, sid.value, n_bands)

    # ------------------------------------------------------------- traces
    def trace_box(self, size, walls: Sequence[Material], src, lis, n_rays: int, energy=None, seed: int = 1):
        """LateBackend::trace (late.rs:28-40): returns (Echogram, ReverbParams)."""
        nb = self.cfg.n_bands
        j = _lib.omg_box_job()
        for k in range(3):
            j.size[k] = size[k]
            j.src[k] = src[k]
            j.lis[k] = lis[k]
        for w in range(6):
            j.walls[w] = walls[w].to_c()
        j.n_rays = n_rays
        for b in range(nb):
            j.energy[b] = 1.0 if energy is None else energy[b]
        j.seed = seed & 0xFFFFFFFF
        e = Echogram(self.cfg.n_bins, nb, self.cfg.bin_dt)
        rv = _lib.omg_reverb()
        self._check(lib().omg_trace_box(self.h, C.byref(j), _p(e.bins), _p(e.dirs), C.byref(rv)), "omg_trace_box")
        return e, _reverb_of(rv, nb)

    def trace_world(self, scene: "Scene", src, lis, n_rays: int, panels: Sequence[Panel] = (), energy=None,
                    seed: int = 1):
        """WorldLateBackend::trace_world (late.rs:81-91): returns (Echogram, ReverbParams)."""
        nb = scene.n_bands
        j = _lib.omg_world_job()
        for k in range(3):
            j.src[k] = src[k]
            j.lis[k] = lis[k]
        j.n_rays = n_rays
        for b in range(nb):
            j.energy[b] = 1.0 if energy is None else energy[b]
        j.seed = seed & 0xFFFFFFFF
        parr = panels_to_c(panels)
        e = Echogram(self.cfg.n_bins, nb, self.cfg.bin_dt)
        rv = _lib.omg_reverb()
        rc = lib().omg_trace_world(self.h, scene.id, C.byref(j), parr, len(panels), _p(e.bins), _p(e.dirs),
                                   C.byref(rv))
        self._check(rc, "omg_trace_world")
        return e, _reverb_of(rv, nb)

    def submit_world(self, scene: "Scene", src, lis, n_rays: int, panels: Sequence[Panel] = (), seed: int = 1,
                     energy=None) -> int:
        nb = scene.n_bands
        j = _lib.omg_world_job()
        for k in range(3):
            j.src[k] = src[k]
            j.lis[k] = lis[k]
        j.n_rays = n_rays
        for b in range(nb):
            j.energy[b] = 1.0 if energy is None else energy[b]
        j.seed = seed & 0xFFFFFFFF
        t = C.c_uint32()
        parr = panels_to_c(panels)
        self._check(lib().omg_submit_world(self.h, scene.id, C.byref(j), parr, len(panels), C.byref(t)),
                    "omg_submit_world")
        return t.value

    def poll(self, ticket: int, n_bands: int = 3):
        """LateBackend::poll_into (late.rs:42-48): None while pending."""
        e = Echogram(self.cfg.n_bins, n_bands, self.cfg.bin_dt)
        rv = _lib.omg_reverb()
        rc = lib().omg_poll(self.h, ticket, _p(e.bins), _p(e.dirs), C.byref(rv))
        if rc == _lib.PENDING:
            return None
        self._check(rc, "omg_poll")
        return e, _reverb_of(rv, n_bands)

    def batch(self, jobs: Sequence["Job"], panels: Sequence[Panel] = ()) -> "Batch":
        return Batch(self, jobs, panels)

    def trace_batch(self, jobs: Sequence["Job"], panels: Sequence[Panel] = ()):
        """One-shot batch through the host-buffer entry point."""
        arr, nbf, ndf = jobs_to_c(jobs, self.cfg)
        bins = np.empty(nbf, np.float32)       # every float is written by the call
        dirs = np.empty(ndf, np.float32)
        rv = (_lib.omg_reverb * len(jobs))()
        parr = panels_to_c(panels)
        rc = lib().omg_trace_batch(self.h, arr, len(jobs), parr, len(panels), _p(bins), _p(dirs), rv)
        self._check(rc, "omg_trace_batch")
        return split_outputs(jobs, self.cfg, bins, dirs, rv)

    # ------------------------------------------------------------- queries
    def raycast(self, scene: "Scene", origins, dirs):
        o = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        t = np.zeros(len(o), np.float32)
        tri = np.zeros(len(o), np.uint32)
        self._check(lib().omg_raycast(self.h, scene.id, _p(o), _p(d), len(o), _p(t), _p(tri)), "omg_raycast")
        return t, tri

    def estimate_reverb(self, bins: np.ndarray, bin_dt: Optional[float] = None):
        """estimate_reverb (tracer.rs:204-257) of one (n_bins, nb) or many (n, n_bins, nb) echograms."""
        b = np.ascontiguousarray(bins, np.float32)
        single = b.ndim == 2
        if single:
            b = b[None]
        n, nbins, nb = b.shape
        out = (_lib.omg_reverb * n)()
        rc = lib().omg_estimate_reverb(self.h, _p(b), nbins, nb, bin_dt or self.cfg.bin_dt, n, out)
        self._check(rc, "omg_estimate_reverb")
        res = [_reverb_of(out[i], nb) for i in range(n)]
        return res[0] if single else res


class Scene:
    def __init__(self, ctx: Context, sid: int, n_bands: int):
        self.ctx, self.id, self.n_bands = ctx, sid, n_bands

    def info(self):
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self.ctx._check(lib().omg_scene_info(self.ctx.h, self.id, C.byref(a), C.byref(b), C.byref(c)),
                        "omg_scene_info")
        return dict(nodes=a.value, prims=b.value, tris=c.value)

    def export_bvh(self, with_nodes: bool = True):
        inf = self.info()
        nb = np.zeros((inf["nodes"], 6), np.float32) if with_nodes else None
        nab = np.zeros((inf["nodes"], 2), np.uint32) if with_nodes else None
        pg = np.zeros((inf["prims"], 9), np.float32)
        pt = np.zeros(inf["prims"], np.uint32)
        pm = np.zeros(inf["prims"], np.uint16)
        rc = lib().omg_scene_export_bvh(self.ctx.h, self.id, _p(nb) if with_nodes else None,
                                        _p(nab) if with_nodes else None, _p(pg), _p(pt), _p(pm))
        self.ctx._check(rc, "omg_scene_export_bvh")
        return dict(node_boxes=nb, node_ab=nab, prim_geo=pg, prim_tri=pt, prim_mat=pm)

    def release(self):
        if self.id:
            self.ctx._check(lib().omg_scene_release(self.ctx.h, self.id), "omg_scene_release")
            self.id = 0


@dataclass
class Job:
    """omg_job: a box (size + 6 walls) or an uploaded mesh scene."""
    src: Sequence[float]
    lis: Sequence[float]
    n_rays: int
    seed: int = 1
    scene: Optional[Scene] = None
    box_size: Optional[Sequence[float]] = None
    box_walls: Optional[Sequence[Material]] = None
    energy: Optional[Sequence[float]] = None
    n_bands: int = 0
    n_bins: int = 0
    max_time: float = 0.0
    panel_offset: int = 0
    n_panels: int = 0

    def bands(self, cfg: TraceConfig) -> int:
        return self.n_bands or (self.scene.n_bands if self.scene is not None else cfg.n_bands)

    def bins_len(self, cfg: TraceConfig) -> int:
        return self.n_bins or cfg.n_bins


def jobs_to_c(jobs: Sequence[Job], cfg: TraceConfig):
    arr = (_lib.omg_job * len(jobs))()
    nbf = ndf = 0
    for i, j in enumerate(jobs):
        c = arr[i]
        nb = j.bands(cfg)
        if j.scene is not None:
            c.geom = _lib.GEOM_MESH
            c.scene_id = j.scene.id
        else:
            c.geom = _lib.GEOM_BOX
            for k in range(3):
                c.box_size[k] = j.box_size[k]
            for w in range(6):
                c.box_walls[w] = j.box_walls[w].to_c()
        for k in range(3):
            c.src[k] = j.src[k]
            c.lis[k] = j.lis[k]
        c.n_rays = j.n_rays
        for b in range(nb):
            c.energy[b] = 1.0 if j.energy is None else j.energy[b]
        c.seed = j.seed & 0xFFFFFFFF
        c.n_bands = nb
        c.n_bins = j.bins_len(cfg)
        c.max_time = j.max_time
        c.panel_offset = j.panel_offset
        c.n_panels = j.n_panels
        nbf += c.n_bins * nb
        ndf += c.n_bins * 3
    return arr, nbf, ndf


def split_outputs(jobs, cfg, bins, dirs, rv):
    """Per-job echograms as views of the batch's output arrays (no copies)."""
    out = []
    bo = do = 0
    rt, lv, fit, seg = _reverbs_of(rv, len(jobs))
    for i, j in enumerate(jobs):
        nb, n = j.bands(cfg), j.bins_len(cfg)
        e = Echogram.wrap(bins[bo:bo + n * nb].reshape(n, nb), dirs[do:do + n * 3].reshape(n, 3), cfg.bin_dt)
        bo += n * nb
        do += n * 3
        out.append((e, ReverbParams(rt[i, :nb], lv[i, :nb], fit[i, :nb], seg[i])))
    return out


class Batch:
    """A device-resident batch: omg_batch_create / launch / read."""

    def __init__(self, ctx: Context, jobs: Sequence[Job], panels: Sequence[Panel] = ()):
        self.ctx, self.jobs = ctx, list(jobs)
        arr, self.n_bin_floats, self.n_dir_floats = jobs_to_c(jobs, ctx.cfg)
        parr = panels_to_c(panels)
        bid = C.c_uint32()
        ctx._check(lib().omg_batch_create(ctx.h, arr, len(jobs), parr, len(panels), C.byref(bid)),
                   "omg_batch_create")
        self.id = bid.value

    def launch(self, part: int = 0):
        """part 0: everything; 1: clear + trace kernel; 2: finalize + reverb."""
        self.ctx._check(lib().omg_batch_launch_part(self.ctx.h, self.id, part), "omg_batch_launch_part")

    def read(self):
        """Fresh arrays on every read: the echograms returned are views of them."""
        bins = np.empty(self.n_bin_floats, np.float32)
        dirs = np.empty(self.n_dir_floats, np.float32)
        rv = (_lib.omg_reverb * len(self.jobs))()
        rc = lib().omg_batch_read(self.ctx.h, self.id, _p(bins), _p(dirs), rv)
        self.ctx._check(rc, "omg_batch_read")
        return split_outputs(self.jobs, self.ctx.cfg, bins, dirs, rv)

    def segments(self) -> int:
        s = C.c_uint64()
        self.ctx._check(lib().omg_batch_segments(self.ctx.h, self.id, C.byref(s)), "omg_batch_segments")
        return s.value

    def kernel_count(self) -> int:
        n = C.c_uint32()
        self.ctx._check(lib().omg_batch_kernel_count(self.ctx.h, self.id, C.byref(n)), "omg_batch_kernel_count")
        return n.value

    @staticmethod
    def _shape_dict(r) -> dict:
        return {k: getattr(r, k) for k, _ in _lib.omg_tune_result._fields_}

    def autotune(self, reps: int = 2) -> dict:
        """Time launch shapes on this batch and keep the fastest (omg_batch_autotune)."""
        r = _lib.omg_tune_result()
        self.ctx._check(lib().omg_batch_autotune(self.ctx.h, self.id, reps, C.byref(r)), "omg_batch_autotune")
        return self._shape_dict(r)

    def shape(self) -> dict:
        r = _lib.omg_tune_result()
        self.ctx._check(lib().omg_batch_get_shape(self.ctx.h, self.id, C.byref(r)), "omg_batch_get_shape")
        return self._shape_dict(r)

    def set_shape(self, **kw):
        """Set launch-shape fields by name (the others keep their values)."""
        cur = self.shape()
        cur.update(kw)
        r = _lib.omg_tune_result(**{k: cur[k] for k, _ in _lib.omg_tune_result._fields_})
        self.ctx._check(lib().omg_batch_set_shape(self.ctx.h, self.id, C.byref(r)), "omg_batch_set_shape")

    def destroy(self):
        if self.id:
            lib().omg_batch_destroy(self.ctx.h, self.id)
            self.id = 0


class MeshBuilder:
    """MeshBuilder (mesh.rs:70-165) in the library: 0.1 mm vertex dedup,
    surfaces, per-triangle tessellation limits."""

    def __init__(self):
        self.h = lib().omg_mb_create()

    def __del__(self):
        if getattr(self, "h", None):
            lib().omg_mb_destroy(self.h)
            self.h = None

    def material(self, m: Material) -> int:
        c = m.to_c()
        return lib().omg_mb_material(self.h, C.byref(c))

    def begin_surface(self) -> int:
        return lib().omg_mb_begin_surface(self.h)

    def coarse(self, max_edge: float):
        lib().omg_mb_coarse(self.h, max_edge)

    def tri(self, a, b, c, m: int):
        fa, fb, fc = _f3(a), _f3(b), _f3(c)
        lib().omg_mb_tri(self.h, _p(fa), _p(fb), _p(fc), m)

    def quad(self, a, b, c, d, m: int):
        fa, fb, fc, fd = _f3(a), _f3(b), _f3(c), _f3(d)
        lib().omg_mb_quad(self.h, _p(fa), _p(fb), _p(fc), _p(fd), m)

    def abox(self, mn, mx, m: int):
        fa, fb = _f3(mn), _f3(mx)
        lib().omg_mb_abox(self.h, _p(fa), _p(fb), m)

    def quads(self, q, mat, new_surface=None, max_edge=None):
        q = np.ascontiguousarray(q, np.float32).reshape(-1, 12)
        mat = np.ascontiguousarray(mat, np.uint16)
        ns = None if new_surface is None else np.ascontiguousarray(new_surface, np.uint8)
        me = None if max_edge is None else np.ascontiguousarray(max_edge, np.float32)
        lib().omg_mb_quads(self.h, _p(q), _p(mat), _p(ns) if ns is not None else None,
                           _p(me) if me is not None else None, len(q))

    def export(self):
        nv, nt, nm = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib().omg_mb_counts(self.h, C.byref(nv), C.byref(nt), C.byref(nm))
        pos = np.zeros((nv.value, 3), np.float32)
        idx = np.zeros((nt.value, 3), np.uint32)
        tm = np.zeros(nt.value, np.uint16)
        ts = np.zeros(nt.value, np.uint16)
        te = np.zeros(nt.value, np.float32)
        lib().omg_mb_export(self.h, _p(pos), _p(idx), _p(tm), _p(ts), _p(te))
        return dict(positions=pos, indices=idx, tri_material=tm, tri_surface=ts, tri_max_edge=te)


class DomeProbe:
    """DomeProbe (dome.rs:293-478) over an uploaded world mesh; every call
    samples many listeners, each with its own EMA slot."""

    def __init__(self, ctx: Context, scene: Scene, glass: Sequence = (), n_fan: int = 384):
        self.ctx, self.scene, self.n_fan = ctx, scene, n_fan
        self.nb = scene.n_bands
        arr = dome_panels_to_c(glass, self.nb)
        pid = C.c_uint32()
        ctx._check(lib().omg_dome_create(ctx.h, scene.id, arr, len(glass), n_fan, self.nb, C.byref(pid)),
                   "omg_dome_create")
        self.id = pid.value

    def sample(self, eyes, leaves: Sequence = (), n_rays: Optional[int] = None, max_events: int = 6):
        eyes = np.ascontiguousarray(eyes, np.float32).reshape(-1, 3)
        n_eyes = len(eyes)
        n_rays = n_rays or self.n_fan
        nb = self.nb
        out = (_lib.omg_dome_bin * (9 * n_eyes))()
        raw = np.zeros((n_eyes, 9, nb), np.float32)
        esc = np.zeros((n_eyes, n_rays), np.uint8)
        tp = np.zeros((n_eyes, n_rays, nb), np.float32)
        arr = dome_panels_to_c(leaves, nb)
        rc = lib().omg_dome_sample(self.ctx.h, self.id, _p(eyes), n_eyes, arr, len(leaves), n_rays, max_events, out,
                                   _p(raw), _p(esc), _p(tp))
        self.ctx._check(rc, "omg_dome_sample")
        return self._result(out, n_eyes, raw, esc, tp)

    def submit(self, eyes, leaves: Sequence = (), n_rays: Optional[int] = None, max_events: int = 6,
               stream: int = 0, want: int = 0):
        """Enqueue a sample on a CUDA stream (0: the context's) and return at
        once (omg_dome_submit); collect() waits for it. want: 1 raw, 2 escape,
        4 per-ray throughput."""
        eyes = np.ascontiguousarray(eyes, np.float32).reshape(-1, 3)
        n_rays = n_rays or self.n_fan
        arr = dome_panels_to_c(leaves, self.nb)
        rc = lib().omg_dome_submit(self.ctx.h, self.id, _p(eyes), len(eyes), arr, len(leaves), n_rays, max_events,
                                   want, C.c_void_p(stream) if stream else None)
        self.ctx._check(rc, "omg_dome_submit")
        self._pending = (len(eyes), n_rays, want)

    def collect(self):
        """Wait for the submitted sample; arrays not asked for at submit() come back as None."""
        n_eyes, n_rays, want = self._pending
        nb = self.nb
        out = (_lib.omg_dome_bin * (9 * n_eyes))()
        raw = np.empty((n_eyes, 9, nb), np.float32) if want & 1 else None
        esc = np.empty((n_eyes, n_rays), np.uint8) if want & 2 else None
        tp = np.empty((n_eyes, n_rays, nb), np.float32) if want & 4 else None
        rc = lib().omg_dome_collect(self.ctx.h, self.id, out, _p(raw) if raw is not None else None,
                                    _p(esc) if esc is not None else None, _p(tp) if tp is not None else None)
        self.ctx._check(rc, "omg_dome_collect")
        return self._result(out, n_eyes, raw, esc, tp)

    def _result(self, out, n_eyes, raw, esc, tp):
        nb = self.nb
        # omg_dome_bin is 11 packed floats: dir[3], energy[8]
        flat = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_float)), (9 * n_eyes * 11,)).reshape(n_eyes, 9, 11)
        energy = flat[:, :, 3:3 + nb].copy()
        dirs = flat[:, :, :3].copy()
        ev, th = C.c_uint64(), C.c_uint64()
        lib().omg_dome_segments(self.ctx.h, self.id, C.byref(ev), C.byref(th))
        return dict(energy=energy, dir=dirs, raw=raw, escape=esc, ray_tp=tp,
                    segments=dict(escape_events=ev.value, through_calls=th.value))

    def destroy(self):
        if self.id:
            lib().omg_dome_destroy(self.ctx.h, self.id)
            self.id = 0


def dome_panels_to_c(panels: Sequence, nb: int):
    """panels: DomePanel objects (dome.py) or dicts with axis/plane/lat/z/glass/trans."""
    arr = (_lib.omg_dome_panel * max(1, len(panels)))()
    for i, p in enumerate(panels):
        d = p if isinstance(p, dict) else p.as_dict()
        arr[i].axis = int(d["axis"])
        arr[i].plane = d["plane"]
        arr[i].lat0, arr[i].lat1 = d["lat"]
        arr[i].z0, arr[i].z1 = d["z"]
        arr[i].glass = int(d["glass"])
        for b in range(nb):
            arr[i].trans[b] = d["trans"][b]
    return arr
