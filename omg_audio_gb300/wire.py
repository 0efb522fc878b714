"""The reference's wire formats over the C ABI (include/omg_cuda.h, "wire formats").

- The web bridge's flat trace jobs: a box job of 57 f32 as the wasm build's
  proxy backend queues it (crates/omg-web/src/lib.rs:150-202), a world job of
  1034 f32 (lib.rs:365-416). `trace_web_box_jobs` / `trace_web_world_jobs`
  trace a whole queue in one batch and return the driver's injection records
  (lib.rs:204-218: n_bins x 3 bin energies, then n_bins x 3 direction sums).
- ParamBlock's flat f32 layout, the simulation -> renderer contract
  (crates/omg-core/src/params.rs:57-141).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import lib
from .materials import Material

BOX_JOB_F32S = _lib.WEB_BOX_JOB_F32S
WORLD_JOB_F32S = _lib.WEB_WORLD_JOB_F32S
WORLD_MAX_PANELS = _lib.WEB_WORLD_MAX_PANELS
FLAT_HEADER, FLAT_PER_TAP = _lib.PARAM_FLAT_HEADER, _lib.PARAM_FLAT_PER_TAP


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def box_job(sim_id: int, size, walls: Sequence[Material], src, lis, n_rays: int, seed: int,
            energy=(1.0, 1.0, 1.0)) -> np.ndarray:
    """One flat box job, packed as WebGpuProxy::trace does (lib.rs:180-193):
    every word an f32, the ids and counts included."""
    out = [float(sim_id), float(n_rays), float(seed), *map(float, size), *map(float, src), *map(float, lis),
           *map(float, energy[:3])]
    for w in walls:
        out += [*w.absorption[:3], w.scattering, *w.transmission[:3]]
    a = np.asarray(out, np.float32)
    assert len(a) == BOX_JOB_F32S
    return a


def world_job(sim_id: int, src, lis, n_rays: int, seed: int, panels=()) -> np.ndarray:
    """One flat world job, packed as WebWorldLateProxy::trace_world does
    (lib.rs:398-412): at most 64 panels of 16 f32, zero-padded to the fixed stride.
    panels: (min, max, Material) triples."""
    a = np.zeros(WORLD_JOB_F32S, np.float32)
    np_ = min(len(panels), WORLD_MAX_PANELS)
    a[:10] = [sim_id, n_rays, seed, *src, *lis, np_]
    for k, (mn, mx, m) in enumerate(panels[:np_]):
        a[10 + 16 * k:26 + 16 * k] = [*mn, m.scattering, *mx, 0.0, *m.absorption[:3], 0.0,
                                      *m.transmission[:3], 0.0]
    return a


def _records(ctx, n_jobs: int, fn, *args):
    nb = ctx.cfg.n_bins
    echo = np.zeros((n_jobs, nb * 6), np.float32)
    ids = np.zeros(n_jobs, np.uint32)
    rv = (_lib.omg_reverb * n_jobs)()
    ctx._check(fn(*args, _p(echo), _p(ids), rv), fn.__name__)
    return echo, ids, [rv[i] for i in range(n_jobs)]


def trace_web_box_jobs(ctx, jobs: np.ndarray):
    """A queue of flat box jobs (n x 57 f32) -> (echo records (n, n_bins*6), sim ids, omg_reverb per job)."""
    f = np.ascontiguousarray(jobs, np.float32).ravel()
    n = len(f) // BOX_JOB_F32S
    return _records(ctx, n, lib().omg_trace_web_box_jobs, ctx.h, _p(f), len(f))


def trace_web_world_jobs(ctx, scene, jobs: np.ndarray):
    """A queue of flat world jobs (n x 1034 f32) over an uploaded scene."""
    f = np.ascontiguousarray(jobs, np.float32).ravel()
    n = len(f) // WORLD_JOB_F32S
    return _records(ctx, n, lib().omg_trace_web_world_jobs, ctx.h, scene.id, _p(f), len(f))


def split_echo(echo: np.ndarray, n_bins: int) -> Tuple[np.ndarray, np.ndarray]:
    """An injection record -> (bins (n_bins, 3), dirs (n_bins, 3)), as poll_into reads it (lib.rs:204-218)."""
    return echo[:n_bins * 3].reshape(n_bins, 3), echo[n_bins * 3:].reshape(n_bins, 3)


# ------------------------------------------------------------------ ParamBlock
@dataclass
class Tap:
    """params.rs:7-16."""
    key: int
    delay_s: float
    dir: Tuple[float, float, float]
    gains: Tuple[float, float, float]


@dataclass
class RemoteReverb:
    """params.rs:44-55."""
    rt60: Tuple[float, float, float]
    send: Tuple[float, float, float]
    sh: Tuple[float, ...]


@dataclass
class ParamBlock:
    """params.rs:57-66."""
    taps: List[Tap] = field(default_factory=list)
    rt60: Tuple[float, float, float] = (0.5, 0.5, 0.5)
    level: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    remote: Optional[RemoteReverb] = None
    version: int = 0

    def _c(self):
        pb = _lib.omg_param_block()
        pb.version = self.version
        for b in range(3):
            pb.rt60[b] = self.rt60[b]
            pb.level[b] = self.level[b]
        if self.remote is not None:
            pb.has_remote = 1
            for b in range(3):
                pb.remote_rt60[b] = self.remote.rt60[b]
                pb.remote_send[b] = self.remote.send[b]
            for k in range(9):
                pb.remote_sh[k] = self.remote.sh[k]
        taps = (_lib.omg_tap * max(1, len(self.taps)))()
        for i, t in enumerate(self.taps):
            taps[i].key = t.key
            taps[i].delay_s = t.delay_s
            for k in range(3):
                taps[i].dir[k] = t.dir[k]
                taps[i].gains[k] = t.gains[k]
        return pb, taps

    def flat_len(self) -> int:
        return int(lib().omg_param_block_flat_len(len(self.taps)))

    def write_flat(self) -> np.ndarray:
        """ParamBlock::write_flat (params.rs:79-106)."""
        pb, taps = self._c()
        out = np.zeros(self.flat_len(), np.float32)
        _lib.check(lib().omg_param_block_write_flat(C.byref(pb), taps, len(self.taps), _p(out), len(out)),
                   "omg_param_block_write_flat")
        return out

    @classmethod
    def read_flat(cls, data: np.ndarray) -> "ParamBlock":
        """ParamBlock::read_flat (params.rs:108-141)."""
        d = np.ascontiguousarray(data, np.float32)
        pb = _lib.omg_param_block()
        n = C.c_uint32()
        cap = max(1, (len(d) - FLAT_HEADER) // FLAT_PER_TAP) if len(d) >= FLAT_HEADER else 1
        taps = (_lib.omg_tap * cap)()
        _lib.check(lib().omg_param_block_read_flat(_p(d), len(d), C.byref(pb), taps, cap, C.byref(n)),
                   "omg_param_block_read_flat")
        remote = None
        if pb.has_remote:
            remote = RemoteReverb(tuple(pb.remote_rt60), tuple(pb.remote_send), tuple(pb.remote_sh))
        return cls([Tap(taps[i].key, taps[i].delay_s, tuple(taps[i].dir), tuple(taps[i].gains))
                    for i in range(n.value)], tuple(pb.rt60), tuple(pb.level), remote, int(pb.version))

    @classmethod
    def from_late_states(cls, states) -> List["ParamBlock"]:
        """The reverb part of one block per late-field slot state (omg_param_block_from_late)."""
        n = len(states)
        arr = (_lib.omg_late_state * max(1, n))(*states)
        out = (_lib.omg_param_block * max(1, n))()
        _lib.check(lib().omg_param_block_from_late(arr, n, out), "omg_param_block_from_late")
        return [cls([], tuple(out[i].rt60), tuple(out[i].level), None, int(out[i].version)) for i in range(n)]
