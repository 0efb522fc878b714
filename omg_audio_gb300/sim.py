"""The consumer side of the late-field seam for many sim instances at once.

The reference's `Sim` (crates/omg-scene/src/sim.rs) keeps, per sound source, a
trace gate (sim.rs:32-75), an averaged echogram fed by the late backend
(sim.rs:79-100, 346-398: the async result lands first, otherwise the gate may
fire within the tick's trace budget; each landed echogram is blended in with
Echogram::ema) and derives the reverb and the late direction from it, with
the level scaled down while the source has moved away since the last trace.

Here the averaged echograms of all instances live in device memory
(`LateField`, the library's omg_late_*): a tick traces every instance whose
gate fired in ONE batched launch and blends, reduces and estimates on the
device; only the per-instance reverb and direction come back. `SimField`
runs the reference's per-instance tick logic over it, with the GPU backend's
async timing: a trace submitted on one tick lands on the next.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import lib
from .engine import Context, Job, Panel, Scene, _p, jobs_to_c, panels_to_c
from .late import _pcg_step
from .tracer import Echogram, ReverbParams

F32_MAX = float(np.finfo(np.float32).max)
GATE_MAX_AGE = 8                    # quality.rs:133-138 (Tier::High), clamped 1..64 (quality.rs:177-179)
WORLD_RAYS = 512                    # quality.rs:185-191 (Tier::High)
WORLD_RAY_MULT, WORLD_RAY_CAP = 8, 8192   # omg-gpu/src/lib.rs:781-782
LATE_DIR_FROM_S = 0.08              # sim.rs:377: late_direction(0.08)


def _dist(a, b) -> float:
    """Vec3 length of a - b in f32 (vec3.rs); a never-set position (f32::MAX)
    is infinitely far, as the f32 square overflows there too."""
    with np.errstate(over="ignore"):
        d = np.asarray(a, np.float32) - np.asarray(b, np.float32)
        return float(np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])))


class TraceGate:
    """sim.rs:38-75: trace again once the source or the listener moved more
    than 0.25 m, an energy changed by more than 10 %, or `max_age` ticks
    passed; `phase` staggers the refresh of instances created together."""

    def __init__(self, phase: int = 0, max_age: int = GATE_MAX_AGE):
        self.last_src = (F32_MAX, 0.0, 0.0)
        self.last_lis = (F32_MAX, 0.0, 0.0)
        self.last_energy = None
        self.age = int(phase)
        self.max_age = int(min(max(max_age, 1), 64))

    def should_trace(self, src, lis, energy) -> bool:
        self.age += 1
        last_e = self.last_energy if self.last_energy is not None else [0.0] * len(energy)
        moved = any(abs(np.float32(e1) - np.float32(e0)) > np.float32(0.1) * max(np.float32(e0), np.float32(e1),
                                                                                np.float32(1e-6))
                    for e0, e1 in zip(last_e, energy))
        if (self.age >= self.max_age or _dist(src, self.last_src) > 0.25 or _dist(lis, self.last_lis) > 0.25
                or moved):
            self.last_src, self.last_lis, self.last_energy = tuple(src), tuple(lis), list(energy)
            self.age = 0
            return True
        return False


@dataclass
class LateState:
    """omg_late_state: one instance's late field."""
    rt60: np.ndarray
    level: np.ndarray
    dir: np.ndarray
    anisotropy: float
    version: int
    updated_tick: int


class LateField:
    """The library's late field (omg_late_*): `n_slots` averaged echograms in
    device memory, with the context's bins and bands."""

    def __init__(self, ctx: Context, n_slots: int, dir_from_s: float = LATE_DIR_FROM_S):
        self.ctx, self.n_slots = ctx, int(n_slots)
        self.nb = ctx.cfg.n_bands
        fid = C.c_uint32()
        ctx._check(lib().omg_late_create(ctx.h, self.n_slots, float(dir_from_s), C.byref(fid)), "omg_late_create")
        self.id = fid.value
        self._states = (_lib.omg_late_state * self.n_slots)()
        self.pending = False

    def submit(self, slots: Sequence[int], jobs: Sequence[Job], panels: Sequence[Panel] = (),
               alpha: Optional[Sequence[float]] = None) -> Optional[int]:
        """Enqueue a tick (returns its number), or None while one is in flight."""
        sl = (C.c_uint32 * max(len(slots), 1))(*[int(s) for s in slots])
        arr, _, _ = jobs_to_c(jobs, self.ctx.cfg) if jobs else (None, 0, 0)
        al = (C.c_float * len(jobs))(*[float(a) for a in alpha]) if alpha is not None and jobs else None
        parr = panels_to_c(panels)
        t = C.c_uint32()
        rc = lib().omg_late_submit(self.ctx.h, self.id, sl, arr, al, len(jobs), parr, len(panels), C.byref(t))
        if rc == _lib.PENDING:
            return None
        self.ctx._check(rc, "omg_late_submit")
        self.pending = True
        return t.value

    def poll(self, wait: bool = False) -> Optional[Tuple[int, List[LateState]]]:
        """(tick, states) once the last tick is done (None while pending,
        unless `wait`: then a bounded wait on the context's timeout)."""
        t = C.c_uint32()
        deadline = time.monotonic() + max(self.ctx.cfg.timeout_ms, 1000) / 1000.0
        while True:
            rc = lib().omg_late_poll(self.ctx.h, self.id, self._states, C.byref(t))
            if rc != _lib.PENDING:
                break
            if not wait:
                return None
            if time.monotonic() > deadline:
                raise TimeoutError("late field: tick not done within the context timeout")
            time.sleep(0.0002)
        self.ctx._check(rc, "omg_late_poll")
        self.pending = False
        nb = self.nb
        out = [LateState(np.array(s.rt60[:nb], np.float32), np.array(s.level[:nb], np.float32),
                         np.array(s.dir[:3], np.float32), float(s.anisotropy), int(s.version),
                         int(s.updated_tick)) for s in self._states]
        return t.value, out

    def _settled(self, rc: int, what: str):
        if rc == _lib.PENDING:
            raise _lib.OmgError(rc, f"{what}: a tick is in flight (poll it first)")
        self.ctx._check(rc, what)

    def reset(self, slot: int):
        """Forget a slot's history (not while a tick is in flight)."""
        self._settled(lib().omg_late_reset(self.ctx.h, self.id, int(slot)), "omg_late_reset")

    def read(self, slot: int) -> Echogram:
        """A slot's averaged echogram (not while a tick is in flight)."""
        cfg = self.ctx.cfg
        e = Echogram(cfg.n_bins, self.nb, cfg.bin_dt)
        self._settled(lib().omg_late_read(self.ctx.h, self.id, int(slot), _p(e.bins), _p(e.dirs)), "omg_late_read")
        return e

    def close(self):
        if self.id:
            lib().omg_late_destroy(self.ctx.h, self.id)
            self.id = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SimField:
    """Sim::reverb_world (sim.rs:346-398) for `n_sims` instances on one world
    scene, over a LateField with the GPU backend's async timing.

    tick(poses, panels) runs one simulation tick: for each instance in order,
    a trace submitted on the previous tick lands (its echogram was blended in
    on the device); otherwise, while the tick's `budget` lasts, the instance's
    gate may fire, and fired instances are traced together after the loop.
    Returns per instance (ReverbParams, late direction, anisotropy), the
    level scaled by min(1, (d_then + 1) / (d_now + 1)) for the distance at the
    last landing (sim.rs:386-394)."""

    def __init__(self, ctx: Context, scene: Scene, n_sims: int, rays: int = WORLD_RAYS, budget: int = 1,
                 max_age: int = GATE_MAX_AGE, dir_from_s: float = LATE_DIR_FROM_S, seed: int = 0x5EEDC6D1):
        self.ctx, self.scene, self.n = ctx, scene, int(n_sims)
        self.rays = min(int(rays) * WORLD_RAY_MULT, WORLD_RAY_CAP)
        self.budget = int(budget)
        self.field = LateField(ctx, self.n, dir_from_s)
        # Sim::new staggers the gates by instance id, phase id % 8 (sim.rs:98-107)
        self.gates = [TraceGate(i % 8, max_age) for i in range(self.n)]
        self.version = [0] * self.n
        self.rp_dist = [F32_MAX] * self.n
        self.seed = seed & 0xFFFFFFFF
        self.inflight: List[int] = []
        self.states: List[LateState] = self._empty_states()
        self.last_jobs: List[Job] = []
        self.last_slots: List[int] = []

    def _empty_states(self):
        nb = self.field.nb
        return [LateState(np.full(nb, 0.5, np.float32), np.zeros(nb, np.float32), np.array([1, 0, 0], np.float32),
                          0.0, 0, 0) for _ in range(self.n)]

    def tick(self, poses: Sequence[Tuple[Sequence[float], Sequence[float]]], panels: Sequence[Panel] = ()):
        assert len(poses) == self.n
        landed = set()
        if self.field.pending:
            _, self.states = self.field.poll(wait=True)
            landed = set(self.inflight)
        budget = self.budget
        fire: List[int] = []
        out = []
        nb = self.field.nb
        for i, (src, lis) in enumerate(poses):
            traced = i in landed
            if not traced and budget > 0 and self.gates[i].should_trace(src, lis, [1.0] * nb):
                budget -= 1
                fire.append(i)
            if traced:
                self.rp_dist[i] = _dist(src, lis)
            self.version[i] += 1
            st = self.states[i]
            level = st.level.copy()
            if self.rp_dist[i] < F32_MAX:
                k = min((np.float32(self.rp_dist[i]) + np.float32(1.0)) / (np.float32(_dist(src, lis)) +
                                                                           np.float32(1.0)), np.float32(1.0))
                level = (level * np.float32(k)).astype(np.float32)
            out.append((ReverbParams(st.rt60.copy(), level), st.dir.copy(), st.anisotropy))
        jobs = []
        for i in fire:
            self.seed = _pcg_step(self.seed)
            src, lis = poses[i]
            jobs.append(Job(tuple(src), tuple(lis), self.rays, seed=self.seed, scene=self.scene, panel_offset=0,
                            n_panels=len(panels)))
        # the result lands on the next call, whose version is already >= 1:
        # sim.rs:372-375 then blends with 0.3
        alpha = [1.0 if self.version[i] == 0 else 0.3 for i in fire]
        self.last_jobs, self.last_slots = jobs, list(fire)
        if jobs:
            t = self.field.submit(fire, jobs, panels, alpha)
            assert t is not None
            self.inflight = list(fire)
        else:
            self.inflight = []
        return out

    def close(self):
        self.field.close()
