"""The late-field backend seam (crates/omg-scene/src/late.rs), GPU side.

`LateBackend` / `WorldLateBackend` mirror the reference traits (late.rs:28-49,
81-91) and the module-level registry mirrors its global Mutex slots
(late.rs:51-64, 93-101). The GPU backends here are what the reference's app
would register under OMG_GPU=1. The reference routes unregistered calls to
its inline CPU tracer (late.rs:107-148); this package has no CPU tracer, so
routing with nothing registered raises instead of falling back.
"""
from __future__ import annotations

import threading
from typing import Optional, Sequence

from .engine import Context, Scene, TraceConfig
from .materials import Material
from .tracer import Echogram


class LateBackend:
    """late.rs:28-49. trace() returns True when `out` holds a fresh echogram."""

    def trace(self, id: int, room, src, lis, n_rays: int, energy, rng, out: Echogram) -> bool:
        raise NotImplementedError

    def poll_into(self, id: int, out: Echogram) -> bool:
        return False


class WorldLateBackend:
    """late.rs:81-91."""

    def trace_world(self, id: int, src, lis, rays: int, panels: Sequence, out: Echogram) -> bool:
        raise NotImplementedError


class Shoebox:
    """scene.rs:27-41: room [0,size]^3 with walls x-,x+,y-,y+,z-,z+."""

    def __init__(self, size, walls: Sequence[Material]):
        self.size = tuple(float(v) for v in size)
        self.walls = list(walls)
        assert len(self.walls) == 6


def _pcg_step(seed: int) -> int:
    """The seed advance of omg-gpu/src/lib.rs:1064 (a PCG LCG step, u32)."""
    return (seed * 747796405 + 2891336453) & 0xFFFFFFFF


class GpuLateBackend(LateBackend):
    """omg-gpu/src/lib.rs:881-890, 1051-1068: a fresh per-ray stream per trace;
    the caller's rng is not consumed (the EMA in Sim does the averaging)."""

    def __init__(self, ctx: Optional[Context] = None, cfg: Optional[TraceConfig] = None):
        self.ctx = ctx or Context(cfg)
        self.seed = 0xD15EA5E

    def trace(self, id, room: Shoebox, src, lis, n_rays, energy, rng, out: Echogram) -> bool:
        self.seed = _pcg_step(self.seed)
        e, _ = self.ctx.trace_box(room.size, room.walls, src, lis, n_rays, energy, self.seed)
        out.bins[:] = e.bins
        out.dirs[:] = e.dirs
        return True


class GpuWorldLateBackend(WorldLateBackend):
    """omg-gpu/src/lib.rs:752-874: the mesh lives with the backend; per call
    only the pose and the panel overlays travel. `ray_mult`/`ray_cap` follow
    WORLD_RAY_MULT / WORLD_RAY_CAP (lib.rs:781-782)."""

    def __init__(self, ctx: Context, scene: Scene, ray_mult: int = 8, ray_cap: int = 8192,
                 max_panels: int = 64):
        self.ctx, self.scene = ctx, scene
        self.seed = 0x5EEDC6D1
        self.ray_mult, self.ray_cap, self.max_panels = ray_mult, ray_cap, max_panels

    def trace_world(self, id, src, lis, rays, panels, out: Echogram) -> bool:
        self.seed = _pcg_step(self.seed)
        n = min(rays * self.ray_mult, self.ray_cap)
        e, _ = self.ctx.trace_world(self.scene, src, lis, n, list(panels)[: self.max_panels], seed=self.seed)
        out.bins[:] = e.bins
        out.dirs[:] = e.dirs
        return True


class AsyncWorldLateBackend(WorldLateBackend):
    """The async form of the seam (late.rs:42-48): trace_world submits and
    returns False; poll_into delivers the result on a later tick."""

    def __init__(self, ctx: Context, scene: Scene, ray_mult: int = 8, ray_cap: int = 8192):
        self.ctx, self.scene = ctx, scene
        self.seed = 0x5EEDC6D1
        self.ray_mult, self.ray_cap = ray_mult, ray_cap
        self.pending = {}

    def trace_world(self, id, src, lis, rays, panels, out: Echogram) -> bool:
        if id in self.pending:
            return False  # one job in flight per id; the gate re-fires later
        self.seed = _pcg_step(self.seed)
        n = min(rays * self.ray_mult, self.ray_cap)
        self.pending[id] = self.ctx.submit_world(self.scene, src, lis, n, list(panels), seed=self.seed)
        return False

    def poll_into(self, id: int, out: Echogram) -> bool:
        t = self.pending.get(id)
        if t is None:
            return False
        r = self.ctx.poll(t, self.scene.n_bands)
        if r is None:
            return False
        del self.pending[id]
        out.bins[:] = r[0].bins
        out.dirs[:] = r[0].dirs
        return True


_LOCK = threading.Lock()
_BACKEND: Optional[LateBackend] = None
_WORLD_BACKEND: Optional[WorldLateBackend] = None


def set_late_backend(b: LateBackend):  # late.rs:56-58
    global _BACKEND
    with _LOCK:
        _BACKEND = b


def clear_late_backend():  # late.rs:62-64
    global _BACKEND
    with _LOCK:
        _BACKEND = None


def set_world_late_backend(b: WorldLateBackend):  # late.rs:95-97
    global _WORLD_BACKEND
    with _LOCK:
        _WORLD_BACKEND = b


def clear_world_late_backend():  # late.rs:99-101
    global _WORLD_BACKEND
    with _LOCK:
        _WORLD_BACKEND = None


def run_trace(id, room, src, lis, n_rays, energy, rng, out: Echogram) -> bool:
    """late.rs:130-148 through the registered backend."""
    with _LOCK:
        if _BACKEND is None:
            raise RuntimeError("no late backend registered (this package has no CPU tracer)")
        return _BACKEND.trace(id, room, src, lis, n_rays, energy, rng, out)


def run_trace_world(id, src, lis, rays, panels, out: Echogram) -> bool:
    """late.rs:107-125 through the registered world backend."""
    with _LOCK:
        if _WORLD_BACKEND is None:
            raise RuntimeError("no world late backend registered (this package has no CPU tracer)")
        return _WORLD_BACKEND.trace_world(id, src, lis, rays, panels, out)


def poll_into(id, out: Echogram) -> bool:
    """late.rs:67-73."""
    with _LOCK:
        if _BACKEND is not None and _BACKEND.poll_into(id, out):
            return True
        if _WORLD_BACKEND is not None and hasattr(_WORLD_BACKEND, "poll_into"):
            return _WORLD_BACKEND.poll_into(id, out)
        return False
