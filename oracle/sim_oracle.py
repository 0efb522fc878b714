"""CPU restatement of the sim's late-field bookkeeping — TEST INFRASTRUCTURE.

Follows crates/omg-scene/src/sim.rs:32-75 (TraceGate), sim.rs:346-398
(Sim::reverb_world: async result first, else the gate within the tick's
budget, EMA, reverb, late direction, staleness compensation) and
crates/omg-core/src/tracer.rs:46-77 (Echogram::ema, late_direction), in f32
where the reference computes in f32. The reverb and late direction come from
the C oracle (oracle.py). Only the tests import this module.
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O

F32_MAX = float(np.finfo(np.float32).max)


class TraceGate:
    """sim.rs:38-75. `phase` staggers the refresh age of a fresh gate."""

    def __init__(self, phase: int, max_age: int):
        self.last_src = (F32_MAX, 0.0, 0.0)
        self.last_lis = (F32_MAX, 0.0, 0.0)
        self.last_energy = [0.0, 0.0, 0.0]
        self.age = phase
        self.max_age = max_age

    def should_trace(self, src, lis, energy) -> bool:
        self.age += 1

        moved = any(abs(e1 - e0) > 0.1 * max(e0, e1, 1e-6) for e0, e1 in zip(self.last_energy, energy))
        if self.age >= self.max_age or _dist(src, self.last_src) > 0.25 or _dist(lis, self.last_lis) > 0.25 or moved:
            self.last_src, self.last_lis, self.last_energy = tuple(src), tuple(lis), list(energy)
            self.age = 0
            return True
        return False


def ema(avg: np.ndarray, cur: np.ndarray, alpha: float) -> np.ndarray:
    """tracer.rs:46-57: a += alpha (o - a), elementwise in f32."""
    a = np.float32(alpha)
    return (avg + a * (cur.astype(np.float32) - avg)).astype(np.float32)


class SimOracle:
    """Sim::reverb_world (sim.rs:346-398) for one instance, with the fresh
    echogram of a landed trace handed in by the caller."""

    def __init__(self, n_bins: int, nb: int, bin_dt: float, phase: int, max_age: int, from_s: float,
                 dir_band: int = 1):
        self.bins = np.zeros((n_bins, nb), np.float32)
        self.dirs = np.zeros((n_bins, 3), np.float32)
        self.bin_dt, self.from_s, self.dir_band = bin_dt, from_s, dir_band
        self.gate = TraceGate(phase, max_age)
        self.version = 0          # calls so far (Sim::version, sim.rs:376)
        self.updates = 0          # traces blended in
        self.rp_dist = F32_MAX

    def step(self, fresh, src, lis, budget: list):
        """fresh: (bins, dirs) of the trace that lands this tick, or None.
        Returns (fire, rt60, level, dir, aniso): whether the gate fired (the
        caller traces) and the outputs of this call."""
        traced = fresh is not None
        fire = False
        if not traced and budget[0] > 0 and self.gate.should_trace(src, lis, [1.0] * self.bins.shape[1]):
            budget[0] -= 1
            fire = True
        if traced:
            alpha = 1.0 if self.version == 0 else 0.3     # sim.rs:372-375
            self.bins = ema(self.bins, fresh[0], alpha)
            self.dirs = ema(self.dirs, fresh[1], alpha)
            self.updates += 1
            self.rp_dist = _dist(src, lis)
        self.version += 1
        d, aniso = O.late_direction(self.bins, self.dirs, self.bin_dt, self.from_s, mid=self.dir_band)
        rt, lv, _ = O.estimate_reverb(self.bins, self.bin_dt)
        lv = lv.astype(np.float32).copy()
        if self.rp_dist < F32_MAX:                         # sim.rs:386-394
            k = min((np.float32(self.rp_dist) + np.float32(1.0)) / (np.float32(_dist(src, lis)) + np.float32(1.0)),
                    np.float32(1.0))
            lv = (lv * np.float32(k)).astype(np.float32)
        return fire, rt, lv, d, aniso


def _dist(a, b) -> float:
    """Vec3 length of a - b in f32; f32::MAX positions overflow to inf as in the reference."""
    with np.errstate(over="ignore"):
        return float(np.sqrt(np.float32(sum((np.float32(x) - np.float32(y)) ** 2 for x, y in zip(a, b)))))


def isclose_dir(a, b, tol=1e-4) -> bool:
    return all(math.isclose(float(x), float(y), abs_tol=tol) for x, y in zip(a, b))
