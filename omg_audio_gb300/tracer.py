"""Echogram and reverb parameters (crates/omg-core/src/tracer.rs:18-78,
crates/omg-core/src/params.rs:17-37).

The echogram is the tracer's output: per-band energy per time bin and the
energy-weighted arrival direction per bin. `ema` and `late_direction` are the
reference's bookkeeping on it (tracer.rs:46-77), kept in f32 as there.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class ReverbParams:
    """params.rs:17-37 plus the least-squares T20 fit and the segment count."""
    rt60: np.ndarray
    level: np.ndarray
    rt60_fit: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))
    segments: int = 0


class Echogram:
    """bins: (n_bins, n_bands) f32; dirs: (n_bins, 3) f32 (tracer.rs:18-33)."""

    def __init__(self, n_bins: int = 300, n_bands: int = 3, bin_dt: float = 0.010):
        self.bin_dt = float(bin_dt)
        self.bins = np.zeros((n_bins, n_bands), np.float32)
        self.dirs = np.zeros((n_bins, 3), np.float32)

    @classmethod
    def wrap(cls, bins: np.ndarray, dirs: np.ndarray, bin_dt: float) -> "Echogram":
        """An echogram over existing (n_bins, n_bands) and (n_bins, 3) f32 arrays, not copied."""
        e = cls.__new__(cls)
        e.bin_dt, e.bins, e.dirs = float(bin_dt), bins, dirs
        return e

    @property
    def n_bins(self) -> int:
        return self.bins.shape[0]

    @property
    def n_bands(self) -> int:
        return self.bins.shape[1]

    def clear(self):  # tracer.rs:35-42
        self.bins[:] = 0
        self.dirs[:] = 0

    def ema(self, other: "Echogram", alpha: float):
        """tracer.rs:46-57: a += alpha * (o - a), f32."""
        a = np.float32(alpha)
        self.bins += a * (other.bins - self.bins)
        self.dirs += a * (other.dirs - self.dirs)

    def late_direction(self, from_s: float, mid: int = 1):
        """tracer.rs:62-77: (unit direction, anisotropy in [0, 1]) from from_s on."""
        start = int(np.float32(from_s) / np.float32(self.bin_dt))
        start = min(max(start, 0), self.n_bins)
        v = np.zeros(3, np.float32)
        e = np.float32(0)
        for i in range(start, self.n_bins):
            v += self.dirs[i]
            e += self.bins[i, mid]
        ln = np.float32(np.sqrt(np.float32(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])))
        if ln < 1e-12 or e < 1e-12:
            return np.array([1.0, 0.0, 0.0], np.float32), 0.0
        return (v / ln).astype(np.float32), float(min(ln / e, np.float32(1.0)))
