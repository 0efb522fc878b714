"""The learned surrogate of the tracer (no reference counterpart).

`Mlp` wraps the C ABI's tensor-core MLP ensemble (omg_mlp_*). `RoomSurrogate`
is the room-acoustics surrogate on top of it: it maps a shoebox room with up
to four apertures and a source/listener pose (38 input floats) to the
energy-decay curve (EDC, Schroeder backward integral) at 64 log-spaced times
per band (192 outputs, dB), is trained on echograms the GPU tracer produces,
and answers with the tracer as its fallback wherever the inputs leave the
training range or the ensemble's spread exceeds a threshold.

Inputs (38): room size (3); per-surface per-band absorption (6 x 3, surfaces in
the shoebox order x-, x+, y-, y+, z-, z+); aperture openness (4, one per side
wall); source and listener position as fractions of the room size (3 + 3);
and seven derived features: log volume, log surface area, log
source-listener distance, the Sabine RT60 per band (3, from the surface and
aperture absorption) and the open aperture area fraction.
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import lib
from .materials import Material

N_IN = 38
N_TIMES = 64
N_BANDS = 3
N_OUT = N_TIMES * N_BANDS
EDC_T0, EDC_T1 = 0.005, 2.0            # seconds: the EDC sample times span this range
EDC_TIMES = np.geomspace(EDC_T0, EDC_T1, N_TIMES)
EDC_FLOOR_DB = -60.0               # below: noise of the finite ray count, and no use to the RT60
APERTURE_W, APERTURE_H = 1.5, 2.0      # metres: one aperture centred on each side wall, from the floor
C_SOUND = 343.0


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Mlp:
    """An ensemble of MLPs on the GPU (omg_mlp_create / set_data / train /
    omg_surrogate_predict / omg_mlp_grad / omg_mlp_params)."""

    def __init__(self, ctx, n_in: int, hidden: int = 256, n_hidden: int = 4, n_out: int = N_OUT, members: int = 4,
                 seed: int = 1):
        self.ctx = ctx
        self.cfg = _lib.omg_mlp_config(n_in, hidden, n_hidden, n_out, members, seed)
        mid = C.c_uint32()
        ctx._check(lib().omg_mlp_create(ctx.h, C.byref(self.cfg), C.byref(mid)), "omg_mlp_create")
        self.id = mid.value

    def set_data(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        assert x.shape[1] == self.cfg.n_in and y.shape[1] == self.cfg.n_out and len(x) == len(y)
        self.ctx._check(lib().omg_mlp_set_data(self.ctx.h, self.id, _p(x), _p(y), len(x)), "omg_mlp_set_data")

    def train(self, epochs: int, batch: int = 4096, lr: float = 1e-3, lr_final: float = 1e-5,
              weight_decay: float = 1e-4, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
              seed: int = 7) -> np.ndarray:
        tc = _lib.omg_mlp_train_config(epochs, batch, lr, lr_final, weight_decay, beta1, beta2, eps, seed)
        losses = np.zeros((self.cfg.members, epochs), np.float32)
        self.ctx._check(lib().omg_mlp_train(self.ctx.h, self.id, C.byref(tc), _p(losses)), "omg_mlp_train")
        return losses

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        mean = np.zeros((len(x), self.cfg.n_out), np.float32)
        std = np.zeros_like(mean)
        self.ctx._check(lib().omg_surrogate_predict(self.ctx.h, self.id, _p(x), len(x), _p(mean), _p(std)),
                        "omg_surrogate_predict")
        return mean, std

    def query(self, x, level: float):
        """Ensemble mean and, per row, the largest spread among outputs whose
        mean is >= level (omg_surrogate_query)."""
        x = np.ascontiguousarray(x, np.float32)
        mean = np.empty((len(x), self.cfg.n_out), np.float32)
        spread = np.empty(len(x), np.float32)
        self.ctx._check(lib().omg_surrogate_query(self.ctx.h, self.id, _p(x), len(x), _p(mean), _p(spread), level),
                        "omg_surrogate_query")
        return mean, spread

    def grad(self, x, y, member: int = 0):
        """Loss and [(dW, db)] of one member on standardized x, y."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        shapes = self._shapes()
        total = sum(o * i + o for o, i in shapes)
        g = np.zeros(total, np.float32)
        loss = C.c_float()
        self.ctx._check(lib().omg_mlp_grad(self.ctx.h, self.id, member, _p(x), _p(y), len(x), C.byref(loss), _p(g)),
                        "omg_mlp_grad")
        out, off = [], 0
        for o, i in shapes:
            out.append((g[off:off + o * i].reshape(o, i), g[off + o * i:off + o * i + o]))
            off += o * i + o
        return loss.value, out

    def _shapes(self):
        c = self.cfg
        dims = [c.n_in] + [c.hidden] * c.n_hidden + [c.n_out]
        return [(dims[k + 1], dims[k]) for k in range(len(dims) - 1)]

    def _params(self, what: int) -> np.ndarray:
        n = C.c_uint64()
        self.ctx._check(lib().omg_mlp_params(self.ctx.h, self.id, what, None, C.byref(n)), "omg_mlp_params")
        out = np.zeros(n.value, np.float32)
        self.ctx._check(lib().omg_mlp_params(self.ctx.h, self.id, what, _p(out), C.byref(n)), "omg_mlp_params")
        return out

    def layers(self, member: int = 0):
        """[(W, b)] of one member (FP32 master weights)."""
        p = self._params(1)
        c = self.cfg
        off = 2 * c.n_in + 2 * c.n_out
        per = sum(o * i + o for o, i in self._shapes())
        off += member * per
        out = []
        for o, i in self._shapes():
            out.append((p[off:off + o * i].reshape(o, i).astype(np.float64),
                        p[off + o * i:off + o * i + o].astype(np.float64)))
            off += o * i + o
        return out

    # checkpoint: a plain binary with a header (magic, version, config, counts)
    MAGIC = b"OMGSURR1"

    def save(self, path: str):
        w, m = self._params(1), self._params(2)
        c = self.cfg
        with open(path, "wb") as fh:
            fh.write(self.MAGIC)
            fh.write(struct.pack("<6I2Q", c.n_in, c.hidden, c.n_hidden, c.n_out, c.members, c.seed, len(w), len(m)))
            fh.write(w.tobytes())
            fh.write(m.tobytes())

    @classmethod
    def load(cls, ctx, path: str) -> "Mlp":
        with open(path, "rb") as fh:
            if fh.read(8) != cls.MAGIC:
                raise ValueError("not a surrogate checkpoint")
            n_in, hidden, n_hidden, n_out, members, seed, nw, nm = struct.unpack("<6I2Q", fh.read(40))
            w = np.frombuffer(fh.read(4 * nw), np.float32)
            m = np.frombuffer(fh.read(4 * nm), np.float32)
        net = cls(ctx, n_in, hidden, n_hidden, n_out, members, seed)
        ctx._check(lib().omg_mlp_set_params(ctx.h, net.id, 1, _p(np.ascontiguousarray(w)), len(w)), "omg_mlp_set_params")
        ctx._check(lib().omg_mlp_set_params(ctx.h, net.id, 2, _p(np.ascontiguousarray(m)), len(m)), "omg_mlp_set_params")
        return net

    def close(self):
        if self.id:
            lib().omg_mlp_destroy(self.ctx.h, self.id)
            self.id = 0


# ------------------------------------------------------------------ rooms
@dataclass
class Rooms:
    """A set of shoebox rooms, column by column."""
    size: np.ndarray          # (n, 3)
    alpha: np.ndarray         # (n, 6, 3) per surface (x-, x+, y-, y+, z-, z+), per band
    openness: np.ndarray      # (n, 4) apertures on x-, x+, y-, y+
    src: np.ndarray           # (n, 3)
    lis: np.ndarray           # (n, 3)

    def __len__(self):
        return len(self.size)

    def take(self, idx) -> "Rooms":
        return Rooms(self.size[idx], self.alpha[idx], self.openness[idx], self.src[idx], self.lis[idx])


# the training family: sizes, absorption and openness ranges (inputs outside
# them make the surrogate fall back to the tracer)
SIZE_LO = np.array([4.0, 4.0, 2.5])
SIZE_HI = np.array([16.0, 12.0, 6.0])
ALPHA_LO, ALPHA_HI = 0.02, 0.4
SCATTERING = 0.1


def sample_rooms(n: int, seed: int) -> Rooms:
    """n rooms of the training family. Absorption: half the rooms draw each of
    their 18 values independently from U[ALPHA_LO, ALPHA_HI]; the other half
    draw a room level from the log-uniform distribution on that range and
    scatter every value around it (a factor exp(N(0, 0.35^2)), clipped to the
    range), so that rooms whose surfaces are all hard, or all soft, are as
    common as the rest (independent draws almost never give them)."""
    rng = np.random.default_rng(seed)
    size = rng.uniform(SIZE_LO, SIZE_HI, (n, 3))
    alpha = rng.uniform(ALPHA_LO, ALPHA_HI, (n, 6, N_BANDS))
    level = np.exp(rng.uniform(np.log(ALPHA_LO), np.log(ALPHA_HI), (n, 1, 1)))
    near = np.clip(level * np.exp(0.35 * rng.standard_normal((n, 6, N_BANDS))), ALPHA_LO, ALPHA_HI)
    alpha = np.where(rng.random((n, 1, 1)) < 0.5, alpha, near)
    openness = rng.uniform(0.0, 1.0, (n, 4))
    # 0 to 4 apertures per room
    n_ap = rng.integers(0, 5, n)
    rank = np.argsort(rng.random((n, 4)), axis=1)
    openness = np.where(rank < n_ap[:, None], openness, 0.0)
    # poses >= 1 m from every wall
    src = 1.0 + rng.random((n, 3)) * (size - 2.0)
    lis = 1.0 + rng.random((n, 3)) * (size - 2.0)
    return Rooms(size, alpha, openness, src, lis)


# the city's octave bands (63 Hz ... 8 kHz) that are the surrogate's 250 Hz, 1 kHz and 4 kHz
CITY_BANDS = (2, 4, 6)
CITY_CELL = (15.0, 11.0)     # largest ground-floor room of a building (x, y), inside the family's sizes


def city_rooms(buildings, sources, absorption, window_frac=0.4, listener_z=1.5) -> Rooms:
    """The city's room/source pairs as shoebox rooms (every building x every
    source): the ground floor of each building is cut into a grid of rooms no
    larger than CITY_CELL, and the pair's room is the cell nearest the source.
    Walls take the facade's absorption, the floor the ground's, the ceiling
    the slabs' (CITY_BANDS of the city's octave bands); a wall on the
    building's perimeter has its windows (window_frac of it open) as the
    aperture's openness, an inner wall none. The source stands in the cell at
    the point nearest the street source, 1 m from the walls; the listener at
    the cell's centre. buildings (n, 6): footprint min x, y, size x, y,
    height, storey height; sources (m, 3)."""
    b = np.asarray(buildings, np.float64)
    src = np.asarray(sources, np.float64)
    nb, ns = len(b), len(src)
    bi = np.repeat(np.arange(nb), ns)
    si = np.tile(np.arange(ns), nb)
    x0, y0, w, d, fh = b[bi, 0], b[bi, 1], b[bi, 2], b[bi, 3], b[bi, 5]
    nx, ny = np.ceil(w / CITY_CELL[0]), np.ceil(d / CITY_CELL[1])
    cw, cd = w / nx, d / ny
    px = np.clip(src[si, 0], x0, x0 + w)
    py = np.clip(src[si, 1], y0, y0 + d)
    ix = np.minimum(np.floor((px - x0) / cw), nx - 1)
    iy = np.minimum(np.floor((py - y0) / cd), ny - 1)
    size = np.stack([cw, cd, fh], 1)
    lo = np.stack([x0 + ix * cw, y0 + iy * cd], 1)
    pick = lambda k: np.asarray(absorption[k], np.float64)[list(CITY_BANDS)]
    alpha = np.empty((len(bi), 6, N_BANDS))
    alpha[:, 0:4, :] = pick("facade")
    alpha[:, 4, :] = pick("ground")
    alpha[:, 5, :] = pick("slab")
    outer = np.stack([ix == 0, ix == nx - 1, iy == 0, iy == ny - 1], 1)
    openness = np.where(outer, window_frac, 0.0)
    s_local = np.stack([np.clip(px - lo[:, 0], 1.0, cw - 1.0), np.clip(py - lo[:, 1], 1.0, cd - 1.0),
                        np.clip(src[si, 2], 1.0, fh - 1.0)], 1)
    l_local = np.stack([0.5 * cw, 0.5 * cd, np.minimum(listener_z, 0.5 * fh)], 1)
    return Rooms(size, alpha, openness, s_local, l_local)


def aperture_boxes(size):
    """One aperture per side wall (x-, x+, y-, y+) of each room: a panel box
    flush with the wall, APERTURE_W wide (clipped to the wall) and APERTURE_H
    high from the floor (clipped). size (n, 3) -> mn (n, 4, 3), mx (n, 4, 3),
    area (n, 4)."""
    size = np.atleast_2d(size)
    n = len(size)
    h = np.minimum(APERTURE_H, size[:, 2] - 0.1)
    mn, mx, area = np.zeros((n, 4, 3)), np.zeros((n, 4, 3)), np.zeros((n, 4))
    for k in range(4):
        axis = 0 if k < 2 else 1
        other = 1 - axis
        span = size[:, other]
        w = np.minimum(APERTURE_W, span - 0.2)
        c = 0.5 * span
        wall = np.zeros(n) if k % 2 == 0 else size[:, axis]
        # a thin slab on the room side of the wall: it is met before the wall
        if k % 2 == 0:
            mn[:, k, axis], mx[:, k, axis] = wall - 0.05, wall + 0.001
        else:
            mn[:, k, axis], mx[:, k, axis] = wall - 0.001, wall + 0.05
        mn[:, k, other], mx[:, k, other] = c - 0.5 * w, c + 0.5 * w
        mn[:, k, 2], mx[:, k, 2] = 0.0, h
        area[:, k] = w * h
    return mn, mx, area


def features(r: Rooms) -> np.ndarray:
    """The 38 inputs of every room, (n, 38)."""
    sx, sy, sz = r.size[:, 0], r.size[:, 1], r.size[:, 2]
    V = sx * sy * sz
    areas = np.stack([sy * sz, sy * sz, sx * sz, sx * sz, sx * sy, sx * sy], 1)
    S = areas.sum(1)
    _, _, ap = aperture_boxes(r.size)
    # Sabine: A_b = sum_s area_s alpha_sb, each aperture area absorbing its
    # openness instead of its wall's alpha
    A = np.einsum("ns,nsb->nb", areas, r.alpha)
    A += np.einsum("nk,nkb->nb", ap, r.openness[:, :, None] - r.alpha[:, :4, :])
    A = np.maximum(A, 1e-3)
    sabine = 0.161 * V[:, None] / A
    d = np.maximum(np.linalg.norm(r.src - r.lis, axis=1), 1e-3)
    return np.concatenate([r.size, r.alpha.reshape(len(r), -1), r.openness, r.src / r.size, r.lis / r.size,
                           np.log(V)[:, None], np.log(S)[:, None], np.log(d)[:, None], sabine,
                           ((ap * r.openness).sum(1) / S)[:, None]], axis=1).astype(np.float32)


SABINE_COLS = slice(34, 37)


def in_range(x: np.ndarray) -> np.ndarray:
    """Rows whose primary inputs lie inside the training family."""
    size = x[:, 0:3]
    alpha = x[:, 3:21]
    op = x[:, 21:25]
    frac = x[:, 25:31]
    return (np.all(size >= SIZE_LO - 1e-6, 1) & np.all(size <= SIZE_HI + 1e-6, 1) &
            np.all(alpha >= ALPHA_LO - 1e-6, 1) & np.all(alpha <= ALPHA_HI + 1e-6, 1) &
            np.all((op >= 0) & (op <= 1), 1) & np.all((frac >= 0) & (frac <= 1), 1))


def edc_db(bins: np.ndarray, bin_dt: float) -> np.ndarray:
    """EDC in dB (Schroeder backward integral, FP64) at EDC_TIMES, per band, for
    one echogram [n_bins x NB] or many [n x n_bins x NB]; the curve is read at
    the start of each bin and interpolated linearly; floor EDC_FLOOR_DB."""
    b = np.asarray(bins, np.float64)
    one = b.ndim == 2
    if one:
        b = b[None]
    tail = np.cumsum(b[:, ::-1], axis=1)[:, ::-1]
    e = tail / np.maximum(tail[:, 0:1], 1e-300)
    t = np.arange(b.shape[1]) * bin_dt
    j = np.clip(np.searchsorted(t, EDC_TIMES, side="right") - 1, 0, len(t) - 2)
    w = ((EDC_TIMES - t[j]) / bin_dt)[None, :, None]
    out = e[:, j] * (1.0 - w) + e[:, j + 1] * w
    out = np.maximum(10.0 * np.log10(np.maximum(out, 1e-30)), EDC_FLOOR_DB)
    return out[0] if one else out


def rt60_from_edc(edc: np.ndarray) -> np.ndarray:
    """RT60 per band from an EDC on the EDC_TIMES grid: 60 dB over the time the
    curve takes from -5 to -25 dB (the reference's T20 form, tracer.rs:205-257),
    crossings interpolated in time. edc: [..., N_TIMES, NB] -> [..., NB]
    (NaN where a crossing is missing)."""
    e = np.asarray(edc, np.float64)
    return 3.0 * (_cross(e, -25.0) - _cross(e, -5.0))


def _cross(e, level):
    below = e <= level
    has = below.any(axis=-2)
    j = np.argmax(below, axis=-2)
    jm = np.maximum(j - 1, 0)
    c0 = np.take_along_axis(e, jm[..., None, :], axis=-2)[..., 0, :]
    c1 = np.take_along_axis(e, j[..., None, :], axis=-2)[..., 0, :]
    t0, t1 = EDC_TIMES[jm], EDC_TIMES[j]
    den = np.where(c1 != c0, c1 - c0, 1.0)
    t = np.where(j == 0, EDC_TIMES[0], np.where(c1 != c0, t0 + (t1 - t0) * (level - c0) / den, t1))
    return np.where(has, t, np.nan)


def trace_rooms(ctx, rooms: Rooms, n_rays: int, seed: int, chunk: int = 8192):
    """Echograms of the rooms from the GPU tracer: shoebox jobs with the
    aperture panels, batched. Returns bins [n x n_bins x NB] and the reverb
    parameters of every room."""
    from .engine import Job
    mn, mx, _ = aperture_boxes(rooms.size)
    bins_all, rv_all = [], []
    for c0 in range(0, len(rooms), chunk):
        jobs, panels = [], []
        for i in range(c0, min(c0 + chunk, len(rooms))):
            walls = [Material(tuple(float(a) for a in rooms.alpha[i, w]), SCATTERING, (0.0,) * N_BANDS)
                     for w in range(6)]
            off = len(panels)
            for k in range(4):
                op = float(rooms.openness[i, k])
                panels.append((tuple(mn[i, k]), tuple(mx[i, k]), Material((op,) * N_BANDS, 0.0, (0.0,) * N_BANDS)))
            jobs.append(Job(tuple(rooms.src[i]), tuple(rooms.lis[i]), n_rays, seed=seed + i,
                            box_size=tuple(rooms.size[i]), box_walls=walls, panel_offset=off, n_panels=4))
        for e, rv in ctx.trace_batch(jobs, panels):
            bins_all.append(e.bins.copy())
            rv_all.append(rv)
    return np.stack(bins_all), rv_all


class RoomSurrogate:
    """Per-room EDC from the MLP ensemble, with the tracer as fallback."""

    def __init__(self, ctx, members: int = 4, hidden: int = 256, n_hidden: int = 4, seed: int = 1):
        self.ctx = ctx
        self.net = Mlp(ctx, N_IN, hidden, n_hidden, N_OUT, members, seed)
        self.threshold_db = 3.0

    def fit(self, rooms: Rooms, edcs, epochs: int, batch: int = 4096, **kw) -> np.ndarray:
        x = features(rooms)
        y = np.asarray(edcs, np.float32).reshape(len(rooms), -1)
        self.net.set_data(x, y)
        return self.net.train(epochs, batch, **kw)

    def predict(self, rooms: Rooms):
        """EDC [n x N_TIMES x NB] (dB), per-room spread (dB) over the part of
        the curve the RT60 reads (down to -30 dB), usable mask."""
        x = features(rooms)
        mean, sig = self.net.query(x, -30.0)
        ok = in_range(x) & (sig <= self.threshold_db)
        return mean.reshape(len(rooms), N_TIMES, N_BANDS), sig, ok

    def answer(self, rooms: Rooms, n_rays: int = 4096, seed: int = 1):
        """EDCs of every room: the surrogate's where usable, the tracer's elsewhere."""
        edc, _, ok = self.predict(rooms)
        fallback = np.nonzero(~ok)[0]
        if len(fallback):
            bins, _ = trace_rooms(self.ctx, rooms.take(fallback), n_rays, seed)
            edc[fallback] = edc_db(bins, self.ctx.cfg.bin_dt)
        return edc, ok
