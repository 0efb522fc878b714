"""CPU restatement of the reference's wire formats — TEST INFRASTRUCTURE.

- ParamBlock::write_flat / read_flat (crates/omg-core/src/params.rs:67-141),
  including Rust's `as` casts (f32 -> integer: truncate, saturate, NaN -> 0;
  integer -> f32: round to nearest).
- The web bridge's flat jobs as the wasm proxy backends pack them
  (crates/omg-web/src/lib.rs:170-193 box jobs, :386-412 world jobs) and as
  the JavaScript driver decodes them (web/gpu.js:181-199, 420-437: each word
  stored into a Uint32Array slot, i.e. ToUint32).
Only the tests import this module.
"""
from __future__ import annotations

import math

import numpy as np

FLAT_HEADER = 24        # params.rs:73
FLAT_PER_TAP = 9        # params.rs:74
GPU_JOB_F32S = 57       # lib.rs:157
WLATE_MAX_PANELS = 64   # lib.rs:371
WLATE_JOB_F32S = 10 + WLATE_MAX_PANELS * 16   # lib.rs:372


def f32(x) -> float:
    return float(np.float32(x))


def rust_as_uint(x: float, bits: int) -> int:
    """Rust `f32 as u32/u64/usize`."""
    if math.isnan(x) or x <= 0.0:
        return 0
    if math.isinf(x):
        return (1 << bits) - 1
    return min(int(math.trunc(x)), (1 << bits) - 1)


def uint_to_f32(v: int) -> float:
    """Rust `u32/u64 as f32`: round to nearest, ties to even."""
    e = v.bit_length() - 24
    if e <= 0:
        return float(v)
    q, r = divmod(v, 1 << e)
    half = 1 << (e - 1)
    if r > half or (r == half and q & 1):
        q += 1
    return float(q << e)


def js_to_uint32(x: float) -> int:
    """ECMAScript ToUint32 (a Number stored into a Uint32Array)."""
    if math.isnan(x) or math.isinf(x):
        return 0
    return int(math.trunc(x)) % (1 << 32)


def write_flat(pb: dict) -> np.ndarray:
    """params.rs:79-106. pb: version, taps [(key, delay, dir3, gains3)], rt60, level,
    remote None or (rt60, send, sh9)."""
    taps = pb["taps"]
    out = np.zeros(FLAT_HEADER + len(taps) * FLAT_PER_TAP, np.float32)
    out[0] = uint_to_f32(pb["version"])
    out[1] = len(taps)
    for b in range(3):
        out[2 + b] = pb["rt60"][b]
        out[5 + b] = pb["level"][b]
    if pb["remote"] is not None:
        rt, send, sh = pb["remote"]
        out[8] = 1.0
        for b in range(3):
            out[9 + b] = rt[b]
            out[12 + b] = send[b]
        out[15:24] = sh
    for i, (key, delay, d, g) in enumerate(taps):
        o = FLAT_HEADER + i * FLAT_PER_TAP
        out[o] = uint_to_f32(key)
        out[o + 1] = delay
        out[o + 2:o + 5] = d
        out[o + 5:o + 8] = g
    return out


def read_flat(data: np.ndarray) -> dict:
    """params.rs:108-141 (raises IndexError where the reference panics)."""
    data = np.asarray(data, np.float32)
    n_taps = rust_as_uint(float(data[1]), 64)
    need = FLAT_HEADER + n_taps * FLAT_PER_TAP
    if need > len(data):
        raise IndexError("flat ParamBlock shorter than its tap count")
    pb = {"version": rust_as_uint(float(data[0]), 64), "rt60": [f32(data[2 + b]) for b in range(3)],
          "level": [f32(data[5 + b]) for b in range(3)], "remote": None, "taps": []}
    if data[8] > 0.5:
        pb["remote"] = ([f32(data[9 + b]) for b in range(3)], [f32(data[12 + b]) for b in range(3)],
                        [f32(v) for v in data[15:24]])
    for i in range(n_taps):
        o = FLAT_HEADER + i * FLAT_PER_TAP
        pb["taps"].append((rust_as_uint(float(data[o]), 32), f32(data[o + 1]),
                           [f32(v) for v in data[o + 2:o + 5]], [f32(v) for v in data[o + 5:o + 8]]))
    return pb


def pack_box_job(sim_id, n_rays, seed_u32, size, src, lis, energy, walls) -> np.ndarray:
    """lib.rs:170-193: walls as (absorption3, scattering, transmission3)."""
    v = [float(sim_id), float(n_rays), float(seed_u32), *size, *src, *lis, *energy]
    for ab, sc, tr in walls:
        v += [*ab, sc, *tr]
    a = np.asarray(v, np.float32)
    assert len(a) == GPU_JOB_F32S
    return a


def decode_box_job(f: np.ndarray) -> dict:
    """gpu.js:181-199 (packJob): the words the trace kernel sees."""
    f = [float(x) for x in np.asarray(f, np.float32)]
    return {"id": js_to_uint32(f[0]), "n_rays": js_to_uint32(f[1]), "seed": js_to_uint32(f[2]),
            "size": f[3:6], "src": f[6:9], "lis": f[9:12], "energy": f[12:15],
            "walls": [(f[15 + 7 * w:18 + 7 * w], f[18 + 7 * w], f[19 + 7 * w:22 + 7 * w]) for w in range(6)]}


def pack_world_job(sim_id, n_rays, seed_u32, src, lis, panels) -> np.ndarray:
    """lib.rs:386-412: panels (min3, max3, absorption3, scattering, transmission3), <= 64, fixed stride."""
    a = np.zeros(WLATE_JOB_F32S, np.float32)
    n = min(len(panels), WLATE_MAX_PANELS)
    a[:10] = [sim_id, n_rays, seed_u32, *src, *lis, n]
    for k, (mn, mx, ab, sc, tr) in enumerate(panels[:n]):
        a[10 + 16 * k:26 + 16 * k] = [*mn, sc, *mx, 0.0, *ab, 0.0, *tr, 0.0]
    return a


def decode_world_job(f: np.ndarray) -> dict:
    """gpu.js:420-437 (pumpWorldLate) with unit energy."""
    f32s = np.asarray(f, np.float32)
    f = [float(x) for x in f32s]
    n = int(min(f[9], WLATE_MAX_PANELS)) if f[9] > 0 else 0
    panels = []
    for k in range(n):
        q = f[10 + 16 * k:26 + 16 * k]
        panels.append((q[0:3], q[4:7], q[8:11], q[3], q[12:15]))
    return {"id": js_to_uint32(f[0]), "n_rays": js_to_uint32(f[1]), "seed": js_to_uint32(f[2]),
            "src": f[3:6], "lis": f[6:9], "energy": [1.0, 1.0, 1.0], "panels": panels}
