"""TEST INFRASTRUCTURE: a numpy restatement of the watertight ray-triangle test
and of the near-tie closest hit over it, the checker of the GPU's watertight
mode (omg_params.tri_test = OMG_TRI_WATERTIGHT). Nothing in the product path
imports this module.

The test is the published one: Woop, Benthin, Wald 2013, "Watertight
Ray/Triangle Intersection", Journal of Computer Graphics Techniques 2(1).
Every f32 operation below is one numpy float32 operation, rounded to nearest
as the device rounds it, in the device's order (omg_audio_gb300/csrc/
device_common.cuh: ray_tri_wt):
  - kz: the axis of the largest |d| (the first of equal ones), kx and ky the
    next two, swapped when d_kz < 0;
  - S = (d_kx / d_kz, d_ky / d_kz, 1 / d_kz);
  - each vertex minus the origin, then sheared: X = v_kx - Sx v_kz,
    Y = v_ky - Sy v_kz;
  - U = Cx By - Cy Bx, V = Ax Cy - Ay Cx, W = Bx Ay - By Ax, each recomputed
    in FP64 (exact products of f32 values, one rounding) when one of them is 0;
  - a miss when the signs differ; det = (U + V) + W, a miss when 0;
  - T = ((U Sz A_kz) + (V Sz B_kz)) + (W Sz C_kz), t = T / det, a hit when
    t > 1e-5 (the reference's minimum, crates/omg-core/src/mesh.rs:455).
The closest hit is the near-tie rule of the tracer (device_common.cuh:
TieState): the nearest hit t_min sets the window t_min * (1 + 1e-6) (both in
f32), and the winner among the hits inside it has the lowest (surface id,
triangle id, t).
"""
from __future__ import annotations

import numpy as np

F = np.float32
TIE_WINDOW = F(F(1.0) + F(1e-6))
T_MIN = F(1e-5)


def _pick(v, k):
    """v[..., k] per row: v (n, 3), k (n,)."""
    return np.take_along_axis(v, k[:, None], axis=1)[:, 0]


def ray_frames(d):
    """Per ray: kx, ky, kz and the shear (Sx, Sy, Sz). d (n, 3) float32."""
    d = np.asarray(d, F)
    a = np.abs(d)
    kz = np.where(a[:, 1] > a[:, 0], 1, 0)
    kz = np.where(a[:, 2] > np.where(kz == 0, a[:, 0], a[:, 1]), 2, kz)
    kx = np.where(kz == 2, 0, kz + 1)
    ky = np.where(kx == 2, 0, kx + 1)
    dkz = _pick(d, kz)
    neg = dkz < 0
    kx, ky = np.where(neg, ky, kx), np.where(neg, kx, ky)
    with np.errstate(divide="ignore", invalid="ignore"):
        sx = (_pick(d, kx) / dkz).astype(F)
        sy = (_pick(d, ky) / dkz).astype(F)
        sz = (F(1.0) / dkz).astype(F)
    return kx, ky, kz, sx, sy, sz


def intersect(o, d, A, B, C):
    """Watertight test of every ray against every triangle.
    o, d: (n, 3); A, B, C: (m, 3). Returns (hit (n, m) bool, t (n, m) float32)."""
    o = np.asarray(o, F)
    d = np.asarray(d, F)
    kx, ky, kz, sx, sy, sz = ray_frames(d)
    n = len(o)

    def sheared(V):
        v = (np.asarray(V, F)[None, :, :] - o[:, None, :]).astype(F)       # (n, m, 3)
        vkx = np.take_along_axis(v, kx[:, None, None].repeat(v.shape[1], 1), axis=2)[:, :, 0]
        vky = np.take_along_axis(v, ky[:, None, None].repeat(v.shape[1], 1), axis=2)[:, :, 0]
        vkz = np.take_along_axis(v, kz[:, None, None].repeat(v.shape[1], 1), axis=2)[:, :, 0]
        X = (vkx - (sx[:, None] * vkz).astype(F)).astype(F)
        Y = (vky - (sy[:, None] * vkz).astype(F)).astype(F)
        return X, Y, vkz

    Ax, Ay, Az = sheared(A)
    Bx, By, Bz = sheared(B)
    Cx, Cy, Cz = sheared(C)
    U = ((Cx * By).astype(F) - (Cy * Bx).astype(F)).astype(F)
    V = ((Ax * Cy).astype(F) - (Ay * Cx).astype(F)).astype(F)
    W = ((Bx * Ay).astype(F) - (By * Ax).astype(F)).astype(F)
    redo = (U == 0) | (V == 0) | (W == 0)
    if redo.any():
        D = np.float64
        U64 = (Cx.astype(D) * By.astype(D) - Cy.astype(D) * Bx.astype(D)).astype(F)
        V64 = (Ax.astype(D) * Cy.astype(D) - Ay.astype(D) * Cx.astype(D)).astype(F)
        W64 = (Bx.astype(D) * Ay.astype(D) - By.astype(D) * Ax.astype(D)).astype(F)
        U = np.where(redo, U64, U)
        V = np.where(redo, V64, V)
        W = np.where(redo, W64, W)
    mixed = ((U < 0) | (V < 0) | (W < 0)) & ((U > 0) | (V > 0) | (W > 0))
    det = ((U + V).astype(F) + W).astype(F)
    szc = sz[:, None]
    T = (((U * (szc * Az).astype(F)).astype(F) + (V * (szc * Bz).astype(F)).astype(F)).astype(F)
         + (W * (szc * Cz).astype(F)).astype(F)).astype(F)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = (T / det).astype(F)
    hit = ~mixed & (det != 0) & (t > T_MIN)
    return hit, np.where(hit, t, F(np.inf)).astype(F)


def closest(o, d, A, B, C, tri_id, surface=None, chunk=512):
    """Near-tie closest hit of every ray over the triangles: (t, tri id) with
    t = inf and id 0xFFFFFFFF for a miss."""
    m = len(A)
    surface = np.zeros(m, np.uint32) if surface is None else np.asarray(surface, np.uint32)
    tri_id = np.asarray(tri_id, np.uint32)
    t_out = np.full(len(o), np.inf, F)
    id_out = np.full(len(o), 0xFFFFFFFF, np.uint32)
    for c0 in range(0, len(o), chunk):
        hit, t = intersect(o[c0:c0 + chunk], d[c0:c0 + chunk], A, B, C)
        tmin = t.min(axis=1)
        win = (tmin * TIE_WINDOW).astype(F)
        inwin = hit & (t <= win[:, None])
        for r in np.nonzero(inwin.any(axis=1))[0]:
            cand = np.nonzero(inwin[r])[0]
            order = np.lexsort((t[r, cand], tri_id[cand], surface[cand]))
            best = cand[order[0]]
            t_out[c0 + r] = t[r, best]
            id_out[c0 + r] = tri_id[best]
    return t_out, id_out
