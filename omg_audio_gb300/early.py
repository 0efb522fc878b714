"""World early reflections over the C ABI (include/omg_cuda.h, "world early
reflections"): the surface table of an uploaded world mesh plus furniture
faces, chain discovery from the listener (the WorldDiscovery seam,
crates/omg-scene/src/early_world.rs:18-26; mesh_chains, pt_mesh.rs:382-457)
and the batched exact solve of every (source, chain) pair (the WorldSolve
seam, early_world.rs:36-48; mesh_record, pt_mesh.rs:186-337)."""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import lib
from .engine import panels_to_c

NO_SURF = _lib.NO_SURF
Chain = Tuple[Tuple[int, int, int], int]


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))


def chains_to_c(chains: Sequence[Chain]):
    arr = (_lib.omg_chain * max(1, len(chains)))()
    for i, (c, o) in enumerate(chains):
        for k in range(3):
            arr[i].surf[k] = c[k]
        arr[i].order = o
    return arr


class WorldEarly:
    """SurfaceTable::build + append_box over an uploaded scene (early_world.rs:114-120).
    furniture: (min, max, Material) triples; their faces reflect, and discovery
    rays bounce off the boxes."""

    def __init__(self, ctx, scene, furniture: Sequence = ()):
        self.ctx = ctx
        self.scene = scene
        pan = [(tuple(mn), tuple(mx), m) for (mn, mx, m) in furniture]
        arr = panels_to_c(pan)
        eid = C.c_uint32()
        ctx._check(lib().omg_early_create(ctx.h, scene.id, arr, len(pan), C.byref(eid)), "omg_early_create")
        self.id = eid.value
        b, n = C.c_uint32(), C.c_uint32()
        ctx._check(lib().omg_early_info(ctx.h, self.id, C.byref(b), C.byref(n)), "omg_early_info")
        self.base_overlay, self.n_surfaces = b.value, n.value

    def close(self):
        if getattr(self, "id", None) and self.ctx.h:
            lib().omg_early_destroy(self.ctx.h, self.id)
            self.id = None

    def __del__(self):
        self.close()

    def discover(self, listener, n_rays: int = 768, rot: int = 0, use_boxes: bool = True) -> List[Chain]:
        """mesh_chains: unique chains in the reference's first-found order."""
        cap = 3 * max(n_rays, 1)
        out = (_lib.omg_chain * cap)()
        n = C.c_uint32()
        self.ctx._check(lib().omg_early_discover(self.ctx.h, self.id, _p(_f3(listener)), n_rays, rot,
                                                 int(use_boxes), out, cap, C.byref(n)), "omg_early_discover")
        return [(tuple(int(v) for v in out[i].surf), int(out[i].order)) for i in range(min(n.value, cap))]

    def solve(self, sources: Sequence[Tuple[int, Sequence[float]]], chains: Sequence[Chain], listener,
              extras: Sequence = ()):
        """mesh_record for every (source, chain) pair: a structured array
        (n_sources, n_chains) with delay_s, dir, gains, key, valid.
        extras: (min, max, transmission3) blockers."""
        ns, nc = len(sources), len(chains)
        ids = np.array([s[0] for s in sources], np.uint16)
        pos = np.ascontiguousarray(np.array([s[1] for s in sources], np.float32).reshape(-1, 3))
        ex = (_lib.omg_aabb * max(1, len(extras)))()
        for i, (mn, mx, tr) in enumerate(extras):
            for k in range(3):
                ex[i].mn[k], ex[i].mx[k], ex[i].transmission[k] = mn[k], mx[k], tr[k]
        out = (_lib.omg_mesh_record * max(1, ns * nc))()
        self.ctx._check(lib().omg_early_solve(self.ctx.h, self.id, _p(ids), _p(pos), ns, chains_to_c(chains), nc,
                                              _p(_f3(listener)), ex, len(extras), out), "omg_early_solve")
        return np.ctypeslib.as_array(out)[:ns * nc].copy().reshape(ns, nc)
