"""Per-band surface materials (crates/omg-core/src/material.rs).

The preset values are the reference's published material table
(material.rs:18-56) and pane/leaf constants (crates/omg-scene/src/
walkthrough.rs:310-326); they are data the tracer's results depend on, so
they are kept identical.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Sequence

from . import _lib

REF_THICKNESS_M = 0.15  # material.rs:23


@dataclass(frozen=True)
class Material:
    """absorption: energy fraction lost per reflection, per band;
    scattering: diffuse fraction of the reflected energy;
    transmission: AMPLITUDE through a 15 cm wall, per band (energy = T^2)."""
    absorption: tuple
    scattering: float
    transmission: tuple = field(default=(0.0, 0.0, 0.0))

    def transmission_at(self, thickness_m: float) -> tuple:
        """Mass-law thickness scaling (material.rs:59-62), f32 arithmetic."""
        import numpy as np
        f = np.float32
        k = min(f(REF_THICKNESS_M) / max(f(thickness_m), f(0.02)), f(2.0))
        return tuple(float(min(f(t) * k, f(0.9))) for t in self.transmission)

    def with_transmission(self, t: Sequence[float]) -> "Material":
        return Material(tuple(self.absorption), self.scattering, tuple(t))

    def to_c(self) -> _lib.omg_material:
        m = _lib.omg_material()
        for i, v in enumerate(self.absorption):
            m.absorption[i] = v
        m.scattering = self.scattering
        for i, v in enumerate(self.transmission):
            m.transmission[i] = v
        return m

    @property
    def n_bands(self) -> int:
        return len(self.absorption)


CONCRETE = Material((0.01, 0.02, 0.04), 0.10, (0.10, 0.014, 0.0015))
DRYWALL = Material((0.20, 0.08, 0.05), 0.10, (0.20, 0.045, 0.0150))
CARPET = Material((0.05, 0.30, 0.60), 0.40, (0.30, 0.100, 0.0300))
WOOD_PANEL = Material((0.20, 0.10, 0.08), 0.15, (0.22, 0.060, 0.0200))
ACOUSTIC_TILE = Material((0.30, 0.70, 0.80), 0.30, (0.30, 0.100, 0.0300))
BRICK = Material((0.02, 0.03, 0.04), 0.12, (0.045, 0.008, 0.0012))
GRASS = Material((0.11, 0.26, 0.60), 0.50, (0.10, 0.020, 0.0050))
# walkthrough.rs:19-23 (the cathedral's stone)
ORNATE_STONE = Material((0.015, 0.03, 0.06), 0.35, (0.10, 0.014, 0.0015))

PRESETS = {
    "CONCRETE": CONCRETE, "DRYWALL": DRYWALL, "CARPET": CARPET, "WOOD_PANEL": WOOD_PANEL,
    "ACOUSTIC_TILE": ACOUSTIC_TILE, "BRICK": BRICK, "GRASS": GRASS, "ORNATE_STONE": ORNATE_STONE,
}

# walkthrough.rs:310-326: pane and leaf AMPLITUDE transmissions per band
GLASS_TRANSMISSION = (0.50, 0.32, 0.20)
HEAVY_GLASS_TRANSMISSION = (0.18, 0.05, 0.012)
DOOR_PANEL_TRANSMISSION = (0.28, 0.12, 0.05)
HEAVY_PANEL_TRANSMISSION = (0.10, 0.03, 0.01)


def glass_transmission(heavy: bool) -> tuple:
    return HEAVY_GLASS_TRANSMISSION if heavy else GLASS_TRANSMISSION
