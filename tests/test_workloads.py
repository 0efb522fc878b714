"""The benchmark's synthetic workloads (omg_audio_gb300/workloads.py) keep the
sizes the bench line and the documents quote, on the CPU, counted by the
oracle's MeshBuilder and tessellation (mesh.rs:70-287):
  - the 40-room scene: 994 authored triangles, 49,242 primitives, 64 pairs,
    22 pane panels;
  - the 256-room batch: 1,425,732 rays, 803,868 primitives, 3 or 8 bands;
  - the city: 1,033,380 triangles, 1,941,396 primitives, 16 sources and
    listeners.
The generators are seeded: the same seed gives the same scene."""
import numpy as np

from omg_audio_gb300 import workloads as W
from oracle import oracle as O


def _mk(m):
    return O.Material.make(m.absorption, m.scattering, m.transmission)


def _mesh(rec):
    mb = O.MeshBuilder()
    rec.replay(mb, _mk)
    return mb


def test_multiroom_sizes():
    case = W.multiroom(seed=2, n_pairs=64)
    info = _mesh(case.recorder).build("f32").info()
    assert (info["tris"], info["prims"]) == (994, 49242)
    assert len(case.pairs) == 64 and len(case.panels) == 22
    again = W.multiroom(seed=2, n_pairs=64)
    assert np.array_equal(np.asarray(case.pairs, float), np.asarray(again.pairs, float))


def test_room_batch_sizes():
    rooms = W.room_batch(seed=3, n_rooms=256)
    assert len(rooms) == 256
    assert sum(r.n_rays for r in rooms) == 1425732
    assert {r.n_bands for r in rooms} == {3, 8}
    assert sum(_mesh(r.recorder).build("f32").info()["prims"] for r in rooms) == 803868


def test_city_sizes():
    case = W.city(seed=5)
    assert case.recorder.n_tris == 1033380
    assert len(case.sources) == 16 and len(case.listeners) == 16 and case.n_bands == 8
    assert _mesh(case.recorder).build("f32").info()["prims"] == 1941396
