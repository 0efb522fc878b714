"""The C-ABI library loads and exports every symbol include/omg_cuda.h
declares (no compute calls: these run without a GPU)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "omg_cuda.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(omg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_lib):
    names = declared_symbols()
    assert len(names) >= 40
    for n in names:
        assert hasattr(built_lib, n), n


def test_bindings_cover_the_header(built_lib):
    from omg_audio_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES), set(declared_symbols()) ^ set(_lib.SIGNATURES)


def test_abi_version_and_status_strings(built_lib):
    from omg_audio_gb300 import _lib
    assert built_lib.omg_abi_version() == 3
    assert _lib.status_string(0) == "ok"
    assert _lib.status_string(_lib.E_TIMEOUT) == "timeout"


def test_params_default_are_reference_constants(built_lib):
    """tracer.rs:12-16, 103, 163; lib.rs:18-22."""
    from omg_audio_gb300 import _lib
    p = _lib.omg_params()
    built_lib.omg_params_default(C.byref(p))
    assert (p.n_bands, p.n_bins, p.max_bounces, p.dir_band) == (3, 300, 64, 1)
    assert abs(p.bin_dt - 0.010) < 1e-9 and abs(p.max_time - 3.0) < 1e-9
    assert abs(p.energy_floor - 1e-7) < 1e-12 and abs(p.receiver_radius - 0.5) < 1e-9
    assert abs(p.wall_eps - 1e-3) < 1e-9 and abs(p.speed_of_sound - 343.0) < 1e-6


def test_struct_sizes_match_the_header(built_lib):
    from omg_audio_gb300 import _lib
    assert C.sizeof(_lib.omg_material) == 68
    assert C.sizeof(_lib.omg_params) == 16 * 4
    assert C.sizeof(_lib.omg_panel) == 24 + 68
    assert C.sizeof(_lib.omg_reverb) == 3 * 32 + 8
    assert C.sizeof(_lib.omg_late_state) == 2 * 32 + 16 + 8
    assert C.sizeof(_lib.omg_dome_bin) == 11 * 4


def test_dome_bins_read_as_arrays(built_lib):
    """DomeProbe reads omg_dome_bin records as one float view: same values as field by field."""
    import numpy as np
    from omg_audio_gb300 import _lib
    from omg_audio_gb300.engine import DomeProbe
    n_eyes, nb = 3, 5
    out = (_lib.omg_dome_bin * (9 * n_eyes))()
    for i in range(9 * n_eyes):
        out[i].dir[:] = [i, i + 0.25, i + 0.5]
        out[i].energy[:] = [100 * i + b for b in range(8)]
    probe = DomeProbe.__new__(DomeProbe)
    probe.nb = nb
    probe.ctx = type("Ctx", (), {"h": None})()     # no context: the segment query is refused, counts stay 0
    probe.id = 0
    r = probe._result(out, n_eyes, None, None, None)
    for e in range(n_eyes):
        for k in range(9):
            assert np.array_equal(r["energy"][e, k], np.float32(out[e * 9 + k].energy[:nb]))
            assert np.array_equal(r["dir"][e, k], np.float32(out[e * 9 + k].dir[:]))
    assert r["energy"].shape == (n_eyes, 9, nb) and r["energy"].flags.owndata


def test_mesh_builder_matches_oracle_on_cpu(built_lib, oracle):
    """MeshBuilder dedup/surfaces/limits (host code, no GPU) equal the oracle's."""
    import numpy as np
    from omg_audio_gb300 import MeshBuilder
    from omg_audio_gb300 import workloads as W
    from test_oracle_golden import omat
    for case in (W.shoebox12(seed=1).recorder, W.multiroom(seed=2).recorder):
        mb = MeshBuilder()
        case.replay(mb)
        ob = oracle.MeshBuilder()
        case.replay(ob, lambda m: omat(oracle, m))
        a, b = mb.export(), ob.export()
        for k in a:
            assert np.array_equal(a[k], b[k]), k


def test_no_context_without_a_device(built_lib):
    """omg_create returns NULL (the caller keeps its CPU path) when no device exists."""
    import torch
    if torch.cuda.is_available():
        return
    from omg_audio_gb300 import _lib
    p = _lib.omg_params()
    built_lib.omg_params_default(C.byref(p))
    assert not built_lib.omg_create(C.byref(p))
