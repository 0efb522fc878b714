"""omg_trace_box_noalloc against omg_trace_box.

The no-alloc entry point serves callers that must not allocate device memory
(a real-time audio thread, or code running while another component owns the
allocator): its scratch lives in a fixed device array. Here it is called
through the C ABI twice in a row, on device buffers this test owns, and each
result must match the allocating entry point's on the same job within the
tolerance the parity tests use (per-bin relative error <= 1e-5 on bins holding
>= 1e-6 of the band total), and its flag word must read 0 (the trace ran to its
end). The second call checks that the shared scratch is cleared between calls.
Jobs beyond the fixed scratch, and jobs with non-finite geometry or materials,
are rejected before anything is launched. This file is collected last on
purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b, frac=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    tot = np.maximum(b.sum(axis=0, keepdims=True), 1e-300)
    m = b >= frac * tot
    return float(np.max(np.abs(a[m] - b[m]) / b[m])) if m.any() else 0.0


def test_noalloc_matches_the_allocating_entry_point_twice(built_lib):
    import torch
    from omg_audio_gb300 import Context, TraceConfig, _lib
    from omg_audio_gb300 import materials as M

    torch.cuda.set_device(0)
    cfg = TraceConfig(n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200, energy_floor=1e-6)
    prm = cfg.to_c()
    walls = [M.CONCRETE] * 4 + [M.WOOD_PANEL, M.CONCRETE]
    size, src, lis = (6.0, 4.0, 3.0), (1.5, 1.0, 1.5), (4.5, 3.0, 1.6)
    n_bins, nb = cfg.n_bins, cfg.n_bands
    assert n_bins * (nb + 3) <= _lib.NOALLOC_MAX_CELLS
    bins_dev = torch.empty(n_bins * nb, dtype=torch.float32, device="cuda")
    dirs_dev = torch.empty(n_bins * 3, dtype=torch.float32, device="cuda")
    flags_dev = torch.empty(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    with Context(cfg) as ctx:
        for seed in (11, 12):
            ref, _ = ctx.trace_box(size, walls, src, lis, 4096, seed=seed)
            job = _lib.omg_box_job()
            for k in range(3):
                job.size[k], job.src[k], job.lis[k] = size[k], src[k], lis[k]
            for w in range(6):
                job.walls[w] = walls[w].to_c()
            job.n_rays = 4096
            for b in range(nb):
                job.energy[b] = 1.0
            job.seed = seed
            bins_dev.fill_(float("nan"))
            dirs_dev.fill_(float("nan"))
            flags_dev.fill_(-1)
            rc = built_lib.omg_trace_box_noalloc(C.byref(job), C.byref(prm), C.c_void_p(bins_dev.data_ptr()),
                                                 C.c_void_p(dirs_dev.data_ptr()), C.c_void_p(flags_dev.data_ptr()),
                                                 C.c_void_p(stream.cuda_stream))
            assert rc == 0, rc
            torch.cuda.synchronize()
            assert int(flags_dev.item()) == 0
            got_b = bins_dev.cpu().numpy().reshape(n_bins, nb)
            got_d = dirs_dev.cpu().numpy().reshape(n_bins, 3)
            assert np.isfinite(got_b).all() and np.isfinite(got_d).all()
            assert _rel(got_b, ref.bins) <= 1e-5, seed
            assert np.allclose(got_d, ref.dirs, rtol=1e-4, atol=1e-9), seed


def _job(M, _lib):
    job = _lib.omg_box_job()
    for k in range(3):
        job.size[k], job.src[k], job.lis[k] = 5.0, 1.0, 2.0
    for w in range(6):
        job.walls[w] = M.CONCRETE.to_c()
    job.n_rays = 64
    return job


def test_noalloc_rejects_sizes_beyond_its_scratch(built_lib):
    from omg_audio_gb300 import TraceConfig, _lib
    from omg_audio_gb300 import materials as M
    prm = TraceConfig(n_bins=6000, bin_dt=0.001, n_bands=8).to_c()
    rc = built_lib.omg_trace_box_noalloc(C.byref(_job(M, _lib)), C.byref(prm), C.c_void_p(1), C.c_void_p(1), None,
                                         None)
    assert rc == _lib.E_INVALID


@pytest.mark.parametrize("bad", ["src", "size", "absorption", "scattering"])
def test_noalloc_rejects_non_finite_jobs(built_lib, bad):
    """The checks omg_trace_box makes: NaN positions, sizes or material values
    never reach the kernel (the buffer pointers are never used)."""
    from omg_audio_gb300 import TraceConfig, _lib
    from omg_audio_gb300 import materials as M
    prm = TraceConfig().to_c()
    job = _job(M, _lib)
    if bad == "src":
        job.src[1] = float("nan")
    elif bad == "size":
        job.size[2] = float("inf")
    elif bad == "absorption":
        job.walls[3].absorption[0] = float("nan")
    else:
        job.walls[0].scattering = float("nan")
    rc = built_lib.omg_trace_box_noalloc(C.byref(job), C.byref(prm), C.c_void_p(1), C.c_void_p(1), None, None)
    assert rc == _lib.E_INVALID
