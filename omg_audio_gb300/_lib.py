"""ctypes bindings of libomg_cuda.so (include/omg_cuda.h).

The library is built in-tree by omg_audio_gb300.build. Loading fails loudly
when it is missing: there is no CPU path behind these bindings.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libomg_cuda.so")

MAX_BANDS = 8
DOME_BINS = 9

OK, PENDING = 0, 1
E_INVALID, E_OOM, E_DEVICE, E_TIMEOUT, E_OVERFLOW, E_NOT_FOUND, E_NO_DEVICE = -1, -2, -3, -4, -5, -6, -7
BVH_SAH, BVH_LBVH, BVH_SAH3, BVH_SAH3_HOST = 0, 1, 2, 3
GEOM_BOX, GEOM_MESH = 0, 1

F8 = C.c_float * MAX_BANDS
F3 = C.c_float * 3


class omg_material(C.Structure):
    _fields_ = [("absorption", F8), ("scattering", C.c_float), ("transmission", F8)]


class omg_params(C.Structure):
    _fields_ = [("n_bands", C.c_uint32), ("n_bins", C.c_uint32), ("bin_dt", C.c_float), ("max_time", C.c_float),
                ("max_bounces", C.c_uint32), ("energy_floor", C.c_float), ("receiver_radius", C.c_float),
                ("wall_eps", C.c_float), ("speed_of_sound", C.c_float), ("dir_band", C.c_uint32),
                ("device", C.c_int32), ("timeout_ms", C.c_uint32), ("tie_mode", C.c_uint32),
                ("walk_budget", C.c_uint32), ("loop_guard", C.c_uint32), ("tri_test", C.c_uint32)]


class omg_box_job(C.Structure):
    _fields_ = [("size", F3), ("walls", omg_material * 6), ("src", F3), ("lis", F3), ("n_rays", C.c_uint32),
                ("energy", F8), ("seed", C.c_uint32)]


class omg_panel(C.Structure):
    _fields_ = [("mn", F3), ("mx", F3), ("material", omg_material)]


class omg_world_job(C.Structure):
    _fields_ = [("src", F3), ("lis", F3), ("n_rays", C.c_uint32), ("energy", F8), ("seed", C.c_uint32)]


class omg_job(C.Structure):
    _fields_ = [("geom", C.c_uint32), ("scene_id", C.c_uint32), ("box_size", F3), ("box_walls", omg_material * 6),
                ("src", F3), ("lis", F3), ("n_rays", C.c_uint32), ("energy", F8), ("seed", C.c_uint32),
                ("n_bands", C.c_uint32), ("n_bins", C.c_uint32), ("max_time", C.c_float),
                ("panel_offset", C.c_uint32), ("n_panels", C.c_uint32)]


class omg_reverb(C.Structure):
    _fields_ = [("rt60", F8), ("level", F8), ("rt60_fit", F8), ("segments", C.c_uint64)]


class omg_late_state(C.Structure):
    _fields_ = [("rt60", F8), ("level", F8), ("dir", C.c_float * 3), ("anisotropy", C.c_float),
                ("version", C.c_uint32), ("updated_tick", C.c_uint32)]


class omg_dome_panel(C.Structure):
    _fields_ = [("axis", C.c_int32), ("plane", C.c_float), ("lat0", C.c_float), ("lat1", C.c_float),
                ("z0", C.c_float), ("z1", C.c_float), ("glass", C.c_int32), ("trans", F8)]


class omg_dome_bin(C.Structure):
    _fields_ = [("dir", F3), ("energy", F8)]


class omg_tune_result(C.Structure):
    _fields_ = [("block_threads", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("refill_min", C.c_uint32),
                ("walk_steps", C.c_uint32), ("shade_min", C.c_uint32), ("mode", C.c_uint32), ("tail_mode", C.c_uint32), ("wide", C.c_uint32), ("wf_rounds", C.c_uint32), ("wf_tail", C.c_uint32),
                ("epochs", C.c_uint32), ("park_pct", C.c_uint32), ("wl_shade_min", C.c_uint32),
                ("ms", C.c_float)]


class omg_chain(C.Structure):
    _fields_ = [("surf", C.c_uint16 * 3), ("order", C.c_uint16)]


class omg_aabb(C.Structure):
    _fields_ = [("mn", F3), ("mx", F3), ("transmission", F3)]


class omg_mesh_record(C.Structure):
    _fields_ = [("source", C.c_uint16), ("chain", C.c_uint16 * 3), ("order", C.c_uint32), ("delay_s", C.c_float),
                ("dir", F3), ("gains", F3), ("key", C.c_uint32), ("valid", C.c_uint32)]


class omg_tap(C.Structure):
    _fields_ = [("key", C.c_uint32), ("delay_s", C.c_float), ("dir", F3), ("gains", F3)]


class omg_param_block(C.Structure):
    _fields_ = [("version", C.c_uint64), ("rt60", F3), ("level", F3), ("has_remote", C.c_int32),
                ("remote_rt60", F3), ("remote_send", F3), ("remote_sh", C.c_float * 9)]


class omg_mlp_config(C.Structure):
    _fields_ = [("n_in", C.c_uint32), ("hidden", C.c_uint32), ("n_hidden", C.c_uint32), ("n_out", C.c_uint32),
                ("members", C.c_uint32), ("seed", C.c_uint32)]


class omg_mlp_train_config(C.Structure):
    _fields_ = [("epochs", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_float), ("lr_final", C.c_float),
                ("weight_decay", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("seed", C.c_uint32)]


P, U32, U64, I32, F = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32, C.c_float
PU32, PU64 = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)

# name -> (restype, argtypes); every symbol include/omg_cuda.h declares
SIGNATURES = {
    "omg_params_default": (None, [C.POINTER(omg_params)]),
    "omg_create": (P, [C.POINTER(omg_params)]),
    "omg_destroy": (None, [P]),
    "omg_abi_version": (I32, []),
    "omg_status_string": (C.c_char_p, [I32]),
    "omg_last_error": (C.c_char_p, [P]),
    "omg_last_flags": (U32, [P]),
    "omg_set_limits": (I32, [P, U32, U32]),
    "omg_set_stream": (I32, [P, P]),
    "omg_mb_create": (P, []),
    "omg_mb_destroy": (None, [P]),
    "omg_mb_material": (U32, [P, C.POINTER(omg_material)]),
    "omg_mb_begin_surface": (U32, [P]),
    "omg_mb_coarse": (None, [P, F]),
    "omg_mb_tri": (None, [P, P, P, P, U32]),
    "omg_mb_quad": (None, [P, P, P, P, P, U32]),
    "omg_mb_abox": (None, [P, P, P, U32]),
    "omg_mb_quads": (None, [P, P, P, P, P, U32]),
    "omg_mb_counts": (None, [P, PU32, PU32, PU32]),
    "omg_mb_export": (None, [P, P, P, P, P, P]),
    "omg_scene_upload": (I32, [P, P, U32, P, U32, P, P, P, U32, U32, U32, PU32]),
    "omg_scene_from_builder": (I32, [P, P, U32, U32, PU32]),
    "omg_scene_release": (I32, [P, U32]),
    "omg_scene_info": (I32, [P, U32, PU32, PU32, PU32]),
    "omg_scene_export_bvh": (I32, [P, U32, P, P, P, P, P]),
    "omg_trace_box": (I32, [P, C.POINTER(omg_box_job), P, P, P]),
    "omg_trace_world": (I32, [P, U32, C.POINTER(omg_world_job), P, U32, P, P, P]),
    "omg_trace_batch": (I32, [P, P, U32, P, U32, P, P, P]),
    "omg_batch_create": (I32, [P, P, U32, P, U32, PU32]),
    "omg_batch_launch": (I32, [P, U32]),
    "omg_batch_launch_part": (I32, [P, U32, U32]),
    "omg_io_bytes": (I32, [P, PU64, PU64]),
    "omg_batch_read": (I32, [P, U32, P, P, P]),
    "omg_batch_sizes": (I32, [P, U32, PU64, PU64]),
    "omg_batch_segments": (I32, [P, U32, PU64]),
    "omg_batch_destroy": (I32, [P, U32]),
    "omg_batch_kernel_count": (I32, [P, U32, PU32]),
    "omg_submit_world": (I32, [P, U32, C.POINTER(omg_world_job), P, U32, PU32]),
    "omg_poll": (I32, [P, U32, P, P, P]),
    "omg_batch_autotune": (I32, [P, U32, U32, C.POINTER(omg_tune_result)]),
    "omg_batch_set_shape": (I32, [P, U32, C.POINTER(omg_tune_result)]),
    "omg_batch_get_shape": (I32, [P, U32, C.POINTER(omg_tune_result)]),
    "omg_raycast": (I32, [P, U32, P, P, U32, P, P]),
    "omg_estimate_reverb": (I32, [P, P, U32, U32, F, U32, P]),
    "omg_dome_create": (I32, [P, U32, P, U32, U32, U32, PU32]),
    "omg_dome_destroy": (I32, [P, U32]),
    "omg_dome_sample": (I32, [P, U32, P, U32, P, U32, U32, U32, P, P, P, P]),
    "omg_dome_submit": (I32, [P, U32, C.c_void_p, U32, C.c_void_p, U32, U32, U32, U32, C.c_void_p]),
    "omg_dome_collect": (I32, [P, U32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "omg_dome_segments": (I32, [P, U32, PU64, PU64]),
    "omg_late_create": (I32, [P, U32, F, PU32]),
    "omg_late_destroy": (I32, [P, U32]),
    "omg_late_submit": (I32, [P, U32, P, P, P, U32, P, U32, PU32]),
    "omg_late_poll": (I32, [P, U32, P, PU32]),
    "omg_late_reset": (I32, [P, U32, U32]),
    "omg_late_read": (I32, [P, U32, U32, P, P]),
    "omg_mlp_create": (I32, [P, C.POINTER(omg_mlp_config), PU32]),
    "omg_mlp_destroy": (I32, [P, U32]),
    "omg_mlp_set_data": (I32, [P, U32, P, P, U32]),
    "omg_mlp_train": (I32, [P, U32, C.POINTER(omg_mlp_train_config), P]),
    "omg_surrogate_predict": (I32, [P, U32, P, U32, P, P]),
    "omg_surrogate_query": (I32, [P, U32, P, U32, P, P, F]),
    "omg_mlp_grad": (I32, [P, U32, U32, P, P, U32, P, P]),
    "omg_mlp_params": (I32, [P, U32, U32, P, PU64]),
    "omg_mlp_set_params": (I32, [P, U32, U32, P, U64]),
    "omg_tc_gemm": (I32, [P, P, P, P, U32, U32, U32]),
    "omg_tc_gemm_bench": (I32, [P, U32, U32, U32, U32, U32, C.POINTER(C.c_float)]),
    "omg_trace_box_noalloc": (I32, [C.POINTER(omg_box_job), C.POINTER(omg_params), P, P, P, P]),
    "omg_early_create": (I32, [P, U32, P, U32, PU32]),
    "omg_early_destroy": (I32, [P, U32]),
    "omg_early_info": (I32, [P, U32, PU32, PU32]),
    "omg_early_discover": (I32, [P, U32, P, U32, U32, I32, P, U32, PU32]),
    "omg_early_solve": (I32, [P, U32, P, P, U32, P, U32, P, P, U32, P]),
    "omg_trace_web_box_jobs": (I32, [P, P, U32, P, P, P]),
    "omg_trace_web_world_jobs": (I32, [P, U32, P, U32, P, P, P]),
    "omg_param_block_flat_len": (U32, [U32]),
    "omg_param_block_write_flat": (I32, [C.POINTER(omg_param_block), P, U32, P, U32]),
    "omg_param_block_read_flat": (I32, [P, U32, C.POINTER(omg_param_block), P, U32, PU32]),
    "omg_param_block_from_late": (I32, [P, U32, P]),
}

NOALLOC_MAX_CELLS = 45056
WEB_BOX_JOB_F32S, WEB_BOX_JOB_VERSION = 57, 2
WEB_WORLD_MAX_PANELS, WEB_WORLD_JOB_VERSION = 64, 3
WEB_WORLD_JOB_F32S = 10 + WEB_WORLD_MAX_PANELS * 16
PARAM_FLAT_HEADER, PARAM_FLAT_PER_TAP = 24, 9
CHAIN_MAX_ORDER, NO_SURF = 3, 0xFFFF

_lib = None


class OmgError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({status})" if what else status_string(status))


def lib() -> C.CDLL:
    """Load libomg_cuda.so; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with omg_audio_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(s: int) -> str:
    return lib().omg_status_string(s).decode()


def check(status: int, what: str = ""):
    if status < 0:
        raise OmgError(status, what)
    return status
