"""ctypes binding of libwoxel_gb300.so (declarations mirror include/woxel_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# WOXEL_GB300_BOUNDS_CHECK=1 loads the bounds-checked build instead (see wx_bounds_violations).
LIB_PATH = Path(__file__).resolve().parent / (
    "libwoxel_gb300_checked.so" if os.environ.get("WOXEL_GB300_BOUNDS_CHECK") == "1" else "libwoxel_gb300.so")

WX_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "unsupported",
          5: "over memory budget", 6: "timed out", 7: "cancelled"}


class wx_state_uniform(C.Structure):
    _fields_ = [("view_projection", C.c_float * 16), ("camera_to_world", C.c_float * 16),
                ("eye", C.c_float * 4), ("u", C.c_float * 4), ("mv", C.c_float * 4), ("wp", C.c_float * 4),
                ("render_mode", C.c_uint32 * 4), ("show_345", C.c_uint32 * 4),
                ("sun_dir", C.c_float * 4), ("sun_color", C.c_float * 4)]


class wx_hit(C.Structure):
    _fields_ = [("p", C.c_float * 3), ("t", C.c_float), ("node", C.c_uint32), ("info", C.c_uint32),
                ("shadow", C.c_uint32), ("reserved", C.c_uint32)]


class wx_vdb345_view(C.Structure):
    _fields_ = [("kids5", C.c_void_p), ("vals5", C.c_void_p), ("kids4", C.c_void_p), ("vals4", C.c_void_p),
                ("vals3", C.c_void_p), ("origins", C.c_void_p), ("n5", C.c_uint64), ("n4", C.c_uint64),
                ("n3", C.c_uint64), ("origin_stride", C.c_uint32), ("atlas", C.c_void_p * 3),
                ("dims", (C.c_uint32 * 3) * 3)]


class wx_grid_info(C.Structure):
    _fields_ = [("n5", C.c_uint64), ("n4", C.c_uint64), ("n3", C.c_uint64), ("device_bytes", C.c_uint64),
                ("active_voxels", C.c_uint64)]


class wx_tuning(C.Structure):
    _fields_ = [("kernel", C.c_int32), ("warps_per_block", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("tile_width", C.c_int32), ("tile_order", C.c_int32), ("rays_per_lane", C.c_int32)]


class wx_frame(C.Structure):
    _fields_ = [("grid", C.c_void_p), ("state", wx_state_uniform), ("width", C.c_uint32), ("height", C.c_uint32),
                ("rgba8", C.c_void_p), ("hits", C.c_void_p)]


class wx_server_config(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("max_inflight", C.c_uint32), ("slice_tiles", C.c_uint32),
                ("max_frames", C.c_uint32), ("flags", C.c_uint32)]


class wx_request(C.Structure):
    _fields_ = [("grid_id", C.c_uint32), ("want_hits", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("state", wx_state_uniform), ("user", C.c_uint64)]


class wx_result(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("user", C.c_uint64), ("status", C.c_int32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("rgba8", C.c_void_p), ("hits", C.c_void_p), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double)]


class wx_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("cancelled", C.c_uint64),
                ("launches", C.c_uint64), ("rays_done", C.c_uint64), ("arena_bytes", C.c_uint64),
                ("arena_in_use", C.c_uint64), ("arena_peak", C.c_uint64), ("pending", C.c_uint64),
                ("active", C.c_uint64), ("tiles_cancelled_queued", C.c_uint64),
                ("tiles_cancelled_launched", C.c_uint64)]


class wx_vdb_info(C.Structure):
    _fields_ = [("file_version", C.c_uint32), ("compression", C.c_uint32), ("half_float", C.c_uint32),
                ("reserved", C.c_uint32), ("file_voxel_count", C.c_int64), ("grid_name", C.c_char * 64)]


assert C.sizeof(wx_state_uniform) == 256
assert C.sizeof(wx_hit) == 32

P = C.c_void_p
U32, U64, I32, F32, INT = C.c_uint32, C.c_uint64, C.c_int32, C.c_float, C.c_int

# name -> (restype, argtypes); every symbol the header declares.
SIGNATURES = {
    "wx_status_string": (C.c_char_p, [INT]),
    "wx_thread_last_error": (C.c_char_p, []),
    "wx_version": (C.c_char_p, []),
    "wx_ctx_create": (INT, [INT, C.POINTER(P)]),
    "wx_ctx_destroy": (INT, [P]),
    "wx_last_error": (C.c_char_p, [P]),
    "wx_grid_upload": (INT, [P, C.POINTER(wx_vdb345_view), C.POINTER(P)]),
    "wx_grid_build": (INT, [P, P, C.POINTER(P)]),
    "wx_grid_build_gpu": (INT, [P, P, C.POINTER(P)]),
    "wx_grid_read_pools": (INT, [P, P, P, P, P, P, C.POINTER(C.c_uint64)]),
    "wx_grid_release": (INT, [P, P]),
    "wx_grid_set_values": (INT, [P, P, P, F32]),
    "wx_grid_get_info": (INT, [P, C.POINTER(wx_grid_info)]),
    "wx_render": (INT, [P, P, C.POINTER(wx_state_uniform), U32, U32, P, P, P]),
    "wx_ctx_set_tuning": (INT, [P, C.POINTER(wx_tuning)]),
    "wx_ctx_get_tuning": (INT, [P, C.POINTER(wx_tuning)]),
    "wx_ctx_set_sdf_wait_limit": (INT, [P, C.c_uint32]),
    "wx_inject_alloc_failures": (INT, [C.c_uint32]),
    "wx_render_batch": (INT, [P, C.POINTER(wx_frame), U32, P]),
    "wx_batch_create": (INT, [P, C.POINTER(wx_frame), U32, C.POINTER(P)]),
    "wx_batch_launch": (INT, [P, P]),
    "wx_batch_info": (INT, [P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U64)]),
    "wx_batch_destroy": (INT, [P]),
    "wx_render_batch_noalloc": (INT, [C.POINTER(wx_frame), U32, P]),
    "wx_server_create": (INT, [P, C.POINTER(wx_server_config), C.POINTER(P)]),
    "wx_server_add_grid": (INT, [P, P, C.POINTER(U32)]),
    "wx_server_submit": (INT, [P, C.POINTER(wx_request), C.POINTER(U64)]),
    "wx_server_cancel": (INT, [P, U64]),
    "wx_server_poll": (INT, [P, C.POINTER(wx_result), U32, C.POINTER(U32), INT]),
    "wx_server_release": (INT, [P, U64]),
    "wx_server_copy_result": (INT, [P, U64, P, P]),
    "wx_server_get_stats": (INT, [P, C.POINTER(wx_server_stats)]),
    "wx_server_replay": (INT, [P, C.POINTER(wx_request), C.POINTER(C.c_double), U32, C.POINTER(wx_result), INT,
                               C.c_double]),
    "wx_server_destroy": (INT, [P]),
    "wx_check_division": (INT, [P, U32, C.POINTER(U64)]),
    "wx_bounds_violations": (INT, [P, C.POINTER(U64)]),
    "wx_autotune": (INT, [P, C.POINTER(wx_frame), U32, C.POINTER(wx_tuning), U32, U32, C.POINTER(wx_tuning),
                          C.POINTER(C.c_double)]),
    "wx_state_build": (INT, [P, P, P, F32, F32, F32, U32, P, P, P, F32, C.POINTER(wx_state_uniform)]),
    "wx_sun_default": (None, [P, P, P]),
    "wx_topology_from_masks": (INT, [P, P, U64, P, P, U64, P, U64, P, U32, C.POINTER(P)]),
    "wx_topology_from_voxels": (INT, [P, U64, C.POINTER(P)]),
    "wx_topology_from_leaves": (INT, [P, P, U64, C.POINTER(P)]),
    "wx_topology_free": (None, [P]),
    "wx_topology_counts": (INT, [P, P]),
    "wx_topology_active_voxels": (U64, [P]),
    "wx_topology_masks": (INT, [P, P, P, P, P, P, P]),
    "wx_topology_sdf": (INT, [P, INT]),
    "wx_topology_atlas": (INT, [P, P, P, P, P, U32]),
    "wx_gen_sphere": (INT, [F32, F32, F32, F32, F32, C.POINTER(P)]),
    "wx_gen_spheres": (INT, [U32, F32, F32, F32, F32, F32, U64, C.POINTER(P)]),
    "wx_gen_sphere_values": (INT, [P, F32, F32, F32, F32, F32, P]),
    "wx_gen_spheres_values": (INT, [P, U32, F32, F32, F32, F32, F32, U64, P]),
    "wx_gen_noise_leaves": (INT, [I32, U32, C.c_double, C.c_double, U64, INT, C.POINTER(P)]),
    "wx_orbit_eyes": (INT, [U32, F32, U64, P]),
    "wx_vdb_read_topology": (INT, [C.c_char_p, C.c_char_p, C.POINTER(P), C.POINTER(wx_vdb_info)]),
    "wx_vdb_read_leaf_values": (INT, [C.c_char_p, C.c_char_p, P, U64, C.POINTER(C.c_uint64), C.POINTER(F32)]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libwoxel_gb300.so; raises if it has not been built (no fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m woxel_gb300.build` (there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class WxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status != WX_OK:
        L = lib()
        msg = (L.wx_last_error(ctx) if ctx else L.wx_thread_last_error()) or b""
        raise WxError(status, msg.decode(errors="replace"))
