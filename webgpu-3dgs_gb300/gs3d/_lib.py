"""ctypes binding of libgs3d.so, the C ABI declared in include/gs3d.h.

The library is the product path; there is no CPU fallback.  Loading fails
loudly when the shared library has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().with_name("libgs3d.so")

# status codes (gs3d.h)
OK = 0
ERR_INVALID_ARG = 1
ERR_OOM = 2
ERR_CAPACITY = 3
ERR_CUDA = 4
ERR_TIMEOUT = 5
ERR_STATE = 6
ERR_NO_DEVICE = 7
STATUS_NAMES = {
    OK: "GS3D_OK", ERR_INVALID_ARG: "GS3D_ERR_INVALID_ARG", ERR_OOM: "GS3D_ERR_OOM",
    ERR_CAPACITY: "GS3D_ERR_CAPACITY", ERR_CUDA: "GS3D_ERR_CUDA",
    ERR_TIMEOUT: "GS3D_ERR_TIMEOUT", ERR_STATE: "GS3D_ERR_STATE",
    ERR_NO_DEVICE: "GS3D_ERR_NO_DEVICE",
}

FLAG_STAGEWISE_REBIN = 1
FLAG_STAGE_TIMING = 2
FLAG_CUDA_GRAPH = 4
FLAG_SPLIT_ALL_TILES = 8
STAGE_NAMES = ["preprocess-splats", "depth-sort", "prefix-scan", "emit-tile-refs", "radix-sort",
               "identify-tile-ranges", "rasterize-tiles"]

# named buffers (gs3d.h, gs3d_buffer)
BUFFERS = {
    "splat_positions": 0, "splat_scales": 1, "splat_rotations": 2, "splat_colors": 3,
    "splat_sh_rest": 4, "projected_splats": 5, "splat_ref_counts": 6,
    "splat_ref_offsets": 7, "ref_counter": 8, "sort_keys_a": 9, "sort_values_a": 10,
    "sort_keys_b": 11, "sort_values_b": 12, "tile_offsets": 13, "splat_target": 14,
    "tile_costs": 15,
}


class Gs3dError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code
        self.message = message


class Camera_t(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("projection", C.c_float * 16),
                ("inverse_view", C.c_float * 16), ("inverse_projection", C.c_float * 16),
                ("position", C.c_float * 4), ("viewport", C.c_float * 4)]


class Config_t(C.Structure):
    _fields_ = [("device", C.c_int), ("tile_w", C.c_uint32), ("tile_h", C.c_uint32),
                ("max_tiles_per_splat", C.c_uint32), ("stream", C.c_void_p),
                ("flags", C.c_uint32)]


class View_t(C.Structure):
    _fields_ = [("camera", Camera_t), ("scene", C.c_uint32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("reserved", C.c_uint32)]


class Tuning_t(C.Structure):
    _fields_ = [("tile_w", C.c_uint32), ("tile_h", C.c_uint32), ("digit_bits", C.c_uint32),
                ("raster_batch", C.c_uint32)]


class TuneResult_t(C.Structure):
    _fields_ = [("tuning", Tuning_t), ("ms_per_view", C.c_float), ("tile_passes", C.c_uint32),
                ("refs", C.c_uint64)]


class PlyInfo_t(C.Structure):
    _fields_ = [("splat_count", C.c_uint64), ("header_bytes", C.c_uint64),
                ("format", C.c_uint32), ("f_rest_count", C.c_uint32),
                ("sh_degree", C.c_uint32), ("vertex_stride", C.c_uint32),
                ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3)]


PLY_NEW_SCENE = 0xFFFFFFFF
COMPOSITE_SPLATS = 0
COMPOSITE_TILE_HEATMAP = 1


class ViewInfo_t(C.Structure):
    _fields_ = [("pixel_offset", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32),
                ("tiles_x", C.c_uint32), ("tiles_y", C.c_uint32), ("tile_base", C.c_uint32),
                ("splat_base", C.c_uint32), ("splat_count", C.c_uint32), ("scene", C.c_uint32)]


SCHEDULE_ROW_MAJOR = 0
SCHEDULE_KEY_COUNT = 1
SCHEDULE_LEARNED = 2


class ScheduleStatus_t(C.Structure):
    _fields_ = [("schedule", C.c_uint32), ("active", C.c_uint32), ("mae_log", C.c_float),
                ("last_mae_log", C.c_float), ("bound", C.c_float), ("frames", C.c_uint32),
                ("fallbacks", C.c_uint32), ("split_tiles", C.c_uint32)]


MLP_FEATURES, MLP_HIDDEN = 16, 64
MLP_PARAMS = 64 * 16 + 64 + 64 * 64 + 64 + 64 + 1

assert C.sizeof(Camera_t) == 288

# every entry point declared in include/gs3d.h, with its ctypes signature
_P, _U32, _I, _SZ = C.c_void_p, C.c_uint32, C.c_int, C.c_size_t
SIGNATURES = {
    "gs3d_abi_version": ([], _I),
    "gs3d_create": ([C.POINTER(C.c_void_p), C.POINTER(Config_t)], _I),
    "gs3d_destroy": ([_P], _I),
    "gs3d_last_error": ([_P], C.c_char_p),
    "gs3d_set_splats": ([_P, _U32, _P, _P, _P, _P, _P, _U32, _I], _I),
    "gs3d_add_scene": ([_P, _U32, _P, _P, _P, _P, _P, _U32, _I, C.POINTER(_U32)], _I),
    "gs3d_rebin_batch": ([_P, _P, _U32], _I),
    "gs3d_get_view_info": ([_P, _U32, C.POINTER(ViewInfo_t)], _I),
    "gs3d_set_schedule": ([_P, _U32], _I),
    "gs3d_set_tuning": ([_P, C.POINTER(Tuning_t)], _I),
    "gs3d_get_tuning": ([_P, C.POINTER(Tuning_t)], _I),
    "gs3d_autotune": ([_P, _P, _U32, _U32, C.POINTER(TuneResult_t), _U32, C.POINTER(_U32)], _I),
    "gs3d_set_tile_size": ([_P, _U32, _U32, C.POINTER(_U32), C.POINTER(_U32)], _I),
    "gs3d_set_camera": ([_P, C.POINTER(Camera_t), _U32, _U32], _I),
    "gs3d_preprocess": ([_P], _I),
    "gs3d_prefix_scan": ([_P], _I),
    "gs3d_emit_tile_refs": ([_P], _I),
    "gs3d_radix_sort": ([_P], _I),
    "gs3d_identify_tile_ranges": ([_P], _I),
    "gs3d_rasterize_tiles": ([_P], _I),
    "gs3d_rebin": ([_P, C.POINTER(Camera_t), _U32, _U32], _I),
    "gs3d_set_flags": ([_P, _U32], _I),
    "gs3d_read_stage_times": ([_P, C.POINTER(C.c_double), C.POINTER(_U32)], _I),
    "gs3d_synchronize": ([_P], _I),
    "gs3d_buffer_info": ([_P, _I, C.POINTER(C.c_void_p), C.POINTER(_SZ)], _I),
    "gs3d_read_buffer": ([_P, _I, _P, _SZ], _I),
    "gs3d_write_buffer": ([_P, _I, _P, _SZ], _I),
    "gs3d_copy_buffer_async": ([_P, _I, _P, _SZ], _I),
    "gs3d_ref_count": ([_P, C.POINTER(_U32)], _I),
    "gs3d_read_tile_counts": ([_P, _P, _SZ], _I),
    "gs3d_prefix_scan_noalloc": ([_P, _P, _U32, _P], _I),
    "gs3d_prefix_scan_noalloc_status": ([_P], _I),
    "gs3d_ply_inspect": ([_P, _SZ, C.POINTER(PlyInfo_t)], _I),
    "gs3d_read_buffer_range": ([_P, _I, _SZ, _P, _SZ], _I),
    "gs3d_composite": ([_P, _U32, _U32, _U32, _P, _P, _SZ, _I], _I),
    "gs3d_load_ply": ([_P, _P, _SZ, _U32, C.POINTER(_U32), C.POINTER(PlyInfo_t)], _I),
    "gs3d_set_cost_model": ([_P, _P, _P, _P], _I),
    "gs3d_set_schedule_gate": ([_P, C.c_float], _I),
    "gs3d_get_schedule_status": ([_P, C.POINTER(ScheduleStatus_t)], _I),
    "gs3d_tile_features": ([_P, _P, _P, _U32, _I], _I),
    "gs3d_mlp_forward": ([_P, _P, _U32, _P, _P, _P], _I),
    "gs3d_mlp_backward": ([_P, _P, _P, _P, _U32, _P, _P], _I),
    "gs3d_mlp_adam": ([_P, _P, _P, _P, _U32, C.c_float, C.c_float, C.c_float, C.c_float,
                       _U32, _P], _I),
    "gs3d_mlp_infer": ([_P, _P, _U32, _P, _P], _I),
}

_lib = None


def load() -> C.CDLL:
    """Loads libgs3d.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with webgpu-3dgs_gb300/build.py "
                "(there is no CPU fallback)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib
