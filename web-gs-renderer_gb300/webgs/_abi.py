"""ctypes declarations of include/gs.h (the C ABI of libwebgs.so)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "lib" / "libwebgs.so"
# WEBGS_CHECKED=1 selects the checked build (canary-padded buffers, bounds-checked stores): a
# test-only library, the stand-in for a memory sanitizer
CHECKED_LIB_PATH = PKG_DIR / "lib" / "libwebgs_checked.so"
HEADER_PATH = PKG_DIR.parent / "include" / "gs.h"

GS_OK = 0
GS_ERR_INVALID = 1
GS_ERR_OOM = 2
GS_ERR_OVERFLOW = 3
GS_ERR_TIMEOUT = 4
GS_ERR_CUDA = 5
GS_ERR_STATE = 6
GS_ERR_UNSUPPORTED = 7
GS_ERR_MEMORY = 8
STATUS_NAMES = {
    0: "GS_OK", 1: "GS_ERR_INVALID", 2: "GS_ERR_OOM", 3: "GS_ERR_OVERFLOW", 4: "GS_ERR_TIMEOUT",
    5: "GS_ERR_CUDA", 6: "GS_ERR_STATE", 7: "GS_ERR_UNSUPPORTED", 8: "GS_ERR_MEMORY",
}

GS_MEM_HOST = 0
GS_MEM_DEVICE = 1
GS_FLAG_PROFILE = 1
GS_FLAG_NO_GRAPH = 2
GS_FLAG_DIFFERENTIABLE = 4
GS_DEV_OVERFLOW = 1
GS_DEV_TIMEOUT = 2
GS_DEV_BOUNDS = 4
GS_DEV_CANARY = 8


class View(C.Structure):
    """GlobalUniforms (preprocess.wgsl:2-12), 176 bytes."""
    _fields_ = [
        ("view", C.c_float * 16), ("view_proj", C.c_float * 16), ("camera_pos", C.c_float * 3),
        ("count", C.c_uint32), ("focal", C.c_float * 2), ("tan_fov", C.c_float * 2),
        ("texture_size", C.c_float * 2), ("pad0", C.c_uint32), ("pad1", C.c_uint32),
    ]


assert C.sizeof(View) == 176


class Config(C.Structure):
    _fields_ = [
        ("tile_size", C.c_uint32), ("digit_bits", C.c_uint32), ("raster_batch", C.c_uint32),
        ("max_instance_factor", C.c_uint32), ("flags", C.c_uint32), ("device", C.c_int32),
        ("sort_block", C.c_uint32),
    ]


class Image(C.Structure):
    _fields_ = [
        ("location", C.c_int32), ("rgba8", C.c_void_p), ("rgb", C.c_void_p), ("final_t", C.c_void_p),
        ("n_contrib", C.c_void_p),
    ]


class FrameInfo(C.Structure):
    _fields_ = [
        ("instance_count", C.c_uint32), ("sorted_count", C.c_uint32), ("max_instance", C.c_uint32),
        ("visible", C.c_uint32), ("near_pass", C.c_uint32), ("tiles_x", C.c_uint32), ("tiles_y", C.c_uint32), ("status", C.c_uint32),
        ("sort_passes", C.c_uint32),
    ]


class Debug(C.Structure):
    _fields_ = [
        ("tiles_touched", C.c_void_p), ("meta", C.c_void_p), ("conic_opacity", C.c_void_p), ("pixel", C.c_void_p),
        ("color", C.c_void_p), ("offsets", C.c_void_p), ("keys", C.c_void_p), ("vals", C.c_void_p),
        ("capacity", C.c_uint64), ("ranges", C.c_void_p),
    ]


class Timing(C.Structure):
    _fields_ = [("label", C.c_char * 24), ("ms", C.c_float)]


class BatchView(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("view", View), ("out", Image)]


class Camera(C.Structure):
    """gs_camera: the input of Camera.getUniform() (camera.js:87-98), 56 bytes."""
    _fields_ = [
        ("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3), ("fovy_deg", C.c_float),
        ("width", C.c_uint32), ("height", C.c_uint32), ("z_near", C.c_float), ("z_far", C.c_float),
    ]


assert C.sizeof(Camera) == 56


class BatchCamera(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("out", Image)]


# (name, restype, argtypes) of every entry point declared in include/gs.h
SIGNATURES = [
    ("gs_version", C.c_char_p, []),
    ("gs_config_default", None, [C.POINTER(Config)]),
    ("gs_ctx_create", C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    ("gs_ctx_destroy", C.c_int, [C.c_void_p]),
    ("gs_last_error", C.c_char_p, [C.c_void_p]),
    ("gs_ctx_synchronize", C.c_int, [C.c_void_p]),
    ("gs_ctx_stream", C.c_void_p, [C.c_void_p]),
    ("gs_scene_upload", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int32, C.POINTER(C.c_void_p)]),
    ("gs_scene_update", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    ("gs_scene_destroy", C.c_int, [C.c_void_p]),
    ("gs_scene_count", C.c_uint32, [C.c_void_p]),
    ("gs_forward", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(View), C.POINTER(Image)]),
    ("gs_get_frame_info", C.c_int, [C.c_void_p, C.POINTER(FrameInfo)]),
    ("gs_forward_batch", C.c_int, [C.c_void_p, C.POINTER(BatchView), C.c_uint32]),
    ("gs_forward_batch_cameras", C.c_int, [C.c_void_p, C.POINTER(BatchCamera), C.c_uint32]),
    ("gs_camera_views", C.c_int, [C.c_void_p, C.POINTER(Camera), C.c_uint32, C.c_void_p, C.c_int32]),
    ("gs_get_batch_frame_info", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(FrameInfo)]),
    ("gs_backward_batch", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, C.c_void_p,
                                    C.c_int32]),
    ("gs_autotune", C.c_int, [C.POINTER(Config), C.c_void_p, C.c_uint32, C.POINTER(View), C.c_uint32, C.c_uint32,
                              C.POINTER(Config), C.POINTER(C.c_float)]),
    ("gs_autotune_scenes", C.c_int, [C.POINTER(Config), C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(View),
                                     C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(Config), C.POINTER(C.c_float)]),
    ("gs_get_debug", C.c_int, [C.c_void_p, C.POINTER(Debug)]),
    ("gs_backward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    ("gs_loss_l1_ssim", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_float,
                                  C.POINTER(C.c_double), C.c_void_p, C.c_int32]),
    ("gs_get_timings", C.c_int, [C.c_void_p, C.POINTER(Timing), C.c_int32, C.POINTER(C.c_int32)]),
    ("gs_sort_pairs", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32]),
    ("gs_exclusive_scan", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.c_int32]),
    ("gs_exp_f32", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int32]),
    ("gs_raster_exp_f32", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int32]),
    ("gs_raster_alpha_f32", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int32]),
    ("gs_check_wait_timeout", C.c_int, [C.c_void_p]),
    ("gs_exclusive_scan_static", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("gs_debug_set_sequence", C.c_int, [C.c_void_p, C.c_uint32]),
    ("gs_checked_build", C.c_int, []),
    ("gs_debug_damage_canary", C.c_int, [C.c_void_p]),
    ("gs_camera_view", C.c_int, [C.POINTER(C.c_float * 3), C.POINTER(C.c_float * 3), C.POINTER(C.c_float * 3),
                                 C.c_float, C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.POINTER(View)]),
    ("gs_synth_scene", C.c_int, [C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_float, C.c_void_p]),
    ("gs_perturb_scene", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_float]),
    ("gs_write_ppm", C.c_int, [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32]),
    ("gs_ply_parse", C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(C.c_uint32), C.c_void_p, C.c_char_p, C.c_size_t]),
]

_LIB = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libwebgs.so. Raises if it has not been built: there is no fallback path."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else (CHECKED_LIB_PATH if os.environ.get("WEBGS_CHECKED") == "1" else LIB_PATH)
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with web-gs-renderer_gb300/build.py (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib
