"""TEST INFRASTRUCTURE ONLY: ctypes front of the CPU restatement in gs_oracle.cpp.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this package, always as
the checker or the timed CPU baseline, never as a product path. PARITY UNPINNED: the reference has
no golden vectors for this path and its WGSL cannot run here (see gs_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"


class _Out(C.Structure):
    _fields_ = [
        ("tiles_touched", C.c_void_p), ("meta", C.c_void_p), ("conic_opacity", C.c_void_p), ("pixel", C.c_void_p),
        ("color", C.c_void_p), ("offsets", C.c_void_p), ("keys", C.c_void_p), ("vals", C.c_void_p),
        ("keys_capacity", C.c_uint64), ("ranges", C.c_void_p), ("rgb", C.c_void_p), ("final_t", C.c_void_p),
        ("n_contrib", C.c_void_p), ("rgba8", C.c_void_p), ("instance_count", C.c_uint32),
        ("sorted_count", C.c_uint32), ("max_instance", C.c_uint32), ("tiles_x", C.c_uint32), ("tiles_y", C.c_uint32),
    ]


_LIB = None


def load() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            import sys
            sys.path.insert(0, str(HERE.parent / "web-gs-renderer_gb300"))
            from build import build_oracle  # type: ignore
            build_oracle()
        lib = C.CDLL(str(LIB_PATH))
        lib.oracle_forward_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                           C.POINTER(_Out), C.c_int]
        lib.oracle_forward_f32_timed.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                                 C.POINTER(_Out), C.c_int, C.POINTER(C.c_double), C.c_uint32]
        lib.oracle_forward_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                           C.c_void_p, C.POINTER(C.c_uint32), C.c_int]
        lib.oracle_expf.restype = C.c_float
        lib.oracle_expf.argtypes = [C.c_float]
        lib.oracle_expf_array.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
        lib.oracle_raster_expf_array.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
        lib.oracle_radix_sort_pairs.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]
        lib.oracle_exclusive_scan.restype = C.c_uint32
        lib.oracle_exclusive_scan.argtypes = [C.c_void_p, C.c_uint32]
        lib.oracle_camera_view.argtypes = [C.POINTER(C.c_float * 3), C.POINTER(C.c_float * 3),
                                           C.POINTER(C.c_float * 3), C.c_float, C.c_uint32, C.c_uint32, C.c_float,
                                           C.c_float, C.c_void_p]
        lib.oracle_synth_scene.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_float, C.c_void_p]
        lib.oracle_perturb_scene.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_float]
        lib.oracle_tile_ranges_reference.restype = C.c_uint32
        lib.oracle_tile_ranges_reference.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p]
        _LIB = lib
    return _LIB


def _threads(threads: int | None) -> int:
    return threads if threads else (os.cpu_count() or 1)


def forward_f32(view: bytes, packed: np.ndarray, count: int, tile: int = 16, factor: int = 64,
                threads: int | None = None, keys: bool = True, timed: bool = False, row_stride: int = 1) -> dict:
    """Runs the fp32 restatement of one frame; returns every intermediate and output."""
    lib = load()
    packed = np.ascontiguousarray(packed, dtype=np.float32)
    assert packed.size == 59 * count and len(view) == 176
    vb = C.create_string_buffer(view, 176)
    w = int(np.frombuffer(view, np.float32, 2, 160)[0])
    h = int(np.frombuffer(view, np.float32, 2, 160)[1])
    tx, ty = (w + tile - 1) // tile, (h + tile - 1) // tile
    cap = count * factor if keys else 0
    r = {
        "tiles_touched": np.zeros(count, np.uint32), "meta": np.zeros(4 * count, np.uint32),
        "conic_opacity": np.zeros(4 * count, np.float32), "pixel": np.zeros(2 * count, np.float32),
        "color": np.zeros(4 * count, np.float32), "offsets": np.zeros(count + 1, np.uint32),
        "keys": np.zeros(max(cap, 1), np.uint32), "vals": np.zeros(max(cap, 1), np.uint32),
        "ranges": np.zeros(2 * tx * ty, np.uint32), "rgb": np.zeros((h, w, 3), np.float32),
        "final_t": np.zeros((h, w), np.float32), "n_contrib": np.zeros((h, w), np.uint32),
        "rgba8": np.zeros((h, w, 4), np.uint8),
    }
    o = _Out(*[r[k].ctypes.data for k in ("tiles_touched", "meta", "conic_opacity", "pixel", "color", "offsets",
                                          "keys", "vals")], cap, *[r[k].ctypes.data for k in
                                                                   ("ranges", "rgb", "final_t", "n_contrib", "rgba8")])
    if timed:
        ms = (C.c_double * 8)()
        rc = lib.oracle_forward_f32_timed(vb, packed.ctypes.data, count, tile, factor, C.byref(o), _threads(threads), ms,
                                          row_stride)
        r["pass_ms"] = {k: ms[i] for i, k in enumerate(("preprocess", "scan", "emit", "sort", "tile ranges", "raster"))}
    else:
        rc = lib.oracle_forward_f32(vb, packed.ctypes.data, count, tile, factor, C.byref(o), _threads(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_forward_f32 failed ({rc})")
    n = o.sorted_count
    r["keys"] = r["keys"][: min(n, cap)]
    r["vals"] = r["vals"][: min(n, cap)]
    r.update(instance_count=o.instance_count, sorted_count=o.sorted_count, max_instance=o.max_instance,
             tiles_x=o.tiles_x, tiles_y=o.tiles_y)
    return r


def forward_f64(view: bytes, packed: np.ndarray, count: int, tile: int = 16, factor: int = 64,
                threads: int | None = None) -> dict:
    """FP64 twin: the same algorithm in double precision (rgb, final_t, instance count)."""
    lib = load()
    packed = np.ascontiguousarray(packed, dtype=np.float32)
    vb = C.create_string_buffer(view, 176)
    w, h = (int(v) for v in np.frombuffer(view, np.float32, 2, 160))
    rgb = np.zeros((h, w, 3), np.float64)
    ft = np.zeros((h, w), np.float64)
    ic = C.c_uint32()
    rc = lib.oracle_forward_f64(vb, packed.ctypes.data, count, tile, factor, rgb.ctypes.data, ft.ctypes.data,
                                C.byref(ic), _threads(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_forward_f64 failed ({rc})")
    return {"rgb": rgb, "final_t": ft, "instance_count": ic.value}


def expf(x: np.ndarray) -> np.ndarray:
    xx = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(xx)
    load().oracle_expf_array(xx.ctypes.data, y.ctypes.data, xx.size)
    return y


def raster_expf(x: np.ndarray) -> np.ndarray:
    """The raster's exp (rule 4b of gs_oracle.h), defined for x in [-5.6, 0]."""
    xx = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(xx)
    load().oracle_raster_expf_array(xx.ctypes.data, y.ctypes.data, xx.size)
    return y


def radix_sort_pairs(keys: np.ndarray, vals: np.ndarray, passes: int = 4) -> tuple[np.ndarray, np.ndarray]:
    k = np.array(keys, dtype=np.uint32, copy=True)
    v = np.array(vals, dtype=np.uint32, copy=True)
    load().oracle_radix_sort_pairs(k.ctypes.data, v.ctypes.data, k.size, passes)
    return k, v


def exclusive_scan(data: np.ndarray) -> tuple[np.ndarray, int]:
    d = np.array(data, dtype=np.uint32, copy=True)
    tot = load().oracle_exclusive_scan(d.ctypes.data, d.size)
    return d, int(tot)


def tile_ranges_reference(keys: np.ndarray, sorted_count: int, instance_count: int, tiles: int) -> tuple[np.ndarray, int]:
    """tile_ranges.wgsl as the reference binds it (unclamped instance count); returns (ranges,
    threads that would read past the keys buffer)."""
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    ranges = np.zeros(2 * tiles, np.uint32)
    beyond = load().oracle_tile_ranges_reference(k.ctypes.data, k.size, sorted_count, instance_count, ranges.ctypes.data)
    return ranges, int(beyond)


def backward_f64(view: bytes, packed: np.ndarray, count: int, dl_drgb: np.ndarray, tile: int = 16, factor: int = 64,
                 threads: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """FP64 adjoint: (dL/d(packed attributes) as 59*count float64, the FP64 rgb image)."""
    lib = load()
    if not hasattr(lib, "_bwd_set"):
        lib.oracle_backward_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_int]
        lib.oracle_loss_l1_ssim.restype = C.c_double
        lib.oracle_loss_l1_ssim.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p]
        lib._bwd_set = True
    packed = np.ascontiguousarray(packed, dtype=np.float32)
    vb = C.create_string_buffer(view, 176)
    w, h = (int(v) for v in np.frombuffer(view, np.float32, 2, 160))
    dl = np.ascontiguousarray(dl_drgb, dtype=np.float64).reshape(h, w, 3)
    grad = np.zeros(59 * count, np.float64)
    rgb = np.zeros((h, w, 3), np.float64)
    rc = lib.oracle_backward_f64(vb, packed.ctypes.data, count, tile, factor, dl.ctypes.data, grad.ctypes.data,
                                 rgb.ctypes.data, _threads(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_backward_f64 failed ({rc})")
    return grad, rgb


def loss_l1_ssim(x: np.ndarray, y: np.ndarray, lam: float = 0.2, grad: bool = True):
    """FP64 L1 + lam * (1 - SSIM) of H x W x 3 images, and dL/dx."""
    lib = load()
    backward_f64.__wrapped__ = True  # argtypes are set on first use of either function
    if not hasattr(lib, "_bwd_set"):
        lib.oracle_loss_l1_ssim.restype = C.c_double
        lib.oracle_loss_l1_ssim.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p]
        lib.oracle_backward_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_int]
        lib._bwd_set = True
    xx = np.ascontiguousarray(x, dtype=np.float64)
    yy = np.ascontiguousarray(y, dtype=np.float64)
    h, w = xx.shape[:2]
    g = np.zeros_like(xx) if grad else None
    val = lib.oracle_loss_l1_ssim(xx.ctypes.data, yy.ctypes.data, w, h, lam, g.ctypes.data if grad else None)
    return float(val), g


# ---- inputs of the benchmark configurations (gs_inputs.cpp), built without the product library ----
def camera_view(eye, target, up=(0.0, 1.0, 0.0), fovy_deg: float = 60.0, width: int = 512, height: int = 512,
                z_near: float = 0.2, z_far: float = 1000.0) -> bytes:
    """The 176-byte GlobalUniforms block of a camera at `eye` looking at `target` (camera.js:87-98)."""
    f3 = C.c_float * 3
    out = C.create_string_buffer(176)
    rc = load().oracle_camera_view(C.byref(f3(*eye)), C.byref(f3(*target)), C.byref(f3(*up)), fovy_deg, width,
                                   height, z_near, z_far, out)
    if rc != 0:
        raise ValueError("oracle_camera_view: bad camera")
    return out.raw


def synth_scene(kind: int, count: int, seed: int, clusters: int = 0, box: float = 0.0) -> np.ndarray:
    """Seeded synthetic scene in the packed layout (59*count float32)."""
    packed = np.empty(59 * count, np.float32)
    if load().oracle_synth_scene(kind, count, seed, clusters, box, packed.ctypes.data) != 0:
        raise ValueError("oracle_synth_scene: bad arguments")
    return packed


def perturb_scene(packed: np.ndarray, count: int, seed: int, sigma_mean: float, sigma_sh: float) -> np.ndarray:
    """A perturbed copy: means + N(0, sigma_mean^2), SH + N(0, sigma_sh^2)."""
    out = np.array(packed, dtype=np.float32, copy=True)
    load().oracle_perturb_scene(out.ctypes.data, count, seed, sigma_mean, sigma_sh)
    return out
