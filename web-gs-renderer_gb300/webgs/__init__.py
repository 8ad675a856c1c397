"""webgs -- host side of the GB300 splat pipeline (ctypes over libwebgs.so).

Mirrors the reference's JavaScript interface (KoS-Y1/Web-GS-Renderer src/renderer/renderer.js and
src/renderer/camera.js): `Renderer.upload_gs_data / set_gs / execute` and `Camera.get_uniform`,
with errors raised as `GsError` like the reference's fail() (src/utils/utils.js:3-47). Every
compute call goes through the CUDA library; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import _abi
from ._abi import (GS_FLAG_DIFFERENTIABLE, GS_FLAG_NO_GRAPH, GS_FLAG_PROFILE, GS_MEM_DEVICE, GS_MEM_HOST,
                   Config, Debug, FrameInfo, Image, Timing, View)

__all__ = [
    "GsError", "Context", "Scene", "Renderer", "Camera", "View", "Config", "camera_view", "make_camera", "synth_scene",
    "perturb_scene", "view_bytes", "FLOATS_PER_GAUSSIAN", "GS_FLAG_PROFILE", "GS_FLAG_NO_GRAPH",
    "GS_FLAG_DIFFERENTIABLE", "GS_MEM_HOST", "GS_MEM_DEVICE", "library",
]

FLOATS_PER_GAUSSIAN = 59  # 3 pos + 3 scale + 4 rot + 3 dc + 1 opacity + 45 rest (loader.js:77)


class GsError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def library() -> C.CDLL:
    return _abi.load()


def _check(code: int, ctx_ptr=None, what: str = "") -> int:
    if code != _abi.GS_OK:
        msg = library().gs_last_error(ctx_ptr).decode() if ctx_ptr else what
        raise GsError(code, msg or what)
    return code


def _ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


# ---- host utilities ----------------------------------------------------------------------------
def camera_view(eye, target, up=(0.0, 1.0, 0.0), fovy_deg: float = 60.0, width: int = 512, height: int = 512,
                z_near: float = 0.2, z_far: float = 1000.0) -> View:
    """Camera.getUniform() (camera.js:87-98) for a camera at `eye` looking at `target`."""
    v = View()
    f3 = C.c_float * 3
    rc = library().gs_camera_view(C.byref(f3(*eye)), C.byref(f3(*target)), C.byref(f3(*up)), float(fovy_deg),
                                  int(width), int(height), float(z_near), float(z_far), C.byref(v))
    _check(rc, None, "gs_camera_view")
    return v


def make_camera(eye, target, up=(0.0, 1.0, 0.0), fovy_deg: float = 60.0, width: int = 512, height: int = 512,
                z_near: float = 0.2, z_far: float = 1000.0) -> "_abi.Camera":
    """A gs_camera: what camera_view takes, for the device-side builders (camera_views,
    forward_batch_cameras)."""
    c = _abi.Camera()
    c.eye[:] = [float(v) for v in eye]
    c.target[:] = [float(v) for v in target]
    c.up[:] = [float(v) for v in up]
    c.fovy_deg, c.width, c.height, c.z_near, c.z_far = float(fovy_deg), int(width), int(height), float(z_near), float(z_far)
    return c


def view_bytes(v: View) -> bytes:
    return bytes(memoryview(v).cast("B"))


def view_from_bytes(b: bytes) -> View:
    v = View()
    C.memmove(C.byref(v), b, C.sizeof(View))
    return v


def synth_scene(kind: int, count: int, seed: int, clusters: int = 0, box: float = 0.0) -> np.ndarray:
    """Seeded synthetic scene in the packed layout (59*count float32), bit-identical on every host."""
    out = np.empty(count * FLOATS_PER_GAUSSIAN, dtype=np.float32)
    _check(library().gs_synth_scene(kind, count, seed, clusters, box, _ptr(out)), None, "gs_synth_scene")
    return out


def load_ply(source) -> dict:
    """loadPly (src/loader/loader.js:56-149): a binary little-endian .ply (path or bytes) ->
    {"count": n, "packed": float32 array of 59*n}, the argument Renderer.upload_gs_data takes."""
    data = source if isinstance(source, (bytes, bytearray, memoryview)) else open(source, "rb").read()
    data = bytes(data)
    lib = library()
    n = C.c_uint32()
    err = C.create_string_buffer(256)
    rc = lib.gs_ply_parse(data, len(data), C.byref(n), None, err, 256)
    if rc != _abi.GS_OK:
        raise GsError(rc, err.value.decode())
    packed = np.empty(n.value * FLOATS_PER_GAUSSIAN, dtype=np.float32)
    _check(lib.gs_ply_parse(data, len(data), C.byref(n), _ptr(packed), err, 256), None, "gs_ply_parse")
    return {"count": n.value, "packed": packed}


def save_ppm(path, rgba8: np.ndarray) -> None:
    """Writes an H x W x 4 rgba8 frame as a binary PPM (gs_write_ppm): the present step of the
    reference (blit.wgsl to the canvas) as a file."""
    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("rgba8 must be H x W x 4")
    _check(library().gs_write_ppm(str(path).encode(), _ptr(img), img.shape[1], img.shape[0]), None,
           f"gs_write_ppm: cannot write {path}")


def save_png(path, rgba8: np.ndarray) -> None:
    """Writes an H x W x 4 rgba8 frame as an 8-bit RGBA PNG (zlib from the standard library)."""
    import struct
    import zlib

    img = np.ascontiguousarray(rgba8, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("rgba8 must be H x W x 4")
    h, w = img.shape[:2]
    raw = np.concatenate([np.zeros((h, 1), np.uint8), img.reshape(h, w * 4)], axis=1).tobytes()

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def perturb_scene(packed: np.ndarray, count: int, seed: int, sigma_mean: float, sigma_sh: float) -> np.ndarray:
    out = np.array(packed, dtype=np.float32, copy=True)
    _check(library().gs_perturb_scene(_ptr(out), count, seed, sigma_mean, sigma_sh), None, "gs_perturb_scene")
    return out


# ---- context -----------------------------------------------------------------------------------
class Scene:
    def __init__(self, ctx: "Context", handle: C.c_void_p, count: int):
        self.ctx = ctx
        self.handle = handle
        self.count = count

    def update(self, packed: np.ndarray | int, location: int = GS_MEM_HOST) -> None:
        ptr = packed if isinstance(packed, int) else _ptr(np.ascontiguousarray(packed, dtype=np.float32))
        self.ctx._ck(library().gs_scene_update(self.ctx.handle, self.handle, ptr, location))

    def close(self) -> None:
        if self.handle:
            library().gs_scene_destroy(self.handle)
            self.handle = None


class Context:
    """One CUDA stream and its frame buffers (include/gs.h gs_ctx)."""

    def __init__(self, tile_size: int = 16, digit_bits: int = 8, raster_batch: int = 256,
                 max_instance_factor: int = 64, flags: int = 0, device: int = 0, sort_block: int = 4096):
        lib = library()
        cfg = Config()
        lib.gs_config_default(C.byref(cfg))
        cfg.tile_size, cfg.digit_bits, cfg.raster_batch = tile_size, digit_bits, raster_batch
        cfg.sort_block = sort_block
        cfg.max_instance_factor, cfg.flags, cfg.device = max_instance_factor, flags, device
        self.config = cfg
        h = C.c_void_p()
        rc = lib.gs_ctx_create(C.byref(cfg), C.byref(h))
        if rc != _abi.GS_OK:
            raise GsError(rc, "gs_ctx_create failed (no CUDA device, or an invalid configuration)")
        self.handle = h

    def _ck(self, rc: int) -> int:
        return _check(rc, self.handle)

    def close(self) -> None:
        if self.handle:
            library().gs_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def stream(self) -> int:
        return library().gs_ctx_stream(self.handle) or 0

    def synchronize(self) -> None:
        self._ck(library().gs_ctx_synchronize(self.handle))

    def upload(self, packed: np.ndarray | int, count: int, location: int = GS_MEM_HOST) -> Scene:
        if isinstance(packed, int):
            ptr = packed
        else:
            packed = np.ascontiguousarray(packed, dtype=np.float32)
            if packed.size != count * FLOATS_PER_GAUSSIAN:
                raise GsError(_abi.GS_ERR_INVALID, "packed array must hold 59*count floats")
            ptr = _ptr(packed)
        h = C.c_void_p()
        self._ck(library().gs_scene_upload(self.handle, ptr, count, location, C.byref(h)))
        return Scene(self, h, count)

    def forward(self, scene: Scene, view: View, rgba8: bool = True, rgb: bool = False, final_t: bool = False,
                n_contrib: bool = False, allow_overflow: bool = False) -> dict:
        """Renders one frame into new host arrays; returns the requested outputs."""
        w, h = int(view.texture_size[0]), int(view.texture_size[1])
        res = {}
        if rgba8:
            res["rgba8"] = np.empty((h, w, 4), dtype=np.uint8)
        if rgb:
            res["rgb"] = np.empty((h, w, 3), dtype=np.float32)
        if final_t:
            res["final_t"] = np.empty((h, w), dtype=np.float32)
        if n_contrib:
            res["n_contrib"] = np.empty((h, w), dtype=np.uint32)
        img = Image(GS_MEM_HOST, _ptr(res.get("rgba8")), _ptr(res.get("rgb")), _ptr(res.get("final_t")),
                    _ptr(res.get("n_contrib")))
        rc = library().gs_forward(self.handle, scene.handle, C.byref(view), C.byref(img))
        if rc == _abi.GS_ERR_OVERFLOW and allow_overflow:
            res["overflow"] = True
            return res
        self._ck(rc)
        return res

    def forward_device(self, scene: Scene, view: View, rgba8: int = 0, rgb: int = 0, final_t: int = 0,
                       n_contrib: int = 0) -> None:
        """Stream-ordered frame into caller device buffers (raw pointers)."""
        img = Image(GS_MEM_DEVICE, rgba8 or None, rgb or None, final_t or None, n_contrib or None)
        self._ck(library().gs_forward(self.handle, scene.handle, C.byref(view), C.byref(img)))

    def frame_info(self) -> dict:
        fi = FrameInfo()
        self._ck(library().gs_get_frame_info(self.handle, C.byref(fi)))
        return {k: getattr(fi, k) for k, _ in FrameInfo._fields_}

    def debug(self, capacity: int | None = None) -> dict:
        """Intermediates of the last frame (per-Gaussian outputs, offsets, sorted keys/vals, ranges)."""
        return self._debug(self.frame_info(), capacity)

    def _debug(self, info: dict, capacity: int | None) -> dict:
        cap = info["sorted_count"] if capacity is None else capacity
        T = info["tiles_x"] * info["tiles_y"]
        n = self._last_count
        out = {
            "tiles_touched": np.zeros(n, np.uint32), "meta": np.zeros(4 * n, np.uint32),
            "conic_opacity": np.zeros(4 * n, np.float32), "pixel": np.zeros(2 * n, np.float32),
            "color": np.zeros(4 * n, np.float32), "offsets": np.zeros(n + 1, np.uint32),
            "keys": np.zeros(cap, np.uint32), "vals": np.zeros(cap, np.uint32), "ranges": np.zeros(2 * T, np.uint32),
        }
        d = Debug(*[_ptr(out[k]) for k in ("tiles_touched", "meta", "conic_opacity", "pixel", "color", "offsets",
                                           "keys", "vals")], cap, _ptr(out["ranges"]))
        self._ck(library().gs_get_debug(self.handle, C.byref(d)))
        out.update(info)
        return out

    def timings(self) -> dict:
        rows = (Timing * 16)()
        n = C.c_int32()
        self._ck(library().gs_get_timings(self.handle, rows, 16, C.byref(n)))
        return {rows[i].label.decode(): {"ms": float(rows[i].ms)} for i in range(n.value)}

    def backward(self, scene: Scene, dl_drgb: np.ndarray) -> np.ndarray:
        """Gradient of the last frame of `scene` (a GS_FLAG_DIFFERENTIABLE context): dL/drgb in,
        dL/d(packed attributes) out (59*count float32)."""
        g = np.zeros(scene.count * FLOATS_PER_GAUSSIAN, np.float32)
        dl = np.ascontiguousarray(dl_drgb, dtype=np.float32)
        self._ck(library().gs_backward(self.handle, scene.handle, _ptr(dl), _ptr(g), GS_MEM_HOST))
        return g

    def forward_batch(self, items: list, rgba8: bool = True, rgb: bool = False) -> list[dict]:
        """Renders [(scene, view), ...] in one batched launch into new host arrays."""
        arr = (_abi.BatchView * len(items))()
        outs = []
        for i, (scene, view) in enumerate(items):
            w, h = int(view.texture_size[0]), int(view.texture_size[1])
            res = {}
            if rgba8:
                res["rgba8"] = np.empty((h, w, 4), dtype=np.uint8)
            if rgb:
                res["rgb"] = np.empty((h, w, 3), dtype=np.float32)
            arr[i].scene = scene.handle
            arr[i].view = view
            arr[i].out = Image(GS_MEM_HOST, _ptr(res.get("rgba8")), _ptr(res.get("rgb")), None, None)
            outs.append(res)
        self._ck(library().gs_forward_batch(self.handle, arr, len(items)))
        return outs

    def forward_batch_cameras(self, items: list, rgba8: bool = True, rgb: bool = False) -> list[dict]:
        """Renders [(scene, camera), ...] in one batched launch whose view blocks are built on the
        device from the cameras (make_camera)."""
        arr = (_abi.BatchCamera * len(items))()
        outs = []
        for i, (scene, cam) in enumerate(items):
            w, h = int(cam.width), int(cam.height)
            res = {}
            if rgba8:
                res["rgba8"] = np.empty((h, w, 4), dtype=np.uint8)
            if rgb:
                res["rgb"] = np.empty((h, w, 3), dtype=np.float32)
            arr[i].scene = scene.handle
            arr[i].camera = cam
            arr[i].out = Image(GS_MEM_HOST, _ptr(res.get("rgba8")), _ptr(res.get("rgb")), None, None)
            outs.append(res)
        self._ck(library().gs_forward_batch_cameras(self.handle, arr, len(items)))
        return outs

    def camera_views(self, cams: list) -> list[View]:
        """View blocks of the cameras, built on the device (gs_camera_views)."""
        arr = (_abi.Camera * len(cams))(*cams)
        out = (View * len(cams))()
        self._ck(library().gs_camera_views(self.handle, arr, len(cams), C.cast(out, C.c_void_p), GS_MEM_HOST))
        return list(out)

    def batch_frame_info(self, index: int) -> dict:
        fi = FrameInfo()
        self._ck(library().gs_get_batch_frame_info(self.handle, index, C.byref(fi)))
        return {k: getattr(fi, k) for k, _ in FrameInfo._fields_}

    def backward_batch(self, scene: Scene, dl_drgbs: list) -> np.ndarray:
        """Summed gradient of views 0..len-1 of the last batch (all of `scene`)."""
        dls = [np.ascontiguousarray(d, dtype=np.float32) for d in dl_drgbs]
        ptrs = (C.c_void_p * len(dls))(*[_ptr(d) for d in dls])
        g = np.zeros(scene.count * FLOATS_PER_GAUSSIAN, np.float32)
        self._ck(library().gs_backward_batch(self.handle, scene.handle, ptrs, len(dls), _ptr(g), GS_MEM_HOST))
        return g

    def loss(self, rgb: np.ndarray, target: np.ndarray, lam: float = 0.2) -> tuple[float, np.ndarray]:
        """L1 + lam * (1 - SSIM) of an H x W x 3 image against a target, and dL/drgb."""
        x = np.ascontiguousarray(rgb, dtype=np.float32)
        y = np.ascontiguousarray(target, dtype=np.float32)
        h, w = x.shape[:2]
        dl = np.empty_like(x)
        val = C.c_double()
        self._ck(library().gs_loss_l1_ssim(self.handle, _ptr(x), _ptr(y), w, h, lam, C.byref(val), _ptr(dl),
                                           GS_MEM_HOST))
        return val.value, dl

    def sort_pairs(self, keys: np.ndarray, vals: np.ndarray, key_bits: int = 32) -> tuple[np.ndarray, np.ndarray]:
        k = np.array(keys, dtype=np.uint32, copy=True)
        v = np.array(vals, dtype=np.uint32, copy=True)
        self._ck(library().gs_sort_pairs(self.handle, _ptr(k), _ptr(v), k.size, key_bits, GS_MEM_HOST))
        return k, v

    def exclusive_scan(self, data: np.ndarray) -> tuple[np.ndarray, int]:
        d = np.array(data, dtype=np.uint32, copy=True)
        tot = C.c_uint32()
        self._ck(library().gs_exclusive_scan(self.handle, _ptr(d), d.size, C.byref(tot), GS_MEM_HOST))
        return d, tot.value

    def set_sequence(self, seq: int) -> None:
        """Test hook: sets the lookback sequence number of every frame control block of the context."""
        self._ck(library().gs_debug_set_sequence(self.handle, seq & 0xFFFFFFFF))

    def exp(self, x: np.ndarray, raster: bool = False) -> np.ndarray:
        """The kernels' pinned exp on the device (raster=True: the raster's exp, x in [-5.6, 0])."""
        xx = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty_like(xx)
        fn = library().gs_raster_exp_f32 if raster else library().gs_exp_f32
        self._ck(fn(self.handle, _ptr(xx), _ptr(y), xx.size, GS_MEM_HOST))
        return y

    def raster_alpha(self, o: np.ndarray, x: np.ndarray) -> np.ndarray:
        """o * exp(x) as the raster forms it, before the 0.99 clamp (x at or above o's cut-off)."""
        oo = np.ascontiguousarray(o, dtype=np.float32)
        xx = np.ascontiguousarray(x, dtype=np.float32)
        if oo.shape != xx.shape:
            raise ValueError("raster_alpha: o and x differ in shape")
        y = np.empty_like(xx)
        self._ck(library().gs_raster_alpha_f32(self.handle, _ptr(oo), _ptr(xx), _ptr(y), xx.size, GS_MEM_HOST))
        return y


def _forward_tracking(fn):
    def wrapper(self, scene, *a, **k):
        self._last_count = scene.count
        return fn(self, scene, *a, **k)
    return wrapper


Context.forward = _forward_tracking(Context.forward)
Context.forward_device = _forward_tracking(Context.forward_device)


def autotune(packed: np.ndarray, count: int, views: list, iters: int = 5, device: int = 0,
             max_instance_factor: int = 64) -> tuple[dict, float]:
    """Sweeps tile size x radix digit width x raster batch depth x sort block for a batch of views of
    one scene (gs_autotune); returns the fastest configuration and its ms per batch."""
    base = Config()
    library().gs_config_default(C.byref(base))
    base.device, base.max_instance_factor = device, max_instance_factor
    arr = (View * len(views))(*views)
    best, ms = Config(), C.c_float()
    p = np.ascontiguousarray(packed, dtype=np.float32)
    _check(library().gs_autotune(C.byref(base), _ptr(p), count, arr, len(views), iters, C.byref(best), C.byref(ms)),
           None, "gs_autotune")
    return _config_dict(best), ms.value


def autotune_scenes(scenes: list, views: list, view_scene: list, iters: int = 3, device: int = 0,
                    max_instance_factor: int = 64) -> tuple[dict, float]:
    """The same sweep over a whole batch (gs_autotune_scenes): scenes = [(packed, count), ...], view i
    renders scenes[view_scene[i]]; returns the fastest configuration and its ms per batch."""
    base = Config()
    library().gs_config_default(C.byref(base))
    base.device, base.max_instance_factor = device, max_instance_factor
    arrays = [np.ascontiguousarray(p, dtype=np.float32) for p, _ in scenes]
    ptrs = (C.c_void_p * len(arrays))(*[_ptr(a) for a in arrays])
    counts = (C.c_uint32 * len(scenes))(*[int(c) for _, c in scenes])
    vs = (C.c_uint32 * len(views))(*[int(i) for i in view_scene])
    arr = (View * len(views))(*views)
    best, ms = Config(), C.c_float()
    _check(library().gs_autotune_scenes(C.byref(base), ptrs, counts, len(scenes), arr, vs, len(views), iters,
                                        C.byref(best), C.byref(ms)), None, "gs_autotune_scenes")
    return _config_dict(best), ms.value


def _config_dict(cfg: Config) -> dict:
    return {"tile_size": cfg.tile_size, "digit_bits": cfg.digit_bits, "raster_batch": cfg.raster_batch,
            "sort_block": cfg.sort_block}


# ---- Camera (src/renderer/camera.js) -------------------------------------------------------------
DEFAULT_YAW, DEFAULT_PITCH, DEFAULT_FOV = 90.0, 0.0, 60.0
DEFAULT_SPEED, DEFAULT_SENSITIVITY = 1.0, 0.5
Z_NEAR, Z_FAR = 0.2, 1000.0


class Camera:
    """Yaw/pitch fly camera of camera.js:16-159 without the DOM listeners: key and mouse input come
    in through `press`/`release`/`mouse_move` instead of window events."""

    def __init__(self, width: int, height: int):
        self.keys: set[str] = set()
        self.reset(width, height)

    def reset(self, width: int, height: int) -> None:
        self.width, self.height = width, height
        self.eye = np.array([0.0, -2.0, -10.0], dtype=np.float32)
        self.yaw, self.pitch, self.fov = DEFAULT_YAW, DEFAULT_PITCH, DEFAULT_FOV
        self.dirty = True

    def resize(self, width: int, height: int) -> None:
        self.width, self.height = width, height
        self.dirty = True

    def poll_dirty(self) -> bool:
        d, self.dirty = self.dirty, False
        return d

    def frame(self):
        y, p = math.radians(self.yaw), math.radians(self.pitch)
        fwd = np.array([math.cos(y) * math.cos(p), math.sin(p), math.sin(y) * math.cos(p)])
        fwd /= np.linalg.norm(fwd)
        right = np.cross(fwd, [0.0, 1.0, 0.0])
        right /= np.linalg.norm(right)
        up = np.cross(right, fwd)
        up /= np.linalg.norm(up)
        return fwd, right, up

    def press(self, code: str) -> None:
        self.keys.add(code)

    def release(self, code: str) -> None:
        self.keys.discard(code)

    def mouse_move(self, dx: float, dy: float) -> None:
        if "ShiftLeft" not in self.keys:
            return
        self.yaw += dx * DEFAULT_SENSITIVITY
        self.pitch = max(-89.0, min(89.0, self.pitch - dy * DEFAULT_SENSITIVITY))
        self.dirty = True

    def update(self, dt: float) -> None:
        fwd, right, _ = self.frame()
        d = DEFAULT_SPEED * dt
        steps = {"KeyW": fwd, "KeyS": -fwd, "KeyD": right, "KeyA": -right,
                 "KeyQ": np.array([0.0, -1.0, 0.0]), "KeyE": np.array([0.0, 1.0, 0.0])}
        moved = False
        for k, v in steps.items():
            if k in self.keys:
                self.eye = (self.eye + v * d).astype(np.float32)
                moved = True
        if moved:
            self.dirty = True

    def get_uniform(self) -> View:
        fwd, _, up = self.frame()
        target = self.eye.astype(np.float64) + fwd
        return camera_view(self.eye.tolist(), target.tolist(), up.tolist(), self.fov, self.width, self.height,
                           Z_NEAR, Z_FAR)


# ---- Renderer (src/renderer/renderer.js) ---------------------------------------------------------
@dataclass
class _Gs:
    scene: Scene
    count: int


class Renderer:
    """Drop-in for the reference Renderer class: same methods, same errors, headless output.

    `device, context, format` of the WebGPU constructor become the output size; the canvas texture
    and blit pass become `self.image` (H x W x 4 uint8, rgba8unorm). `on_profile(rows)` receives the
    profiler's `{label: {"ms": ...}}` rows (profiler.js:113-121) after every frame when set.
    """

    def __init__(self, width: int, height: int, on_profile: Callable[[dict], None] | None = None, **config):
        flags = config.pop("flags", 0) | (GS_FLAG_PROFILE if on_profile else 0)
        self._ctx = Context(flags=flags, **config)
        self._on_profile = on_profile
        self._gs: dict[str, _Gs] = {}
        self._current: str | None = None
        self._previous: str | None = None
        self.width, self.height = width, height
        self._resized = True
        self.camera = Camera(width, height)
        self.image = np.zeros((height, width, 4), dtype=np.uint8)
        self.frame_count = 0

    def upload_gs_data(self, data: dict, name: str) -> None:
        """renderer.js:468-479: copies data["packed"] (59*count float32) to the device."""
        packed = np.ascontiguousarray(data["packed"], dtype=np.float32)
        sc = self._ctx.upload(packed, int(data["count"]))
        old = self._gs.pop(name, None)
        if old:
            old.scene.close()
        self._gs[name] = _Gs(sc, int(data["count"]))

    uploadGsData = upload_gs_data

    def set_gs(self, name: str) -> None:
        """renderer.js:461-466: unknown names fail like fail()."""
        if name not in self._gs:
            raise GsError(_abi.GS_ERR_INVALID, f'Invalid Gs buffer for name "{name}"')
        self._current = name

    setGs = set_gs

    def resize(self, width: int, height: int) -> None:
        if (width, height) != (self.width, self.height):
            self.width, self.height = width, height
            self.camera.resize(width, height)
            self.image = np.zeros((height, width, 4), dtype=np.uint8)
            self._resized = True

    def execute(self, dt: float = 0.0) -> bool:
        """renderer.js:481-508: renders when the camera, size or scene changed; returns True if a
        frame was rendered into self.image."""
        self.camera.update(dt)
        if self._current not in self._gs:
            return False
        if not self.camera.poll_dirty() and not self._resized and self._current == self._previous:
            return False
        self._previous = self._current
        self._resized = False
        gs = self._gs[self._current]
        view = self.camera.get_uniform()
        img = Image(GS_MEM_HOST, _ptr(self.image), None, None, None)
        self._ctx._last_count = gs.count
        rc = library().gs_forward(self._ctx.handle, gs.scene.handle, C.byref(view), C.byref(img))
        if rc != _abi.GS_ERR_OVERFLOW:  # the reference truncates silently at 64 instances per Gaussian
            self._ctx._ck(rc)
        self.frame_count += 1
        if self._on_profile:
            self._on_profile(self._ctx.timings())
        return True

    def close(self) -> None:
        for g in self._gs.values():
            g.scene.close()
        self._gs.clear()
        self._ctx.close()
