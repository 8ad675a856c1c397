"""CPU tests of the C ABI boundary: the library loads and exports every entry point include/gs.h
declares; the ctypes structs match the header; the host utilities (no GPU) behave."""
import ctypes as C
import re

import numpy as np
import pytest

import webgs
from webgs import _abi


def _declared_functions() -> list[str]:
    text = _abi.HEADER_PATH.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = webgs.library()
    names = _declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), f"libwebgs.so does not export {name}"
    bound = {n for n, _, _ in _abi.SIGNATURES}
    assert set(names) <= bound | {"gs_last_error"}, set(names) - bound


def test_struct_sizes_match_header():
    assert C.sizeof(_abi.View) == 176
    assert C.sizeof(_abi.Config) == 28
    assert C.sizeof(_abi.FrameInfo) == 4 * 9
    assert C.sizeof(_abi.Timing) == 28


def test_config_defaults_are_reference_constants():
    cfg = _abi.Config()
    webgs.library().gs_config_default(C.byref(cfg))
    assert (cfg.tile_size, cfg.digit_bits, cfg.raster_batch, cfg.max_instance_factor) == (16, 8, 256, 64)
    assert cfg.sort_block == 4096


def test_version_string():
    assert b"sm_103a" in webgs.library().gs_version()


def test_null_context_calls_fail_cleanly():
    lib = webgs.library()
    assert lib.gs_ctx_destroy(None) == _abi.GS_ERR_INVALID
    assert lib.gs_forward(None, None, None, None) == _abi.GS_ERR_INVALID
    assert lib.gs_ctx_synchronize(None) == _abi.GS_ERR_INVALID
    assert lib.gs_last_error(None) == b"invalid context"
    assert lib.gs_scene_count(None) == 0


def _lookat_perspective(eye, target, up, fovy, w, h, near, far):
    """wgpu-matrix lookAt / perspective (0..1 depth), restated in numpy."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    z = eye - target
    z /= np.linalg.norm(z)
    x = np.cross(up, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    y /= np.linalg.norm(y)
    view = np.zeros((4, 4))  # [col][row]
    view[0] = (x[0], y[0], z[0], 0)
    view[1] = (x[1], y[1], z[1], 0)
    view[2] = (x[2], y[2], z[2], 0)
    view[3] = (-x @ eye, -y @ eye, -z @ eye, 1)
    f = np.tan(np.pi / 2 - np.radians(fovy) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0] = f / (w / h)
    proj[1, 1] = f
    proj[2, 2] = far / (near - far)
    proj[2, 3] = -1
    proj[3, 2] = near * far / (near - far)
    return view.astype(np.float32), proj.astype(np.float32)


def test_camera_view_matches_lookat_perspective():
    eye, tgt = (0.3, 1.0, -9.0), (0.0, 0.0, 0.0)
    v = webgs.camera_view(eye, tgt, (0.0, 1.0, 0.0), 70.0, 1920, 1080, 0.2, 1000.0)
    view, proj = _lookat_perspective(eye, tgt, (0, 1, 0), 70.0, 1920, 1080, 0.2, 1000.0)
    np.testing.assert_allclose(np.array(v.view).reshape(4, 4), view, rtol=1e-6, atol=1e-6)
    vp = (proj.T.astype(np.float64) @ view.T.astype(np.float64)).T  # column-major product proj*view
    np.testing.assert_allclose(np.array(v.view_proj).reshape(4, 4), vp, rtol=1e-5, atol=1e-5)
    tan_y = np.tan(np.radians(35.0))
    assert np.isclose(v.tan_fov[1], tan_y) and np.isclose(v.tan_fov[0], tan_y * 1920 / 1080)
    assert np.isclose(v.focal[1], 1080 / (2 * tan_y)) and np.isclose(v.focal[0], 1920 / (2 * tan_y * 1920 / 1080))
    assert tuple(v.texture_size) == (1920.0, 1080.0)
    # a point in front of the camera has negative view z and clip depth in (0, 1)
    p = np.array([0.0, 0.0, 0.0, 1.0])
    pv = np.array(v.view).reshape(4, 4).T @ p
    clip = np.array(v.view_proj).reshape(4, 4).T @ p
    assert pv[2] < 0 and 0 < clip[2] / clip[3] < 1


def test_camera_view_rejects_bad_arguments():
    with pytest.raises(webgs.GsError):
        webgs.camera_view((0, 0, 0), (0, 0, 1), (0, 1, 0), 0.0, 10, 10)
    with pytest.raises(webgs.GsError):
        webgs.camera_view((0, 0, 0), (0, 0, 1), (0, 1, 0), 60.0, 0, 10)


def test_synth_scene_is_deterministic_and_distributed():
    a = webgs.synth_scene(0, 20_000, 0)
    b = webgs.synth_scene(0, 20_000, 0)
    c = webgs.synth_scene(0, 20_000, 1)
    assert a.dtype == np.float32 and a.size == 59 * 20_000
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    n = 20_000
    pos, scale = a[: 3 * n], a[3 * n: 6 * n]
    quat = a[6 * n: 10 * n].reshape(n, 4)
    dc, op, rest = a[10 * n: 13 * n], a[13 * n: 14 * n], a[14 * n:]
    assert abs(pos.mean()) < 0.03 and abs(pos.std() - 1.0) < 0.02
    assert abs(scale.mean() + 4.0) < 0.02 and abs(scale.std() - 0.5) < 0.01
    np.testing.assert_allclose(np.linalg.norm(quat, axis=1), 1.0, atol=1e-6)
    assert abs(op.std() - 1.5) < 0.03 and abs(dc.std() - 0.5) < 0.01 and abs(rest.std() - 0.05) < 0.001


def test_synth_cluster_scene_stays_in_box():
    n = 10_000
    a = webgs.synth_scene(1, n, 3, 64, 20.0)
    pos = a[: 3 * n]
    assert pos.min() >= -10.0 and pos.max() <= 10.0
    assert pos.std() > 2.0


def test_perturb_scene_moves_only_means_and_sh():
    n = 1000
    a = webgs.synth_scene(0, n, 0)
    b = webgs.perturb_scene(a, n, 7, 0.01, 0.02)
    d = b - a
    assert 0.005 < d[: 3 * n].std() < 0.015
    assert np.all(d[3 * n: 10 * n] == 0) and np.all(d[13 * n: 14 * n] == 0)
    assert 0.01 < d[10 * n: 13 * n].std() < 0.03 and 0.015 < d[14 * n:].std() < 0.025


def test_product_library_is_not_the_checked_build():
    lib = webgs.library()
    assert lib.gs_checked_build() == 0
    assert lib.gs_debug_damage_canary(None) == _abi.GS_ERR_INVALID


def test_new_entry_points_reject_null_context():
    lib = webgs.library()
    assert lib.gs_camera_views(None, None, 0, None, webgs.GS_MEM_HOST) == _abi.GS_ERR_INVALID
    assert lib.gs_forward_batch_cameras(None, None, 1) == _abi.GS_ERR_INVALID
    assert lib.gs_raster_exp_f32(None, None, None, 0, webgs.GS_MEM_HOST) == _abi.GS_ERR_INVALID
    assert lib.gs_raster_alpha_f32(None, None, None, None, 0, webgs.GS_MEM_HOST) == _abi.GS_ERR_INVALID
    assert lib.gs_debug_set_sequence is not None  # a test hook (needs a GPU to do anything)
    assert C.sizeof(_abi.Camera) == 56 and C.sizeof(_abi.BatchCamera) == C.sizeof(_abi.BatchView) - 176 + 56
