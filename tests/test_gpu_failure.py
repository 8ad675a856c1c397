"""Failure detection without a GPU fault: a device-side wait that never gets its predecessor's
publication gives up at its iteration limit, the kernel records GS_DEV_TIMEOUT and returns, the
call reports GS_ERR_TIMEOUT, and the context keeps working."""
import time

import numpy as np
import pytest

import webgs
from webgs import _abi

pytestmark = pytest.mark.gpu


def test_lookback_wait_times_out_and_context_survives():
    with webgs.Context() as ctx:
        t0 = time.perf_counter()
        rc = webgs.library().gs_check_wait_timeout(ctx.handle)
        elapsed = time.perf_counter() - t0
        assert rc == _abi.GS_ERR_TIMEOUT
        assert b"iteration limit" in webgs.library().gs_last_error(ctx.handle)
        assert elapsed < 30.0
        # the same context still scans, sorts and renders correctly afterwards
        data = np.arange(10_000, dtype=np.uint32) % 7
        out, tot = ctx.exclusive_scan(data)
        assert tot == int(data.sum()) and out[-1] == tot - data[-1]
        keys = np.random.default_rng(0).integers(0, 2 ** 32, 5000, dtype=np.uint64).astype(np.uint32)
        k, _ = ctx.sort_pairs(keys, np.arange(5000, dtype=np.uint32))
        assert np.all(k[1:] >= k[:-1])
        packed = webgs.synth_scene(0, 1000, 1)
        sc = ctx.upload(packed, 1000)
        img = ctx.forward(sc, webgs.camera_view((0, 0, -4), (0, 0, 0), (0, 1, 0), 60.0, 64, 64))
        sc.close()
        assert img["rgba8"].shape == (64, 64, 4)


def test_invalid_arguments_are_reported_not_thrown(gpu_ctx):
    lib = webgs.library()
    img = _abi.Image(webgs.GS_MEM_HOST, None, None, None, None)
    assert lib.gs_forward(gpu_ctx.handle, None, None, None) == _abi.GS_ERR_INVALID
    with pytest.raises(webgs.GsError):
        gpu_ctx.upload(np.zeros(10, np.float32), 1)  # wrong size
    sc = gpu_ctx.upload(webgs.synth_scene(0, 10, 0), 10)
    try:
        big = webgs.camera_view((0, 0, -4), (0, 0, 0), (0, 1, 0), 60.0, 8192, 8192)  # 262144 tiles > 2^16
        import ctypes as C
        assert lib.gs_forward(gpu_ctx.handle, sc.handle, C.byref(big), C.byref(img)) == _abi.GS_ERR_INVALID
        assert b"16-bit tile field" in lib.gs_last_error(gpu_ctx.handle)
    finally:
        sc.close()
    with pytest.raises(webgs.GsError):
        webgs.Context(tile_size=12)
    with pytest.raises(webgs.GsError):
        webgs.Context(sort_block=1000)
