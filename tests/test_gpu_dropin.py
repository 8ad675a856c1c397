"""The drop-in path the reference app takes (main.js): loadPly -> Renderer.uploadGsData -> setGs ->
execute, with the reference's dirty-frame rule, resize and profiler rows, through libwebgs.so. The
frame equals the oracle's render of the same packed data and uniform block, bit for bit."""
import numpy as np
import pytest

import oracle
import webgs
from test_ply import REQUIRED, write_ply
from webgs import workloads as W

pytestmark = pytest.mark.gpu


def _ply_scene(n, seed):
    packed = W.SceneSpec(n, seed, 0).build()
    blocks = [(0, 3), (3, 3), (6, 4), (10, 3), (13, 1), (14, 45)]  # packed attribute blocks
    vals, names = {}, iter(REQUIRED)
    for off, width in blocks:
        blk = packed[off * n:(off + width) * n].reshape(n, width)
        for c in range(width):
            vals[next(names)] = blk[:, c]
    return write_ply([("float", k) for k in REQUIRED], vals, n), packed


def test_load_upload_set_execute_matches_oracle():
    n = 20_000
    data, packed = _ply_scene(n, 31)
    scene = webgs.load_ply(data)
    np.testing.assert_array_equal(scene["packed"], packed)
    rows = []
    r = webgs.Renderer(320, 240, on_profile=rows.append)
    try:
        r.upload_gs_data(scene, "garden")
        with pytest.raises(webgs.GsError):
            r.set_gs("missing")  # fail() on an unknown name
        r.set_gs("garden")
        assert r.execute(0.0)
        view = r.camera.get_uniform()
        o = oracle.forward_f32(webgs.view_bytes(view), packed, n)
        np.testing.assert_array_equal(r.image, o["rgba8"])
        assert rows and {"preprocess", "raster"} <= set(rows[-1])
        # nothing changed: no frame (renderer.js:489-493)
        assert not r.execute(0.016)
        # camera input marks the frame dirty
        r.camera.press("KeyW")
        assert r.execute(0.05)
        r.camera.release("KeyW")
        o2 = oracle.forward_f32(webgs.view_bytes(r.camera.get_uniform()), packed, n)
        np.testing.assert_array_equal(r.image, o2["rgba8"])
        # a resize renders again at the new size
        r.resize(200, 120)
        assert r.execute(0.0) and r.image.shape == (120, 200, 4)
        o3 = oracle.forward_f32(webgs.view_bytes(r.camera.get_uniform()), packed, n)
        np.testing.assert_array_equal(r.image, o3["rgba8"])
        # switching scenes renders the other scene
        r.upload_gs_data({"count": 5000, "packed": W.SceneSpec(5000, 32, 0).build()}, "other")
        r.set_gs("other")
        assert r.execute(0.0)
    finally:
        r.close()
