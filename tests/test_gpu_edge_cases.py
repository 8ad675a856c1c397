"""Edge cases through the C ABI: a frame in which nothing is visible (every Gaussian behind the
camera: no instances, all ranges empty, a black opaque image), a batch that mixes an empty scene with
ordinary ones, and the batch-by-cameras entry point's argument checks."""
import numpy as np
import pytest

import webgs
from webgs import workloads as W
from helpers import assert_frame_parity, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu


def test_nothing_visible(gpu_ctx):
    spec = W.SceneSpec(20_000, 14, 0)
    packed = spec.build()
    # the camera looks away from the cluster at the origin: every Gaussian is behind the near plane
    view = webgs.camera_view((0.0, 0.0, -6.0), (0.0, 0.0, -12.0), (0.0, 1.0, 0.0), 60.0, 200, 150, 0.2, 100.0)
    sc = gpu_ctx.upload(packed, spec.count)
    try:
        g = gpu_frame(gpu_ctx, sc, view)
    finally:
        sc.close()
    o = oracle_frame(view, packed, spec.count)
    assert g["instance_count"] == 0 and g["sorted_count"] == 0 and g["visible"] == 0
    assert not g["ranges"].any()
    assert np.all(g["rgba8"][..., :3] == 0) and np.all(g["rgba8"][..., 3] == 255)
    assert np.all(g["final_t"] == 1.0)
    assert_frame_parity(g, o)


def test_batch_with_an_empty_scene():
    spec = W.SceneSpec(30_000, 15, 1, 16, 12.0)
    packed = spec.build()
    cams = [c for _, c in W.orbit_cameras(3, 7, 8.0, resolutions=((160, 120), (320, 180)))]
    with webgs.Context() as ctx:
        sc = ctx.upload(packed, spec.count)
        empty = ctx.upload(np.zeros(0, np.float32), 0)
        items = [(sc, cams[0].view()), (empty, cams[1].view()), (sc, cams[2].view()), (empty, cams[0].view())]
        outs = ctx.forward_batch(items, rgba8=True, rgb=True)
        for k, ((scene, view), out) in enumerate(zip(items, outs)):
            single = ctx.forward(scene, view, rgba8=True, rgb=True)
            np.testing.assert_array_equal(out["rgb"].view(np.uint32), single["rgb"].view(np.uint32))
            np.testing.assert_array_equal(out["rgba8"], single["rgba8"])
            if scene is empty:
                assert ctx.batch_frame_info(k)["instance_count"] == 0 and not out["rgb"].any()
        sc.close()
        empty.close()


def test_batch_by_cameras_rejects_bad_arguments():
    spec = W.SceneSpec(2_000, 16, 0)
    with webgs.Context() as ctx:
        sc = ctx.upload(spec.build(), spec.count)
        good = webgs.make_camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 64, 48)
        for bad in (webgs.make_camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 0.0, 64, 48),
                    webgs.make_camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 0, 48),
                    webgs.make_camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 64, 48, 1.0, 0.5)):
            with pytest.raises(webgs.GsError) as ei:
                ctx.forward_batch_cameras([(sc, good), (sc, bad)])
            assert ei.value.code == webgs._abi.GS_ERR_INVALID
        # the context is still usable, and a good batch matches the single frame
        out = ctx.forward_batch_cameras([(sc, good)], rgba8=True, rgb=True)[0]
        single = ctx.forward(sc, webgs.camera_view((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 64, 48),
                             rgba8=True, rgb=True)
        np.testing.assert_array_equal(out["rgb"].view(np.uint32), single["rgb"].view(np.uint32))
        assert webgs.library().gs_forward_batch_cameras(ctx.handle, None, 0) == webgs._abi.GS_ERR_INVALID
        sc.close()
