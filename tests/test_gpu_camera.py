"""The uniform builder on the device (gs_camera_views, gs_forward_batch_cameras) against the host's
gs_camera_view (Camera.getUniform(), camera.js:87-98, with lookAt / perspective of :135-142): the
176-byte blocks bit for bit, and a batch rendered from device-built blocks equal, bit for bit, to the
batch rendered from host-built ones."""
import math

import numpy as np
import pytest

import webgs
from webgs import workloads as W

pytestmark = pytest.mark.gpu


def _random_cameras(count, seed):
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(count):
        eye = rng.normal(0, 8, 3)
        target = rng.normal(0, 2, 3)
        up = (0.0, 1.0, 0.0) if rng.uniform() < 0.7 else tuple(rng.normal(0, 1, 3))
        fovy = float(rng.choice([rng.uniform(1.0, 179.0), 45.0, 60.0, 70.0, 90.0]))
        w, h = int(rng.integers(1, 4096)), int(rng.integers(1, 4096))
        near = float(rng.uniform(0.01, 1.0))
        cams.append((tuple(eye), tuple(target), tuple(up), fovy, w, h, near, near + float(rng.uniform(1, 1000))))
    return cams


def test_device_blocks_equal_host_blocks(gpu_ctx):
    params = _random_cameras(500, 1) + [(c.eye, c.target, (0.0, 1.0, 0.0), c.fovy, c.width, c.height, c.z_near,
                                         c.z_far) for _, c in W.orbit_cameras(16, 2024, 9.0)]
    dev = gpu_ctx.camera_views([webgs.make_camera(*p) for p in params])
    for p, v in zip(params, dev):
        assert webgs.view_bytes(v) == webgs.view_bytes(webgs.camera_view(*p)), p


def test_device_builder_rejects_bad_cameras(gpu_ctx):
    bad = webgs.make_camera((0, 0, -4), (0, 0, 0), (0, 1, 0), 180.0, 64, 64)
    with pytest.raises(webgs.GsError):
        gpu_ctx.camera_views([bad])


def test_batch_from_cameras_equals_batch_from_views():
    specs = [W.SceneSpec(20_000, 3, 1, 64, 20.0), W.SceneSpec(60_000, 4, 1, 64, 20.0)]
    packs = [s.build() for s in specs]
    cams = W.orbit_cameras(9, 23, 9.0, resolutions=((160, 120), (320, 180), (256, 256)))
    with webgs.Context() as ctx:
        sc = [ctx.upload(p, s.count) for s, p in zip(specs, packs)]
        ref = ctx.forward_batch([(sc[i % 2], c.view()) for i, c in cams], rgba8=True, rgb=True)
        for _ in range(2):  # the second call replays the cached graph
            out = ctx.forward_batch_cameras([(sc[i % 2], c.camera()) for i, c in cams], rgba8=True, rgb=True)
            for a, b in zip(out, ref):
                np.testing.assert_array_equal(a["rgb"].view(np.uint32), b["rgb"].view(np.uint32))
                np.testing.assert_array_equal(a["rgba8"], b["rgba8"])
        # an orbit that moves: new cameras, same graph, still the host blocks' frames
        moved = [(i, W.CameraSpec((c.eye[0] * math.cos(0.1), c.eye[1], c.eye[2]), c.target, c.fovy, c.width,
                                  c.height)) for i, c in cams]
        out = ctx.forward_batch_cameras([(sc[i % 2], c.camera()) for i, c in moved], rgba8=True, rgb=True)
        ref = ctx.forward_batch([(sc[i % 2], c.view()) for i, c in moved], rgba8=True, rgb=True)
        for a, b in zip(out, ref):
            np.testing.assert_array_equal(a["rgb"].view(np.uint32), b["rgb"].view(np.uint32))
        for s in sc:
            s.close()
