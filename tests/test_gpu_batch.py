"""Batched multi-view rendering (one CUDA graph over many views and scenes) and the autotuner,
through the C ABI: every batched view equals the single-view frame bit for bit (and so the oracle),
batched gradients equal the sum of single-view gradients."""
import numpy as np
import pytest

import oracle
import webgs
from webgs import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes():
    specs = [W.SceneSpec(20_000, 3, 1, 64, 20.0), W.SceneSpec(60_000, 4, 1, 64, 20.0),
             W.SceneSpec(150_000, 5, 1, 64, 20.0)]
    return specs, [s.build() for s in specs]


def test_batch_equals_single_views(scenes):
    specs, packs = scenes
    cams = W.orbit_cameras(7, 11, 9.0, resolutions=((160, 120), (320, 180), (256, 256)))
    with webgs.Context() as ctx:
        sc = [ctx.upload(p, s.count) for s, p in zip(specs, packs)]
        items = [(sc[i], cam.view()) for i, cam in cams]
        batch = ctx.forward_batch(items, rgba8=True, rgb=True)
        infos = [ctx.batch_frame_info(k) for k in range(len(items))]
        again = ctx.forward_batch(items, rgba8=True, rgb=True)  # graph replay
        for k, ((scene, view), b, b2, info) in enumerate(zip(items, batch, again, infos)):
            single = ctx.forward(scene, view, rgba8=True, rgb=True)
            np.testing.assert_array_equal(b["rgb"].view(np.uint32), single["rgb"].view(np.uint32))
            np.testing.assert_array_equal(b["rgba8"], single["rgba8"])
            np.testing.assert_array_equal(b2["rgb"].view(np.uint32), b["rgb"].view(np.uint32))
            assert info["instance_count"] == ctx.frame_info()["instance_count"]
        for s in sc:
            s.close()
    # one batched view against the oracle directly
    i, cam = cams[0]
    o = oracle.forward_f32(webgs.view_bytes(cam.view()), packs[i], specs[i].count)
    np.testing.assert_array_equal(batch[0]["rgb"].view(np.uint32), o["rgb"].view(np.uint32))


def test_batch_of_twenty_views_of_one_scene(scenes):
    """More views than side streams and than one shared preprocess takes (16): the scene's views
    are preprocessed in two groups and four streams carry two views each; every view equals its
    single frame bit for bit."""
    specs, packs = scenes
    cams = W.orbit_cameras(20, 17, 9.0, resolutions=((96, 64), (128, 96)))
    with webgs.Context() as ctx:
        sc = ctx.upload(packs[1], specs[1].count)
        items = [(sc, cam.view()) for _, cam in cams]
        batch = ctx.forward_batch(items, rgba8=True, rgb=True)
        for (scene, view), b in zip(items, batch):
            single = ctx.forward(scene, view, rgba8=True, rgb=True)
            np.testing.assert_array_equal(b["rgb"].view(np.uint32), single["rgb"].view(np.uint32))
            np.testing.assert_array_equal(b["rgba8"], single["rgba8"])
        sc.close()


@pytest.mark.parametrize("views,w,h", [(3, 256, 192), (18, 96, 64)])
def test_batch_backward_is_sum_of_views(views, w, h):
    """The batched backward (one preprocess backward per group of up to 16 views, the later groups
    added to the first) equals the sum of the single-view gradients."""
    spec = W.SceneSpec(30_000, 6, 1, 64, 20.0)
    packed = spec.build()
    cams = [c for _, c in W.orbit_cameras(views, 5, 9.0, fixed_resolution=(w, h))]
    rng = np.random.default_rng(0)
    dls = [rng.normal(0, 1e-3, (h, w, 3)).astype(np.float32) for _ in cams]
    with webgs.Context(flags=webgs.GS_FLAG_DIFFERENTIABLE) as ctx:
        sc = ctx.upload(packed, spec.count)
        ctx.forward_batch([(sc, c.view()) for c in cams], rgba8=False, rgb=True)
        g_batch = ctx.backward_batch(sc, dls)
        g_sum = np.zeros_like(g_batch, dtype=np.float64)
        for c, dl in zip(cams, dls):
            ctx.forward(sc, c.view(), rgba8=False)
            g_sum += ctx.backward(sc, dl)
        sc.close()
    err = np.linalg.norm(g_batch - g_sum) / np.linalg.norm(g_sum)
    assert err < 1e-5, err


def test_autotune_picks_a_valid_configuration():
    spec = W.SceneSpec(20_000, 7, 0)
    views = [W.CameraSpec((0.0, 0.0, -4.0), (0, 0, 0), 60.0, 320, 240).view()]
    cfg, ms = webgs.autotune(spec.build(), spec.count, views, iters=2)
    assert cfg["tile_size"] in (8, 16, 32) and cfg["digit_bits"] in (4, 8)
    assert cfg["raster_batch"] in (32, 64, 128, 256) and cfg["sort_block"] in (2048, 4096) and ms > 0
    with webgs.Context(**cfg) as ctx:  # the pick is a configuration a context accepts
        assert ctx.config.sort_block == cfg["sort_block"]


def _batch_ms(cfg: dict, items_spec, packs, reps: int = 30) -> float:
    """Best of three timings of `reps` device-output batches (wall clock around a synchronized queue
    of launches; the queue keeps the GPU busy, so this is the device time per batch)."""
    import time

    import torch

    specs, cams = items_spec
    with webgs.Context(**cfg) as ctx:
        scs = [ctx.upload(p, s.count) for s, p in zip(specs, packs)]
        imgs = [torch.empty(c.width * c.height, dtype=torch.int32, device="cuda") for _, c in cams]
        arr = (webgs._abi.BatchView * len(cams))()
        for k, (si, c) in enumerate(cams):
            arr[k].scene = scs[si].handle
            arr[k].view = c.view()
            arr[k].out = webgs._abi.Image(webgs.GS_MEM_DEVICE, imgs[k].data_ptr(), None, None, None)
        lib = webgs.library()
        best = float("inf")
        for _ in range(3):
            for _ in range(3):
                ctx._ck(lib.gs_forward_batch(ctx.handle, arr, len(cams)))
            ctx.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                ctx._ck(lib.gs_forward_batch(ctx.handle, arr, len(cams)))
            ctx.synchronize()
            best = min(best, (time.perf_counter() - t0) / reps * 1e3)
        for sc in scs:
            sc.close()
    return best


def test_autotune_pick_is_not_slower_than_the_defaults():
    """The pick re-timed on the batch it was tuned on: no slower than the default configuration (5%
    allowance for run-to-run noise; the sweep's last stage already re-times its three best
    candidates with four times as many batches)."""
    specs = [W.SceneSpec(150_000, 5, 1, 64, 20.0), W.SceneSpec(400_000, 4, 1, 64, 20.0)]
    packs = [s.build() for s in specs]
    cams = [(i % 2, c) for i, (_, c) in enumerate(W.orbit_cameras(6, 31, 9.0))]
    cfg, _ = webgs.autotune_scenes([(p, s.count) for s, p in zip(specs, packs)], [c.view() for _, c in cams],
                                   [si for si, _ in cams], iters=3)
    # interleaved, the best of two each, so that a drift of the clock between the two does not land
    # on one side only
    runs = [_batch_ms(c, (specs, cams), packs) for c in (cfg, {}, cfg, {})]
    tuned, default = min(runs[0::2]), min(runs[1::2])
    assert tuned <= default * 1.05, (cfg, tuned, default)


def test_autotune_over_several_scenes():
    specs = [W.SceneSpec(8_000, 7, 0), W.SceneSpec(12_000, 8, 1, 16, 8.0)]
    scenes = [(s.build(), s.count) for s in specs]
    views = [W.CameraSpec((0.0, 0.0, -4.0), (0, 0, 0), 60.0, 160, 120).view(),
             W.CameraSpec((0.0, 0.5, -6.0), (0, 0, 0), 60.0, 200, 100).view(),
             W.CameraSpec((1.0, 0.0, -5.0), (0, 0, 0), 70.0, 96, 96).view()]
    cfg, ms = webgs.autotune_scenes(scenes, views, [0, 1, 1], iters=1)
    assert cfg["tile_size"] in (8, 16, 32) and cfg["digit_bits"] in (4, 8) and ms > 0
    with pytest.raises(webgs.GsError):
        webgs.autotune_scenes(scenes, views, [0, 1, 2], iters=1)  # scene index out of range
