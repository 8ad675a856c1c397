"""GPU pipeline vs the CPU oracle: bit-exact binning (tilesTouched, meta, offsets, I, keys, values,
tile ranges) and pixels within 1e-4 max-abs (bit-exact under the pinned fp32 semantics), through
the C ABI (libwebgs.so)."""
import numpy as np
import pytest

import webgs
from webgs import workloads as W
from helpers import assert_frame_parity, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu


def _run(ctx, packed, count, view, tile=16, factor=64, allow_overflow=False):
    scene = ctx.upload(packed, count)
    try:
        g = gpu_frame(ctx, scene, view, allow_overflow=allow_overflow)
    finally:
        scene.close()
    o = oracle_frame(view, packed, count, tile=tile, factor=factor)
    return g, o


def test_small_config_parity(gpu_ctx):
    """The 50k-Gaussian, 512x512 configuration (seed 0)."""
    packed = W.SMALL_SCENE.build()
    g, o = _run(gpu_ctx, packed, W.SMALL_SCENE.count, W.SMALL_CAMERA.view())
    assert o["instance_count"] > 100_000
    assert_frame_parity(g, o)


def test_error_against_fp64_small_config(gpu_ctx):
    """The 50k / 512x512 frame against the FP64 twin of the algorithm: the error is rounding except
    at the discrete decisions (alpha below 1/255, the 1e-4 termination), where fp32 and FP64 can take
    different branches; measured: mean |err| 3.7e-7, PSNR 98 dB, max 3.3e-3."""
    import oracle

    packed = W.SMALL_SCENE.build()
    view = W.SMALL_CAMERA.view()
    scene = gpu_ctx.upload(packed, W.SMALL_SCENE.count)
    try:
        rgb = gpu_ctx.forward(scene, view, rgba8=False, rgb=True)["rgb"].astype(np.float64)
    finally:
        scene.close()
    r64 = oracle.forward_f64(webgs.view_bytes(view), packed, W.SMALL_SCENE.count)["rgb"]
    err = np.abs(rgb - r64)
    mse = np.mean((np.clip(rgb, 0, 1) - np.clip(r64, 0, 1)) ** 2)
    psnr = 10.0 * np.log10(1.0 / mse) if mse > 0 else np.inf
    assert err.mean() < 1e-5 and psnr > 90.0 and err.max() < 0.05, (err.mean(), psnr, err.max())


def test_cluster_scene_parity(gpu_ctx):
    """Cluster mixture inside a box, camera inside the box (a reduced scene-scale case)."""
    spec = W.SceneSpec(200_000, 11, 1, 64, 20.0)
    packed = spec.build()
    view = W.CameraSpec((0.0, 1.0, -9.0), (0.0, 0.0, 0.0), 70.0, 960, 540).view()
    g, o = _run(gpu_ctx, packed, spec.count, view)
    assert_frame_parity(g, o)


@pytest.mark.parametrize("w,h", [(1, 1), (17, 17), (1000, 7), (33, 250), (640, 480)])
def test_odd_image_sizes(gpu_ctx, w, h):
    packed = W.SceneSpec(3000, 5, 0).build()
    view = webgs.camera_view((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, w, h, 0.2, 100.0)
    g, o = _run(gpu_ctx, packed, 3000, view)
    assert_frame_parity(g, o)


@pytest.mark.parametrize("w,h", [(640, 480), (1280, 720), (2048, 1152), (3200, 1800)])
def test_tile_digit_widths(gpu_ctx, w, h):
    """The tile passes rank by matching the high half of a w-bit digit and separating the low w/2 bits
    by ballots (w/2 >= 2): the last tile digit is 3 bits wide here at 640x480 (1200 tiles, plain
    match), 4 at 1280x720 (split 2), 6 at 2048x1152 and 7 at 3200x1800 (split 3); the first tile digit
    takes split 4 throughout. Keys, values and pixels bit-exact against the oracle."""
    spec = W.SceneSpec(60_000, 13, 1, 16, 8.0)
    packed = spec.build()
    view = W.CameraSpec((0.0, 0.5, -5.0), (0.0, 0.0, 0.0), 70.0, w, h).view()
    g, o = _run(gpu_ctx, packed, spec.count, view)
    assert o["sorted_count"] > 100_000
    assert_frame_parity(g, o)


@pytest.mark.parametrize("count", [0, 1, 2, 33, 2047, 2048, 2049, 4097])
def test_counts_across_partition_edges(gpu_ctx, count):
    packed = W.SceneSpec(count, 7, 0).build() if count else np.zeros(0, np.float32)
    view = webgs.camera_view((0.0, 0.0, -3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, 128, 96, 0.2, 100.0)
    g, o = _run(gpu_ctx, packed, count, view)
    assert_frame_parity(g, o)


@pytest.mark.parametrize("tile", [8, 16, 32])
@pytest.mark.parametrize("digit_bits", [4, 8])
def test_tile_and_digit_configs(tile, digit_bits):
    packed = W.SceneSpec(20_000, 3, 0).build()
    view = W.CameraSpec((0.0, 0.5, -4.0), (0.0, 0.0, 0.0), 60.0, 300, 200).view()
    with webgs.Context(tile_size=tile, digit_bits=digit_bits) as ctx:
        g, o = _run(ctx, packed, 20_000, view, tile=tile)
    assert_frame_parity(g, o)


@pytest.mark.parametrize("digit_bits", [4, 8])
def test_small_sort_block_parity(digit_bits):
    """2048-key sort blocks (the autotuner's other block size) across many partitions."""
    spec = W.SceneSpec(100_000, 12, 1, 16, 8.0)
    view = W.CameraSpec((0.0, 0.5, -6.0), (0.0, 0.0, 0.0), 60.0, 640, 480).view()
    with webgs.Context(digit_bits=digit_bits, sort_block=2048) as ctx:
        g, o = _run(ctx, spec.build(), spec.count, view)
    assert o["sorted_count"] > 20 * 2048
    assert_frame_parity(g, o)


@pytest.mark.parametrize("batch", [32, 64, 128, 256])
def test_raster_batch_depths(batch):
    packed = W.SceneSpec(20_000, 4, 0).build()
    view = W.CameraSpec((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), 60.0, 256, 256).view()
    with webgs.Context(raster_batch=batch) as ctx:
        g, o = _run(ctx, packed, 20_000, view)
    assert_frame_parity(g, o)


def test_instance_overflow_truncates_like_reference():
    """factor 1: far more instances than slots; emit drops slots >= max_instance (emit.wgsl:57-59),
    the call reports GS_ERR_OVERFLOW and still writes the truncated frame."""
    packed = W.SceneSpec(5000, 8, 0).build()
    view = W.CameraSpec((0.0, 0.0, -2.5), (0.0, 0.0, 0.0), 60.0, 256, 256).view()
    with webgs.Context(max_instance_factor=1) as ctx:
        g, o = _run(ctx, packed, 5000, view, factor=1, allow_overflow=True)
        assert g.get("overflow")
        with pytest.raises(webgs.GsError) as ei:
            s = ctx.upload(packed, 5000)
            try:
                ctx.forward(s, view)
            finally:
                s.close()
        assert ei.value.code == 3
    assert o["instance_count"] > o["max_instance"] == 5000
    assert_frame_parity(g, o)


def test_equal_depth_ties_keep_gaussian_order(gpu_ctx):
    """All splats on one plane facing the camera: heavy depth16 ties; ties sort by Gaussian index."""
    n = 4000
    packed = W.SceneSpec(n, 9, 0).build()
    pos = packed[: 3 * n].reshape(n, 3)
    pos[:, 2] = 0.0
    view = W.CameraSpec((0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 60.0, 200, 200).view()
    g, o = _run(gpu_ctx, packed, n, view)
    assert_frame_parity(g, o)
    k, v = g["keys"], g["vals"]
    same = k[1:] == k[:-1]
    assert same.any() and (v[1:][same] > v[:-1][same]).all()


@pytest.mark.parametrize("seed", [21, 22])
def test_needle_splats_parity(gpu_ctx, seed):
    """Very anisotropic splats (one long axis, two thin ones, random orientation, high opacity): the
    thin rotated ellipses stress the warp cull, whose skipped splats must be exactly those every pixel
    of the warp rejects."""
    n = 20_000
    rng = np.random.default_rng(seed)
    packed = W.SceneSpec(n, seed, 0).build()
    scale = packed[3 * n: 6 * n].reshape(n, 3)
    scale[:] = np.log(rng.uniform(0.0005, 0.004, (n, 3))).astype(np.float32)
    scale[np.arange(n), rng.integers(0, 3, n)] = np.log(rng.uniform(0.02, 0.25, n)).astype(np.float32)
    packed[13 * n: 14 * n] = rng.uniform(1.0, 6.0, n).astype(np.float32)  # opacity logits
    view = W.CameraSpec((0.3, -0.2, -3.5), (0.0, 0.0, 0.0), 60.0, 480, 320).view()
    g, o = _run(gpu_ctx, packed, n, view)
    assert o["max_instance"] > o["instance_count"] > 200_000
    assert_frame_parity(g, o)


def test_pinned_host_output_is_written_directly(gpu_ctx):
    """Host images in pinned memory are written by the raster itself (no staging copy): same bytes
    as through the pageable path, for a single frame and for a batch."""
    import ctypes as C

    import torch

    from webgs import _abi

    packed = W.SMALL_SCENE.build()
    view = W.SMALL_CAMERA.view()
    scene = gpu_ctx.upload(packed, W.SMALL_SCENE.count)
    try:
        ref = gpu_ctx.forward(scene, view, rgba8=True, rgb=True)
        h8 = torch.zeros(512 * 512 * 4, dtype=torch.uint8, pin_memory=True)
        hrgb = torch.zeros(512 * 512 * 3, dtype=torch.float32, pin_memory=True)
        img = _abi.Image(webgs.GS_MEM_HOST, h8.data_ptr(), hrgb.data_ptr(), None, None)
        assert webgs.library().gs_forward(gpu_ctx.handle, scene.handle, C.byref(view), C.byref(img)) == 0
        np.testing.assert_array_equal(h8.numpy().reshape(512, 512, 4), ref["rgba8"])
        np.testing.assert_array_equal(hrgb.numpy().reshape(512, 512, 3).view(np.uint32), ref["rgb"].view(np.uint32))
        arr = (_abi.BatchView * 2)()
        outs = [torch.zeros(512 * 512 * 4, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        for k in range(2):
            arr[k].scene = scene.handle
            arr[k].view = view
            arr[k].out = _abi.Image(webgs.GS_MEM_HOST, outs[k].data_ptr(), None, None, None)
        assert webgs.library().gs_forward_batch(gpu_ctx.handle, arr, 2) == 0
        for o in outs:
            np.testing.assert_array_equal(o.numpy().reshape(512, 512, 4), ref["rgba8"])
    finally:
        scene.close()


def test_repeat_frames_are_deterministic(gpu_ctx):
    packed = W.SceneSpec(30_000, 10, 0).build()
    view = W.CameraSpec((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), 60.0, 320, 240).view()
    scene = gpu_ctx.upload(packed, 30_000)
    try:
        a = gpu_frame(gpu_ctx, scene, view)
        b = gpu_frame(gpu_ctx, scene, view)
    finally:
        scene.close()
    for key in ("keys", "vals", "ranges", "rgba8"):
        np.testing.assert_array_equal(a[key], b[key])
    np.testing.assert_array_equal(a["rgb"].view(np.uint32), b["rgb"].view(np.uint32))


@pytest.mark.parametrize("flags", [webgs.GS_FLAG_NO_GRAPH, webgs.GS_FLAG_PROFILE])
def test_eager_launches_match_oracle(flags):
    """Frames launched eagerly (no graph; and the profiling context, with events between the passes)
    chain their kernels as programmatic dependent launches, as the captured graph does: the result is
    the oracle's, bit for bit, on repeated frames."""
    packed = W.SceneSpec(60_000, 12, 0).build()
    view = W.CameraSpec((0.3, 0.2, -3.8), (0.0, 0.0, 0.0), 60.0, 400, 300).view()
    o = oracle_frame(view, packed, 60_000)
    with webgs.Context(flags=flags) as ctx:
        scene = ctx.upload(packed, 60_000)
        try:
            for _ in range(3):
                assert_frame_parity(gpu_frame(ctx, scene, view), o)
        finally:
            scene.close()


def test_scene_scale_config_parity(gpu_ctx):
    """1M Gaussians, 64-cluster mixture in a 20^3 box, 1920x1080, camera inside the box."""
    packed = W.SCENE_1M.build()
    g, o = _run(gpu_ctx, packed, W.SCENE_1M.count, W.CAMERA_1080P.view())
    assert_frame_parity(g, o)


def _golden():
    import json
    from pathlib import Path

    return json.loads((Path(__file__).parent / "golden" / "oracle_fixtures.json").read_text())


@pytest.mark.parametrize("case", _golden(), ids=[c["name"] for c in _golden()])
def test_gpu_matches_committed_fixtures(case):
    """The GPU frame reproduces the committed digests (no CPU oracle run needed on the GPU host)."""
    import hashlib

    def digest(a):
        return hashlib.sha256(memoryview(np.ascontiguousarray(a)).cast("B")).hexdigest()

    kind, count, seed, clusters, box = case["scene"]
    packed = webgs.synth_scene(kind, count, seed, clusters, box)
    assert digest(packed) == case["scene_digest"]
    view = webgs.view_from_bytes(bytes.fromhex(case["view_hex"]))
    with webgs.Context(tile_size=case["tile"], max_instance_factor=case["factor"]) as ctx:
        scene = ctx.upload(packed, count)
        out = ctx.forward(scene, view, rgba8=True, rgb=True, allow_overflow=True)
        dbg = ctx.debug()
        scene.close()
    assert dbg["instance_count"] == case["instance_count"] and dbg["sorted_count"] == case["sorted_count"]
    assert digest(dbg["keys"]) == case["keys"] and digest(dbg["vals"]) == case["vals"]
    assert digest(dbg["ranges"]) == case["ranges"]
    assert digest(out["rgb"]) == case["rgb"] and digest(out["rgba8"]) == case["rgba8"]
