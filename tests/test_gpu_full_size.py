"""Full-size frames checked through properties that do not need the oracle: the 3M-Gaussian scene
(128 clusters in a 40^3 box) at 1920x1080 and the 1M scene at 3840x2160. The offsets are the
exclusive scan of tilesTouched, the keys are sorted with equal keys in ascending Gaussian order, each
instance's key is its Gaussian's tile and depth16 (emit order within a rect), the tile ranges are the
runs of equal tiles, and the image is finite and opaque."""
import numpy as np
import pytest

import webgs
from webgs import workloads as W

pytestmark = pytest.mark.gpu


def _check(ctx, scene, view, w, h):
    out = ctx.forward(scene, view, rgba8=True, rgb=True)
    d = ctx.debug()
    counts = d["tiles_touched"].astype(np.int64)
    off = d["offsets"].astype(np.int64)
    assert off[0] == 0 and np.array_equal(np.diff(off), counts)
    I = int(off[-1])
    assert d["instance_count"] == I and d["sorted_count"] == min(I, d["max_instance"])
    S = d["sorted_count"]
    keys = d["keys"][:S].astype(np.int64)
    vals = d["vals"][:S].astype(np.int64)
    assert np.all(np.diff(keys) >= 0), "keys not sorted"
    same = np.diff(keys) == 0
    assert np.all(np.diff(vals)[same] > 0), "equal keys out of Gaussian order"
    # every instance of Gaussian g carries g's depth16 and a tile of g's rect
    meta = d["meta"].reshape(-1, 4).astype(np.int64)
    m = meta[vals]
    tile = keys >> 16
    tx_n = d["tiles_x"]
    tx, ty = tile % tx_n, tile // tx_n
    assert np.array_equal(keys & 0xFFFF, m[:, 2] & 0xFFFF)
    assert np.all((tx >= (m[:, 0] & 0xFFFF)) & (tx <= (m[:, 1] & 0xFFFF)))
    assert np.all((ty >= (m[:, 0] >> 16)) & (ty <= (m[:, 1] >> 16)))
    # each Gaussian appears once per tile of its rect
    np.testing.assert_array_equal(np.bincount(vals, minlength=len(counts)), counts)
    # ranges are the runs of equal tiles
    T = d["tiles_x"] * d["tiles_y"]
    ranges = d["ranges"].reshape(T, 2).astype(np.int64)
    starts = np.searchsorted(tile, np.arange(T), side="left")
    ends = np.searchsorted(tile, np.arange(T), side="right")
    nonempty = ends > starts
    np.testing.assert_array_equal(ranges[nonempty, 0], starts[nonempty])
    np.testing.assert_array_equal(ranges[nonempty, 1], ends[nonempty])
    assert np.all(ranges[~nonempty] == 0)
    rgb = out["rgb"]
    assert rgb.shape == (h, w, 3) and np.isfinite(rgb).all() and rgb.min() >= 0.0
    assert np.all(out["rgba8"][..., 3] == 255)
    return S


def test_3m_scene_1080p():
    spec = W.SCENE_3M
    packed = spec.build()
    view = W.CameraSpec((0.0, 2.0, -18.0), (0.0, 0.0, 0.0), 70.0, 1920, 1080).view()
    with webgs.Context() as ctx:
        scene = ctx.upload(packed, spec.count)
        try:
            assert _check(ctx, scene, view, 1920, 1080) > 1_000_000
        finally:
            scene.close()


def test_1m_scene_4k():
    spec = W.SCENE_1M
    packed = spec.build()
    view = W.CameraSpec((0.0, 1.0, -9.0), (0.0, 0.0, 0.0), 70.0, 3840, 2160).view()
    with webgs.Context() as ctx:
        scene = ctx.upload(packed, spec.count)
        try:
            assert _check(ctx, scene, view, 3840, 2160) > 2_000_000
        finally:
            scene.close()
