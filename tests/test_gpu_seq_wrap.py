"""Lookback-word tags across their wrap, through the C ABI.

Every lookback word carries the low 30 bits of its frame's sequence number, which advances by 16 per
frame or scan, so the tags repeat every 2^26 calls. The call whose tags start again at zero clears the
words first; without that, a word left from 2^26 calls earlier would read as published by the current
call. gs_debug_set_sequence puts the sequence just below the wrap, and each test first plants words
with tag 0 from a different input (a call made right after a wrap), then runs a call that does not
overwrite them, then the call that wraps again: its results must match an ordinary call's.
"""
import numpy as np
import pytest

import webgs
from webgs import workloads as W

pytestmark = pytest.mark.gpu

WRAP_NEXT = 0xFFFFFFF0          # the next call's sequence number is 0: tags 0..15
BELOW_WRAP = (1 << 30) - 32     # the next call's tags are 2^30 - 16 .. 2^30 - 1; the one after wraps


def _cumsum_excl(data: np.ndarray) -> tuple[np.ndarray, int]:
    c = np.cumsum(data.astype(np.uint64))
    excl = np.concatenate([[0], c[:-1]]).astype(np.uint64) if data.size else np.zeros(0, np.uint64)
    return (excl & 0xFFFFFFFF).astype(np.uint32), int(c[-1] & 0xFFFFFFFF) if data.size else 0


def test_context_scan_across_the_wrap(gpu_ctx):
    rng = np.random.default_rng(31)
    n = 3_000_001
    planted = rng.integers(0, 1000, n).astype(np.uint32)
    small = rng.integers(0, 1000, 1000).astype(np.uint32)
    data = rng.integers(0, 300, n).astype(np.uint32)
    gpu_ctx.set_sequence(WRAP_NEXT)
    for d in (planted, small, data):  # tag 0 (plants), tag 2^30 - 16 (one word), tag 0 again
        if d is small:
            gpu_ctx.set_sequence(BELOW_WRAP)
        out, tot = gpu_ctx.exclusive_scan(d)
        ref, rtot = _cumsum_excl(d)
        np.testing.assert_array_equal(out, ref)
        assert tot == rtot


def test_context_sort_across_the_wrap(gpu_ctx):
    rng = np.random.default_rng(32)
    n = 2_000_000
    planted = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    gpu_ctx.set_sequence(WRAP_NEXT)
    gpu_ctx.sort_pairs(planted, vals, 32)
    gpu_ctx.set_sequence(BELOW_WRAP)
    gpu_ctx.sort_pairs(keys[:100], vals[:100], 32)
    k, v = gpu_ctx.sort_pairs(keys, vals, 32)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(k, keys[order])
    np.testing.assert_array_equal(v, vals[order])


def test_frames_across_the_wrap():
    spec = W.SceneSpec(200_000, 12, 1, 32, 12.0)
    packed = spec.build()
    tiny = W.SceneSpec(64, 13, 0).build()
    v1 = W.CameraSpec((0.0, 1.0, -8.0), (0.0, 0.0, 0.0), 70.0, 640, 480).view()
    v2 = W.CameraSpec((3.0, -1.0, -7.0), (0.5, 0.0, 0.0), 60.0, 800, 600).view()
    with webgs.Context() as ctx:
        sc = ctx.upload(packed, spec.count)
        sc_tiny = ctx.upload(tiny, 64)
        ref = ctx.forward(sc, v1, rgba8=True, rgb=True)
        ref_info = ctx.frame_info()
        ref_batch = ctx.forward_batch([(sc, v1), (sc, v2)], rgba8=True, rgb=True)

        ctx.set_sequence(WRAP_NEXT)
        ctx.forward(sc, v2, rgba8=True)                       # plants tag-0 words of another view
        ctx.forward_batch([(sc, v2), (sc, v1)], rgba8=True)   # the batch frames too, views swapped
        ctx.set_sequence(BELOW_WRAP)
        ctx.forward(sc_tiny, v1, rgba8=True)                  # overwrites a few words only
        ctx.forward_batch([(sc_tiny, v1), (sc_tiny, v2)], rgba8=True)
        out = ctx.forward(sc, v1, rgba8=True, rgb=True)       # tags 0.. again: cleared first
        info = ctx.frame_info()
        out_batch = ctx.forward_batch([(sc, v1), (sc, v2)], rgba8=True, rgb=True)
        sc.close()
        sc_tiny.close()
    assert info["status"] == 0 and info["instance_count"] == ref_info["instance_count"]
    np.testing.assert_array_equal(out["rgb"].view(np.uint32), ref["rgb"].view(np.uint32))
    np.testing.assert_array_equal(out["rgba8"], ref["rgba8"])
    for a, b in zip(out_batch, ref_batch):
        np.testing.assert_array_equal(a["rgb"].view(np.uint32), b["rgb"].view(np.uint32))
