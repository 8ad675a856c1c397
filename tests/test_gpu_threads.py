"""Separate contexts are independent (the C ABI's contract): two host threads, each with its own
context, render different scenes concurrently through the C ABI, and every frame equals the
oracle's bit for bit."""
import threading

import pytest

import webgs
from webgs import workloads as W
from helpers import assert_frame_parity, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu


def test_two_contexts_on_two_threads():
    cases = []
    for seed, count, eye, (w, h) in ((21, 40_000, (0.0, 0.3, -3.6), (320, 240)),
                                      (22, 70_000, (0.5, -0.2, -4.2), (480, 270))):
        packed = W.SceneSpec(count, seed, 0).build()
        view = W.CameraSpec(eye, (0.0, 0.0, 0.0), 60.0, w, h).view()
        cases.append((packed, count, view, oracle_frame(view, packed, count)))
    errors = []

    def worker(packed, count, view, ref):
        try:
            with webgs.Context() as ctx:
                scene = ctx.upload(packed, count)
                try:
                    for _ in range(6):
                        assert_frame_parity(gpu_frame(ctx, scene, view), ref)
                finally:
                    scene.close()
        except Exception as exc:  # reported on the main thread
            errors.append(exc)

    threads = [threading.Thread(target=worker, args=c) for c in cases]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
