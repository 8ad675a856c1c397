"""Parity at the benchmark configurations' full sizes, through the C ABI, against the CPU oracle.

  differentiation workload  500k Gaussians (seed 2), 1280x720: the forward frame bit for bit
                            (binning, per-Gaussian records, rgb, final T, contributor counts, rgba8).
  batched forward           the bench's exact batch: scenes of 100k / 400k / 1.5M Gaussians (seeds
                            3-5) and 16 orbit cameras (seed 2024) at 640x480 .. 1920x1080, one
                            gs_forward_batch; every view's rgb and rgba8 bit for bit, and its
                            instance counts.
  batched forward+backward  3M Gaussians (seed 6, 128 clusters, 40^3 box), 8 orbit views at
                            1920x1080 in one batch: every view bit for bit; the batched backward
                            (views summed on the device) against the sum of eight single-view
                            backwards, per parameter group relative L2 <= 1e-5 (both are fp32 sums
                            of atomics in different orders); view 0's gradient against the FP64
                            adjoint: relative L2 <= 1e-2 per group and cosine >= 0.9999. The
                            bound is wider than the 2e-3 of the 500k / 720p case because these
                            views stack more splats per pixel, so more pixels take a different
                            branch in fp32 and FP64 at the 1/255 and 1e-4 thresholds (measured:
                            3.6e-3 on the SH DC group, cosine 0.999993).
"""
import numpy as np
import pytest

import oracle
import webgs
from webgs import workloads as W
from helpers import assert_frame_parity, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu

GROUPS = ("means", "log-scales", "quaternions", "sh-dc", "opacity", "sh-rest")


def _groups(n):
    return {"means": (0, 3 * n), "log-scales": (3 * n, 6 * n), "quaternions": (6 * n, 10 * n),
            "sh-dc": (10 * n, 13 * n), "opacity": (13 * n, 14 * n), "sh-rest": (14 * n, 59 * n)}


def test_differentiation_config_forward_parity():
    spec, cam = W.SCENE_500K, W.CAMERA_720P
    packed = spec.build()
    view = cam.view()
    with webgs.Context() as ctx:
        sc = ctx.upload(packed, spec.count)
        try:
            g = gpu_frame(ctx, sc, view)
        finally:
            sc.close()
    o = oracle_frame(view, packed, spec.count)
    assert o["instance_count"] > 500_000
    assert_frame_parity(g, o)


def _assert_view(out: dict, info: dict, view, packed, count):
    o = oracle.forward_f32(webgs.view_bytes(view), packed, count, keys=False)
    assert info["instance_count"] == o["instance_count"] and info["sorted_count"] == o["sorted_count"]
    assert info["status"] == 0
    np.testing.assert_array_equal(out["rgb"].view(np.uint32), o["rgb"].view(np.uint32))
    np.testing.assert_array_equal(out["rgba8"], o["rgba8"])


def test_batched_forward_workload_every_view():
    packs = [s.build() for s in W.BATCH_SCENES]
    cams = W.orbit_cameras(16, 2024, 9.0)
    with webgs.Context() as ctx:
        scs = [ctx.upload(p, s.count) for s, p in zip(W.BATCH_SCENES, packs)]
        items = [(scs[si], c.view()) for si, c in cams]
        outs = ctx.forward_batch(items, rgba8=True, rgb=True)
        infos = [ctx.batch_frame_info(k) for k in range(len(items))]
        for s in scs:
            s.close()
    assert {c.width for _, c in cams} == {640, 1280, 1920}
    for (si, cam), out, info in zip(cams, outs, infos):
        _assert_view(out, info, cam.view(), packs[si], W.BATCH_SCENES[si].count)


def test_3m_scene_eight_1080p_views_forward_and_backward():
    spec = W.SCENE_3M
    n = spec.count
    packed = spec.build()
    cams = [c for _, c in W.orbit_cameras(8, 77, 18.0, fixed_resolution=(1920, 1080))]
    views = [c.view() for c in cams]
    with webgs.Context(flags=webgs.GS_FLAG_DIFFERENTIABLE) as ctx:
        ts = ctx.upload(webgs.perturb_scene(packed, n, 99, 0.01, 0.02), n)
        targets = [ctx.forward(ts, v, rgba8=False, rgb=True)["rgb"] for v in views]
        ts.close()
        sc = ctx.upload(packed, n)
        outs = ctx.forward_batch([(sc, v) for v in views], rgba8=True, rgb=True)
        infos = [ctx.batch_frame_info(k) for k in range(len(views))]
        dls = [ctx.loss(o["rgb"], t, 0.2)[1] for o, t in zip(outs, targets)]
        g_batch = ctx.backward_batch(sc, dls)
        g_seq = np.zeros(59 * n, np.float64)
        g_view0 = None
        for k, (v, dl) in enumerate(zip(views, dls)):
            ctx.forward(sc, v, rgba8=False)
            g = ctx.backward(sc, dl)
            g_seq += g
            if k == 0:
                g_view0 = g
        sc.close()
    for v, out, info in zip(views, outs, infos):
        _assert_view(out, info, v, packed, n)
    for name, (a, b) in _groups(n).items():
        y = g_seq[a:b]
        rel = np.linalg.norm(g_batch[a:b] - y) / np.linalg.norm(y)
        assert rel <= 1e-5, (name, rel)
    g64, _ = oracle.backward_f64(webgs.view_bytes(views[0]), packed, n, dls[0])
    report = {}
    for name, (a, b) in _groups(n).items():
        x, y = g_view0[a:b].astype(np.float64), g64[a:b]
        ny = np.linalg.norm(y)
        report[name] = (float(np.linalg.norm(x - y) / ny), float(x @ y / (np.linalg.norm(x) * ny)))
    print("3M view 0 vs FP64 adjoint (rel L2, cosine):", report)
    for name, (rel, cos) in report.items():
        assert rel <= 1e-2 and cos >= 0.9999, (name, rel, cos, report)
