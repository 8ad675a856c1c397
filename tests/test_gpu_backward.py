"""CUDA backward and loss vs the FP64 oracle, through the C ABI: the L1 + SSIM loss and its image
gradient, and dL/d(attributes) of the splat pipeline against the FP64 adjoint fed the same dL/drgb.

Tolerances (fp32 kernels with atomics and T recovered by division, against FP64):
  loss value 1e-5 absolute, dL/drgb 1e-4 of its largest entry;
  per parameter group ||g32 - g64|| <= 2e-3 ||g64|| and cosine similarity >= 0.9999."""
import numpy as np
import pytest

import oracle
import webgs
from webgs import workloads as W

pytestmark = pytest.mark.gpu
LAMBDA = 0.2


def _groups(n):
    return {"means": (0, 3 * n), "log-scales": (3 * n, 6 * n), "quaternions": (6 * n, 10 * n),
            "sh-dc": (10 * n, 13 * n), "opacity": (13 * n, 14 * n), "sh-rest": (14 * n, 59 * n)}


def _compare(g32, g64, n, tol=2e-3):
    report = {}
    for name, (a, b) in _groups(n).items():
        x, y = g32[a:b].astype(np.float64), g64[a:b]
        ny = np.linalg.norm(y)
        assert ny > 0, name
        rel = np.linalg.norm(x - y) / ny
        cos = float(x @ y / (np.linalg.norm(x) * ny))
        report[name] = (rel, cos)
        assert rel <= tol and cos >= 0.9999, (name, rel, cos)
    return report


@pytest.mark.parametrize("w,h", [(96, 80), (1280, 720)])
def test_loss_matches_oracle(gpu_ctx, w, h):
    rng = np.random.default_rng(w)
    x = rng.uniform(0, 1, (h, w, 3)).astype(np.float32)
    y = np.clip(x + rng.normal(0, 0.1, x.shape), 0, 1).astype(np.float32)
    val, dl = gpu_ctx.loss(x, y, LAMBDA)
    rval, rdl = oracle.loss_l1_ssim(x, y, LAMBDA)
    assert abs(val - rval) < 1e-5
    assert np.abs(dl - rdl).max() <= 1e-4 * np.abs(rdl).max()


def _fwd_bwd_case(spec, cam, tile=16):
    packed = spec.build()
    target_scene = webgs.perturb_scene(packed, spec.count, 99, 0.01, 0.02)
    view = cam.view()
    with webgs.Context(flags=webgs.GS_FLAG_DIFFERENTIABLE, tile_size=tile) as ctx:
        ts = ctx.upload(target_scene, spec.count)
        target = ctx.forward(ts, view, rgba8=False, rgb=True)["rgb"]
        ts.close()
        sc = ctx.upload(packed, spec.count)
        rgb = ctx.forward(sc, view, rgba8=False, rgb=True)["rgb"]
        loss, dl = ctx.loss(rgb, target, LAMBDA)
        g32 = ctx.backward(sc, dl)
        sc.close()
    g64, rgb64 = oracle.backward_f64(webgs.view_bytes(view), packed, spec.count, dl, tile=tile)
    return g32, g64, rgb, rgb64, loss


def test_backward_small_scene():
    g32, g64, rgb, rgb64, _ = _fwd_bwd_case(W.SceneSpec(3000, 21, 0), W.CameraSpec((0.2, 0.1, -4.0), (0, 0, 0), 60.0, 160, 120))
    assert np.abs(rgb - rgb64).max() < 0.05
    _compare(g32, g64, 3000)


@pytest.mark.parametrize("tile", [8, 32])
def test_backward_other_tile_sizes(tile):
    g32, g64, *_ = _fwd_bwd_case(W.SceneSpec(3000, 22, 0), W.CameraSpec((0.0, 0.3, -4.0), (0, 0, 0), 60.0, 200, 136), tile)
    _compare(g32, g64, 3000)


def test_backward_forward_backward_config():
    """500k Gaussians, seed 2, cluster mixture, 1280x720; target from means N(0,0.01^2), SH N(0,0.02^2)."""
    g32, g64, rgb, rgb64, loss = _fwd_bwd_case(W.SCENE_500K, W.CAMERA_720P)
    assert 0.0 < loss < 1.0
    print(_compare(g32, g64, W.SCENE_500K.count))


def test_backward_needs_a_differentiable_forward(gpu_ctx):
    packed = W.SceneSpec(500, 1, 0).build()
    view = W.CameraSpec((0.0, 0.0, -4.0), (0, 0, 0), 60.0, 64, 64).view()
    sc = gpu_ctx.upload(packed, 500)
    try:
        gpu_ctx.forward(sc, view)
        with pytest.raises(webgs.GsError) as ei:
            gpu_ctx.backward(sc, np.zeros((64, 64, 3), np.float32))
        assert ei.value.code == 6  # GS_ERR_STATE
    finally:
        sc.close()
    with webgs.Context(flags=webgs.GS_FLAG_DIFFERENTIABLE) as ctx:
        a = ctx.upload(packed, 500)
        b = ctx.upload(packed, 500)
        ctx.forward(a, view)
        with pytest.raises(webgs.GsError):
            ctx.backward(b, np.zeros((64, 64, 3), np.float32))
        a.close(); b.close()


def test_backward_hostile_inputs():
    """The hostile scene of the forward test (zero quaternions, extreme scales and opacities,
    Gaussians at the eye and on the near plane, huge colours) through forward, backward and the
    FP64 adjoint: no fault, and the gradients of the ordinary Gaussians are finite and agree with
    the adjoint (the hostile ones may carry NaN in both)."""
    from test_gpu_hostile import _hostile_scene

    n, seed = 10_000, 43
    packed = _hostile_scene(n, seed)
    hostile = np.random.default_rng(seed).permutation(n)[:1400]
    ordinary = np.ones(n, bool)
    ordinary[hostile] = False
    view = W.CameraSpec((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), 60.0, 320, 240).view()
    dl = np.random.default_rng(7).normal(0.0, 1e-3, (240, 320, 3)).astype(np.float32)
    with webgs.Context(flags=webgs.GS_FLAG_DIFFERENTIABLE) as ctx:
        sc = ctx.upload(packed, n)
        try:
            ctx.forward(sc, view, rgba8=False, rgb=True, allow_overflow=True)
            g32 = ctx.backward(sc, dl)
        finally:
            sc.close()
    g64, _ = oracle.backward_f64(webgs.view_bytes(view), packed, n, dl)
    for name, (a, b) in _groups(n).items():
        width = (b - a) // n
        x = g32[a:b].reshape(n, width)[ordinary].astype(np.float64).ravel()
        y = g64[a:b].reshape(n, width)[ordinary].ravel()
        assert np.isfinite(x).all(), name
        ny = np.linalg.norm(y)
        if ny == 0.0:
            assert np.abs(x).max() == 0.0, name
            continue
        cos = float(x @ y / (np.linalg.norm(x) * ny))
        assert cos >= 0.999, (name, cos, np.linalg.norm(x - y) / ny)


def test_repeated_backward_calls_do_not_accumulate():
    """The 2D gradient buffer is cleared by the preprocess backward that consumed it, not by a memset
    before each call: gradients of repeated calls, and of a scene after another of a different size,
    equal the first call's (up to the order of the atomic sums)."""
    a_spec, b_spec = W.SceneSpec(3000, 31, 0), W.SceneSpec(1200, 32, 0)
    view = W.CameraSpec((0.1, 0.2, -4.0), (0, 0, 0), 60.0, 160, 120).view()
    dl = np.random.default_rng(3).normal(0.0, 1e-3, (120, 160, 3)).astype(np.float32)
    with webgs.Context(flags=webgs.GS_FLAG_DIFFERENTIABLE) as ctx:
        a = ctx.upload(a_spec.build(), a_spec.count)
        b = ctx.upload(b_spec.build(), b_spec.count)
        runs = []
        for sc in (a, a, b, a, b):
            ctx.forward(sc, view, rgba8=False, rgb=True)
            runs.append(ctx.backward(sc, dl))
        a.close(); b.close()
    for ref, other in ((runs[0], runs[1]), (runs[0], runs[3]), (runs[2], runs[4])):
        scale = np.abs(ref).max()
        assert scale > 0 and np.abs(other - ref).max() <= 1e-5 * scale
