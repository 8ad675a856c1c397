"""The CUDA gradients against central finite differences, directly (through the C ABI).

A small scene (400 Gaussians with enlarged splats, 64x48) and the differentiation workload's loss,
L1 + 0.2 (1 - SSIM) against the render of a perturbed copy of the scene. The CUDA pipeline gives the
gradient: gs_forward, gs_loss_l1_ssim, gs_backward. 256 parameters are drawn at random, stratified
over the six parameter groups, among those whose gradient is not negligible; each is moved by
+-h, h = 1e-4 (the float32 step actually taken is used), and the loss is evaluated again with the
FP64 oracle forward and the FP64 loss (the same loss definition, checked against gs_loss_l1_ssim in
test_gpu_backward.py), so the differences are free of fp32 rounding noise.

Tolerance per parameter group: median relative error <= 1e-4 and at least 90% of the group's
parameters within 1e-3 (measured: medians of 2e-6 to 3e-6). The loss is piecewise smooth (L1
kinks, the alpha and colour clamps, the 1/255 and 1e-4 thresholds, tile boundaries), so a few
parameters straddle a kink within +-h; that is why the bound is on the median and on a fraction
rather than on every parameter. (Differences of the fp32 CUDA forward itself at h = 1e-4 are
dominated by fp32 rounding of the pixels, medians of 3% to 20%, and are not a usable check.)
"""
import numpy as np
import pytest

import oracle
import webgs

pytestmark = pytest.mark.gpu

LAMBDA = 0.2
H = 1e-4
N = 400
W_, H_ = 64, 48


def _groups(n):
    return {"means": (0, 3 * n), "log-scales": (3 * n, 6 * n), "quaternions": (6 * n, 10 * n),
            "sh-dc": (10 * n, 13 * n), "opacity": (13 * n, 14 * n), "sh-rest": (14 * n, 59 * n)}


@pytest.fixture(scope="module")
def problem():
    packed = webgs.synth_scene(0, N, 5)
    packed[3 * N: 6 * N] += 2.0  # larger splats: each covers several pixels of the 64x48 image
    view = webgs.camera_view((0.3, 0.2, -4.0), (0, 0, 0), (0, 1, 0), 60.0, W_, H_, 0.2, 100.0)
    ctx = webgs.Context(flags=webgs.GS_FLAG_DIFFERENTIABLE)
    ts = ctx.upload(webgs.perturb_scene(packed, N, 3, 0.01, 0.02), N)
    target = ctx.forward(ts, view, rgba8=False, rgb=True)["rgb"]
    ts.close()
    sc = ctx.upload(packed, N)
    rgb = ctx.forward(sc, view, rgba8=False, rgb=True)["rgb"]
    loss, dl = ctx.loss(rgb, target, LAMBDA)
    g = ctx.backward(sc, dl).astype(np.float64)
    rng = np.random.default_rng(11)
    sel = []
    groups = _groups(N)
    per = [256 // len(groups) + (1 if k < 256 % len(groups) else 0) for k in range(len(groups))]
    for (name, (a, b)), k in zip(groups.items(), per):
        cand = a + np.flatnonzero(np.abs(g[a:b]) > 1e-3 * np.abs(g[a:b]).max())
        sel.append((name, rng.choice(cand, min(k, cand.size), replace=False)))
    yield {"ctx": ctx, "scene": sc, "packed": packed, "view": view, "target": target, "g": g, "sel": sel,
           "loss": loss}
    sc.close()
    ctx.close()


def _rel(fd, g):
    return np.abs(fd - g) / np.maximum(np.maximum(np.abs(fd), np.abs(g)), 1e-12)


def _check(p, loss_of, med_tol, frac_tol, frac_min):
    assert sum(idx.size for _, idx in p["sel"]) == 256
    report = {}
    for name, idx in p["sel"]:
        fd = np.empty(idx.size)
        for j, i in enumerate(idx):
            p1 = p["packed"].copy(); p1[i] += np.float32(H)
            p2 = p["packed"].copy(); p2[i] -= np.float32(H)
            fd[j] = (loss_of(p1) - loss_of(p2)) / (float(p1[i]) - float(p2[i]))
        rel = _rel(fd, p["g"][idx])
        report[name] = (float(np.median(rel)), float(np.mean(rel <= frac_tol)))
    for name, (med, frac) in report.items():
        assert med <= med_tol and frac >= frac_min, (name, med, frac, report)
    return report


def test_cuda_gradient_against_fp64_central_differences(problem):
    p = problem
    vb = webgs.view_bytes(p["view"])
    target = p["target"].astype(np.float64)

    def loss_of(packed):
        return oracle.loss_l1_ssim(oracle.forward_f64(vb, packed, N)["rgb"], target, LAMBDA, False)[0]

    # the FP64 loss at the unperturbed scene is the CUDA loss up to fp32 rounding of the pixels
    assert abs(loss_of(p["packed"]) - p["loss"]) < 1e-5
    print(_check(p, loss_of, 1e-4, 1e-3, 0.90))
