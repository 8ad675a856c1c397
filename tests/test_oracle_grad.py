"""CPU checks of the FP64 adjoint (the reference for the CUDA backward) against FP64 central finite
differences, and of the L1 + SSIM loss gradient. h = 1e-4 on 256 random parameters of a small
scene; the step actually taken is the float32 difference of the perturbed parameter."""
import numpy as np
import pytest

import oracle
import webgs

LAMBDA = 0.2


@pytest.fixture(scope="module")
def small_problem():
    n = 400
    packed = webgs.synth_scene(0, n, 5)
    packed[3 * n: 6 * n] += 2.0  # larger splats: each covers several pixels of the 64x48 image
    view = webgs.camera_view((0.3, 0.2, -4.0), (0, 0, 0), (0, 1, 0), 60.0, 64, 48, 0.2, 100.0)
    vb = webgs.view_bytes(view)
    target = oracle.forward_f64(vb, webgs.perturb_scene(packed, n, 3, 0.01, 0.02), n)["rgb"]
    return n, packed, vb, target


def test_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 1, (24, 40, 3))
    y = np.clip(x + rng.normal(0, 0.1, x.shape), 0, 1)
    val, g = oracle.loss_l1_ssim(x, y, LAMBDA)
    assert 0 < val < 1
    for i in rng.choice(x.size, 40, replace=False):
        h = 1e-6
        xp = x.copy().ravel(); xp[i] += h
        xm = x.copy().ravel(); xm[i] -= h
        fd = (oracle.loss_l1_ssim(xp.reshape(x.shape), y, LAMBDA, False)[0] -
              oracle.loss_l1_ssim(xm.reshape(x.shape), y, LAMBDA, False)[0]) / (2 * h)
        assert abs(fd - g.ravel()[i]) <= 1e-6 * max(abs(fd), 1e-3)


def test_loss_of_identical_images_is_zero():
    x = np.random.default_rng(2).uniform(0, 1, (16, 16, 3))
    val, g = oracle.loss_l1_ssim(x, x, LAMBDA)
    assert abs(val) < 1e-12


def test_adjoint_matches_central_differences(small_problem):
    n, packed, vb, target = small_problem
    rgb = oracle.forward_f64(vb, packed, n)["rgb"]
    _, dl = oracle.loss_l1_ssim(rgb, target, LAMBDA)
    g, rgb_b = oracle.backward_f64(vb, packed, n, dl)
    np.testing.assert_allclose(rgb_b, rgb, rtol=0, atol=1e-12)

    def loss(p):
        return oracle.loss_l1_ssim(oracle.forward_f64(vb, p, n)["rgb"], target, LAMBDA, False)[0]

    rng = np.random.default_rng(7)
    cand = np.flatnonzero(np.abs(g) > 1e-8)
    sel = rng.choice(cand, 256, replace=False)
    rel = []
    for i in sel:
        p1 = packed.copy(); p1[i] += np.float32(1e-4)
        p2 = packed.copy(); p2[i] -= np.float32(1e-4)
        fd = (loss(p1) - loss(p2)) / (float(p1[i]) - float(p2[i]))
        rel.append(abs(fd - g[i]) / max(abs(fd), abs(g[i])))
    rel = np.array(rel)
    # piecewise-smooth loss (L1 kinks, alpha/colour clamps, 1/255 and 1e-4 thresholds): a few
    # parameters straddle a kink within +-h; everything else agrees to FD accuracy
    assert np.mean(rel < 1e-4) >= 0.95, np.sort(rel)[-20:]
    assert np.median(rel) < 1e-5


def test_adjoint_zero_for_culled_gaussians(small_problem):
    n, packed, vb, target = small_problem
    o = oracle.forward_f32(vb, packed, n)
    dl = np.ones((48, 64, 3))
    g, _ = oracle.backward_f64(vb, packed, n, dl)
    culled = np.flatnonzero(o["tiles_touched"] == 0)
    gg = g.reshape(-1)
    for gi in culled:
        assert gg[3 * gi: 3 * gi + 3].tolist() == [0.0, 0.0, 0.0]
        assert gg[13 * n + gi] == 0.0
