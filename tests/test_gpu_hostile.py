"""Hostile but finite inputs through the GPU pipeline and the oracle: zero quaternions (NaN
covariances), huge and tiny scales, saturated opacities, Gaussians at the eye and on the near plane,
huge colours. The pipeline must not fault, binning must match bit for bit and pixels must match
(NaN-carrying intermediates compared as values, where NaNs count as equal)."""
import numpy as np
import pytest

import webgs
from helpers import gpu_frame, oracle_frame
from webgs import workloads as W

pytestmark = pytest.mark.gpu


def _hostile_scene(n, seed):
    rng = np.random.default_rng(seed)
    packed = W.SceneSpec(n, seed, 0).build()
    pos = packed[0:3 * n].reshape(n, 3)
    scale = packed[3 * n:6 * n].reshape(n, 3)
    quat = packed[6 * n:10 * n].reshape(n, 4)
    dc = packed[10 * n:13 * n].reshape(n, 3)
    opac = packed[13 * n:14 * n]
    idx = rng.permutation(n)
    groups = np.array_split(idx[:1400], 7)
    quat[groups[0]] = 0.0                                   # zero quaternion: 0/0 in the normalisation
    scale[groups[1]] = 9.0                                  # e^9 ~ 8100: covers the whole image
    scale[groups[2]] = -40.0                                # e^-40: only the 0.3 low-pass is left
    opac[groups[3][: len(groups[3]) // 2]] = 80.0            # sigmoid saturates to 1
    opac[groups[3][len(groups[3]) // 2:]] = -80.0            # and to 0
    eye = np.array([0.0, 0.0, -4.0], np.float32)
    pos[groups[4]] = eye                                    # at the eye: view z = 0, near-culled
    pos[groups[5]] = eye + np.array([0.0, 0.0, 0.2], np.float32)  # on the near plane
    dc[groups[6]] = rng.choice([-1e4, 1e4], (len(groups[6]), 3)).astype(np.float32)
    return packed


def _assert_values_equal(g, o):
    assert g["instance_count"] == o["instance_count"] and g["sorted_count"] == o["sorted_count"]
    np.testing.assert_array_equal(g["tiles_touched"], o["tiles_touched"])
    vis = o["tiles_touched"] > 0
    np.testing.assert_array_equal(g["meta"].reshape(-1, 4)[vis], o["meta"].reshape(-1, 4)[vis])
    np.testing.assert_array_equal(g["offsets"], o["offsets"])
    for name, width in (("conic_opacity", 4), ("pixel", 2), ("color", 4)):
        np.testing.assert_array_equal(g[name].reshape(-1, width)[vis], o[name].reshape(-1, width)[vis], err_msg=name)
    n = o["sorted_count"]
    np.testing.assert_array_equal(g["keys"][:n], o["keys"][:n])
    np.testing.assert_array_equal(g["vals"][:n], o["vals"][:n])
    np.testing.assert_array_equal(g["ranges"], o["ranges"])
    np.testing.assert_array_equal(g["rgb"], o["rgb"])
    np.testing.assert_array_equal(g["final_t"], o["final_t"])
    np.testing.assert_array_equal(g["n_contrib"], o["n_contrib"])
    np.testing.assert_array_equal(g["rgba8"], o["rgba8"])


@pytest.mark.parametrize("seed", [41, 42])
def test_hostile_inputs_match_oracle(gpu_ctx, seed):
    n = 10_000
    packed = _hostile_scene(n, seed)
    view = W.CameraSpec((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), 60.0, 320, 240).view()
    scene = gpu_ctx.upload(packed, n)
    try:
        g = gpu_frame(gpu_ctx, scene, view, allow_overflow=True)
    finally:
        scene.close()
    o = oracle_frame(view, packed, n)
    assert o["instance_count"] > 0
    _assert_values_equal(g, o)
