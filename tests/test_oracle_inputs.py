"""The oracle's own input generators (oracle/gs_inputs.cpp) against the product's host utilities
(gs_synth_scene, gs_perturb_scene, gs_camera_view): bit-identical bytes. The timed CPU baseline
builds its inputs with the oracle's copies, so it never loads the product library; this test is
what guarantees it times the same workload."""
import numpy as np
import pytest

import oracle
import webgs
from webgs import workloads as W


@pytest.mark.parametrize("spec", [W.SceneSpec(20_000, 0, 0), W.SceneSpec(30_000, 3, 1, 64, 20.0),
                                  W.SceneSpec(10_000, 6, 1, 128, 40.0)])
def test_synth_scene_matches_product(spec):
    a = oracle.synth_scene(spec.kind, spec.count, spec.seed, spec.clusters, spec.box)
    b = webgs.synth_scene(spec.kind, spec.count, spec.seed, spec.clusters, spec.box)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    pa = oracle.perturb_scene(a, spec.count, 99, 0.01, 0.02)
    pb = webgs.perturb_scene(b, spec.count, 99, 0.01, 0.02)
    np.testing.assert_array_equal(pa.view(np.uint32), pb.view(np.uint32))
    assert not np.array_equal(pa, a)


@pytest.mark.parametrize("cam", [W.SMALL_CAMERA, W.CAMERA_1080P, W.CAMERA_720P]
                         + [c for _, c in W.orbit_cameras(16, 2024, 9.0)])
def test_camera_view_matches_product(cam):
    a = oracle.camera_view(cam.eye, cam.target, (0.0, 1.0, 0.0), cam.fovy, cam.width, cam.height, cam.z_near,
                           cam.z_far)
    b = webgs.view_bytes(cam.view())
    assert a == b


def test_camera_view_rejects_bad_cameras():
    with pytest.raises(ValueError):
        oracle.camera_view((0, 0, -4), (0, 0, 0), fovy_deg=180.0)
    with pytest.raises(ValueError):
        oracle.camera_view((0, 0, -4), (0, 0, 0), width=0)
