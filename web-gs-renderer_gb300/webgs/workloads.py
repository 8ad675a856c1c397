"""Seeded synthetic workloads standing in for the reference's scenes (its .ply assets are Git LFS
pointers and no public dataset is involved). Sizes and distributions follow the five benchmark
configurations of the splat pipeline; all data comes from gs_synth_scene, so every host builds the
same bytes.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import View, camera_view, make_camera, synth_scene


@dataclass(frozen=True)
class SceneSpec:
    count: int
    seed: int
    kind: int          # 0: one N(0,1)^3 cluster, 1: cluster mixture in a box
    clusters: int = 0
    box: float = 0.0

    def build(self) -> np.ndarray:
        return synth_scene(self.kind, self.count, self.seed, self.clusters, self.box)


@dataclass(frozen=True)
class CameraSpec:
    eye: tuple
    target: tuple
    fovy: float
    width: int
    height: int
    z_near: float = 0.2
    z_far: float = 1000.0

    def view(self) -> View:
        return camera_view(self.eye, self.target, (0.0, 1.0, 0.0), self.fovy, self.width, self.height,
                           self.z_near, self.z_far)

    def camera(self):
        """The same camera as a gs_camera, for the device-side uniform builder."""
        return make_camera(self.eye, self.target, (0.0, 1.0, 0.0), self.fovy, self.width, self.height,
                           self.z_near, self.z_far)


# Plain forward, small: 50k Gaussians, unit cluster, camera at distance 4, fov 60, 512x512, near 0.2, far 100.
SMALL_SCENE = SceneSpec(50_000, 0, 0)
SMALL_CAMERA = CameraSpec((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), 60.0, 512, 512, 0.2, 100.0)

# Plain forward, scene scale: 1M Gaussians, 64-cluster mixture in a 20^3 box, camera inside the box,
# fov 70, 1920x1080.
SCENE_1M = SceneSpec(1_000_000, 1, 1, 64, 20.0)
CAMERA_1080P = CameraSpec((0.0, 1.0, -9.0), (0.0, 0.0, 0.0), 70.0, 1920, 1080)

# Forward+backward: 500k Gaussians, seed 2, mixture as above, 1280x720.
SCENE_500K = SceneSpec(500_000, 2, 1, 64, 20.0)
CAMERA_720P = CameraSpec((0.0, 1.0, -9.0), (0.0, 0.0, 0.0), 70.0, 1280, 720)

# Batched forward: 3 scenes (100k, 400k, 1.5M; seeds 3-5), 16 cameras on random orbits with
# resolutions drawn from {640x480, 1280x720, 1920x1080}.
BATCH_SCENES = (SceneSpec(100_000, 3, 1, 64, 20.0), SceneSpec(400_000, 4, 1, 64, 20.0),
                SceneSpec(1_500_000, 5, 1, 64, 20.0))
RESOLUTIONS = ((640, 480), (1280, 720), (1920, 1080))

# Batched forward+backward: one 3M scene, seed 6, 128 clusters in a 40^3 box, 8 x 1080p views.
SCENE_3M = SceneSpec(3_000_000, 6, 1, 128, 40.0)


def orbit_cameras(count: int, seed: int, radius: float, fovy: float = 70.0, resolutions=RESOLUTIONS,
                  fixed_resolution: tuple | None = None) -> list[tuple[int, CameraSpec]]:
    """Cameras on random orbits around the origin; returns (scene slot, camera) pairs with the scene
    slot drawn uniformly from 0..2 for the batched workload."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        theta = rng.uniform(0.0, 2.0 * math.pi)
        phi = rng.uniform(-0.35, 0.35)
        r = radius * rng.uniform(0.8, 1.0)
        eye = (r * math.cos(phi) * math.sin(theta), r * math.sin(phi), r * math.cos(phi) * math.cos(theta))
        w, h = fixed_resolution or resolutions[int(rng.integers(len(resolutions)))]
        out.append((int(rng.integers(3)), CameraSpec(eye, (0.0, 0.0, 0.0), fovy, w, h)))
    return out
