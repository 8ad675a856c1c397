"""Known-answer tests of the CPU oracle (the restatement of the reference shaders), worked out by hand
from preprocess.wgsl / emit.wgsl / radix_parallel.wgsl / tile_ranges.wgsl / raseter.wgsl. The
reference ships no tests or golden vectors, so these analytic cases and the committed regression
fixtures (test_oracle_golden.py) are what pins the oracle."""
import math

import numpy as np
import pytest

import oracle
import webgs

SH_C0 = 0.28209479177387814


def packed_scene(pos, logscale, quat_wxyz, dc, logit, rest=None):
    pos = np.asarray(pos, np.float64).reshape(-1, 3)
    n = len(pos)
    rest = np.zeros((n, 45)) if rest is None else np.asarray(rest, np.float64).reshape(n, 45)
    blocks = [pos, np.asarray(logscale, np.float64).reshape(n, 3), np.asarray(quat_wxyz, np.float64).reshape(n, 4),
              np.asarray(dc, np.float64).reshape(n, 3), np.asarray(logit, np.float64).reshape(n, 1), rest]
    return np.concatenate([b.ravel() for b in blocks]).astype(np.float32), n


def camera(w=64, h=64, eye=(0.0, 0.0, -4.0), fov=60.0):
    return webgs.camera_view(eye, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), fov, w, h, 0.2, 100.0)


def run(view, packed, n, **kw):
    return oracle.forward_f32(webgs.view_bytes(view), packed, n, **kw)


def test_single_centered_gaussian_analytic():
    s = 0.05
    packed, n = packed_scene([0, 0, 0], [math.log(s)] * 3, [1, 0, 0, 0], [0.2, -0.1, 0.4], [2.0])
    v = camera()
    r = run(v, packed, n)
    f = 32.0 / math.tan(math.radians(30.0))  # focal = H / (2 tan(fov/2))
    var = s * s * f * f / 16.0 + 0.3         # cov2D of an isotropic splat at depth 4, plus the low-pass
    conic = r["conic_opacity"][:4]
    assert conic[0] == pytest.approx(1 / var, rel=1e-5) and conic[2] == pytest.approx(1 / var, rel=1e-5)
    assert abs(conic[1]) < 1e-6
    assert conic[3] == pytest.approx(1 / (1 + math.exp(-2.0)), rel=1e-6)
    assert tuple(r["pixel"][:2]) == pytest.approx((31.5, 31.5), abs=1e-4)
    radius = math.ceil(3 * math.sqrt(var + math.sqrt(0.1)))
    lo, hi = math.floor((31.5 - radius) / 16), math.floor((31.5 + radius) / 16)
    assert r["meta"][0] == (lo << 16) | lo and r["meta"][1] == (hi << 16) | hi
    assert r["tiles_touched"][0] == (hi - lo + 1) ** 2
    # clip depth of view z = -4 with near 0.2, far 100 (0..1 depth), truncated to 16 bits
    zf, zn = 100.0, 0.2
    ndcz = (zf / (zn - zf) * -4.0 + zf * zn / (zn - zf)) / 4.0
    assert abs(int(r["meta"][2]) - int(ndcz * 65535)) <= 1
    col = [SH_C0 * c + 0.5 for c in (0.2, -0.1, 0.4)]
    assert tuple(r["color"][:3]) == pytest.approx(col, abs=1e-6)
    # the pixel under the centre: alpha = min(0.99, o * exp(-0.5 * conic * 0.5^2 * 2)), blended once
    o = 1 / (1 + math.exp(-2.0))
    alpha = min(0.99, o * math.exp(-0.5 * (0.25 / var + 0.25 / var)))
    assert tuple(r["rgb"][31, 31]) == pytest.approx([c * alpha for c in col], rel=1e-5)
    assert r["final_t"][31, 31] == pytest.approx(1 - alpha, rel=1e-5)
    assert r["n_contrib"][31, 31] == 1


def test_behind_camera_and_near_plane_are_culled():
    packed, n = packed_scene([[0, 0, -4.1], [0, 0, -3.9], [0, 0, -6]], [[-3] * 3] * 3, [[1, 0, 0, 0]] * 3,
                             [[0, 0, 0]] * 3, [0, 0, 0])
    r = run(camera(), packed, n)
    assert r["tiles_touched"].tolist() == [0, 0, 0]  # 0.1 units in front (< 0.2 near) and two behind
    assert r["instance_count"] == 0 and r["rgb"].max() == 0 and np.all(r["final_t"] == 1)


def test_frustum_cull_and_inclusive_tile_rect():
    # far to the side: culled by isInFrustum; splats near the image edges keep clamped tile rects
    # (world +x is image -x for this camera, which looks down +z with up = +y)
    packed, n = packed_scene([[30, 0, 0], [2.1, 0, 0], [-2.1, 0, 0]], [[-2] * 3] * 3, [[1, 0, 0, 0]] * 3,
                             [[0, 0, 0]] * 3, [0, 0, 0])
    r = run(camera(), packed, n)
    assert r["tiles_touched"][0] == 0
    left, right = r["meta"][4:8], r["meta"][8:12]
    assert r["pixel"][2] < 16 and (left[0] & 0xFFFF) == 0      # floor of a negative edge clamps to 0
    assert r["pixel"][4] > 48 and (right[1] & 0xFFFF) == 3     # ... and to tilesPerRow - 1 = 3


def test_equal_depth_ties_sort_by_gaussian_index():
    # four identical splats: same tiles, same depth16 -> keys tie, values must come out 0, 1, 2, 3
    packed, n = packed_scene([[0, 0, 0]] * 4, [[-2.5] * 3] * 4, [[1, 0, 0, 0]] * 4, [[0.1, 0.2, 0.3]] * 4, [0] * 4)
    r = run(camera(), packed, n)
    keys, vals = r["keys"], r["vals"]
    for t in np.unique(keys >> 16):
        sel = vals[(keys >> 16) == t]
        assert sel.tolist() == [0, 1, 2, 3]


def test_saturating_stack_stops_before_the_saturating_splat():
    # eight opaque splats at the same spot, front to back; alpha clamps at 0.99. In fp32,
    # T after one splat is 1 - 0.99f = 0.00999999, and the second splat's testT = 9.99998e-5 is below
    # the f32 threshold 1e-4 (1.00000005e-4): the pixel ends without blending it (raseter.wgsl:91-95)
    z = [0.0 + 0.01 * k for k in range(8)]
    packed, n = packed_scene([[0, 0, zz] for zz in z], [[0.0] * 3] * 8, [[1, 0, 0, 0]] * 8, [[1, 1, 1]] * 8,
                             [20.0] * 8)
    r = run(camera(), packed, n)
    assert r["n_contrib"][31, 31] == 1
    assert r["final_t"][31, 31] == np.float32(1) - np.float32(0.99)
    c = SH_C0 + 0.5
    assert r["rgb"][31, 31, 0] == pytest.approx(c * 0.99, rel=1e-6)


@pytest.mark.parametrize("w,h", [(1, 1), (17, 17), (31, 7)])
def test_odd_image_sizes(w, h):
    packed = webgs.synth_scene(0, 500, 3)
    r = run(camera(w, h), packed, 500)
    assert r["tiles_x"] == (w + 15) // 16 and r["tiles_y"] == (h + 15) // 16
    assert r["rgb"].shape == (h, w, 3)
    assert np.all((r["keys"] >> 16) < r["tiles_x"] * r["tiles_y"])


def test_overflow_truncates_at_max_instance():
    packed = webgs.synth_scene(0, 300, 4)
    full = run(camera(), packed, 300)
    trunc = run(camera(), packed, 300, factor=1)
    assert full["instance_count"] > 300 and trunc["sorted_count"] == 300
    # the kept slots are the first 300 emitted: the Gaussians with offsets < 300
    first = np.flatnonzero((full["offsets"][:-1] < 300) & (full["tiles_touched"] > 0))
    assert set(np.unique(trunc["vals"]).tolist()) == set(first.tolist())
    starts, ends = trunc["ranges"][0::2], trunc["ranges"][1::2]
    assert ends.max() == 300 and np.all(ends >= starts)


def test_overflow_tile_ranges_differ_from_reference_only_at_the_last_tile():
    """The deliberate deviation of the overflow contract. With I > max_instance the reference's tile
    ranges pass is bounded by the unclamped count I (renderer.js:612, tile_ranges.wgsl:14,32), so the
    last kept tile's end is never written and that tile rasterizes nothing; this pipeline bounds the
    pass by min(I, max_instance) and closes the last tile at max_instance. Every other range agrees.
    256 slots fill the indirect grid exactly, so no reference thread reads past the keys."""
    packed = webgs.synth_scene(0, 256, 4)
    trunc = run(camera(), packed, 256, factor=1)
    I, cap = trunc["instance_count"], trunc["sorted_count"]
    assert I > cap == 256
    tiles = trunc["tiles_x"] * trunc["tiles_y"]
    ref, beyond = oracle.tile_ranges_reference(trunc["keys"], cap, I, tiles)
    assert beyond == 0
    last = int(trunc["keys"][cap - 1] >> 16)
    ours = trunc["ranges"].copy()
    assert ours[2 * last + 1] == cap and ref[2 * last + 1] == 0 and ref[2 * last] == ours[2 * last] > 0
    ours[2 * last + 1] = 0
    np.testing.assert_array_equal(ref, ours)
    # without overflow both bounds are the same count and the ranges agree everywhere
    full = run(camera(), packed, 256)
    ref_full, beyond = oracle.tile_ranges_reference(full["keys"], full["sorted_count"], full["instance_count"], tiles)
    assert beyond == 0
    np.testing.assert_array_equal(ref_full, full["ranges"])


def test_scan_restatement_is_exclusive_prefix_sum():
    rng = np.random.default_rng(0)
    d = rng.integers(0, 1000, 10_001).astype(np.uint32)
    out, tot = oracle.exclusive_scan(d)
    ref = np.concatenate([[0], np.cumsum(d.astype(np.uint64))[:-1]]).astype(np.uint32)
    np.testing.assert_array_equal(out, ref)
    assert tot == int(d.astype(np.uint64).sum()) % (1 << 32)


def test_literal_radix_sort_is_a_stable_sort():
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 2 ** 32, 50_000, dtype=np.uint64).astype(np.uint32)
    keys[::7] = keys[0]  # many ties
    vals = np.arange(keys.size, dtype=np.uint32)
    k, v = oracle.radix_sort_pairs(keys, vals, 4)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(k, keys[order])
    np.testing.assert_array_equal(v, vals[order])


def test_pinned_exp_accuracy():
    x = np.concatenate([np.linspace(-87, 88, 1_000_001, dtype=np.float32),
                        np.random.default_rng(2).uniform(-10, 0, 200_000).astype(np.float32)])
    y = oracle.expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.abs(y - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert ulp.max() < 1.0
    special = oracle.expf(np.array([0.0, -200.0, 200.0, np.inf, -np.inf, np.nan], np.float32))
    assert special[0] == 1.0 and special[1] == 0.0 and np.isinf(special[2]) and np.isinf(special[3])
    assert special[4] == 0.0 and np.isnan(special[5])


def test_raster_exp_accuracy():
    """The raster's exp (rule 4b) on its whole domain [-5.6, 0]: under 1 ulp from the FP64 exp
    (WGSL allows 3 + 2|x| ulp for exp)."""
    x = np.concatenate([np.linspace(-5.6, 0.0, 2_000_001, dtype=np.float32),
                        np.random.default_rng(3).uniform(-5.6, 0.0, 500_000).astype(np.float32),
                        np.array([0.0, -0.0, -1e-30, -1e-8], np.float32)])
    y = oracle.raster_expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.abs(y - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert ulp.max() < 1.0, ulp.max()
    assert oracle.raster_expf(np.array([0.0], np.float32))[0] == 1.0


def test_fp64_twin_close_to_fp32():
    packed = webgs.synth_scene(0, 2000, 5)
    v = camera(96, 80)
    r32 = run(v, packed, 2000)
    r64 = oracle.forward_f64(webgs.view_bytes(v), packed, 2000)
    err = np.abs(r32["rgb"] - r64["rgb"])
    assert np.median(err) < 1e-6 and np.mean(err) < 1e-4
