"""Comparison helpers shared by the parity tests (GPU path vs the CPU oracle)."""
from __future__ import annotations

import numpy as np

import oracle
import webgs

# fp32 RGB before quantization: the pipeline is pinned bit for bit, the written tolerance is the
# contract's 1e-4 max-abs.
RGB_TOL = 1e-4


def oracle_frame(view: webgs.View, packed: np.ndarray, count: int, tile: int = 16, factor: int = 64) -> dict:
    return oracle.forward_f32(webgs.view_bytes(view), packed, count, tile=tile, factor=factor)


def gpu_frame(ctx: webgs.Context, scene: webgs.Scene, view: webgs.View, allow_overflow: bool = False) -> dict:
    out = ctx.forward(scene, view, rgba8=True, rgb=True, final_t=True, n_contrib=True, allow_overflow=allow_overflow)
    dbg = ctx.debug()
    dbg.update(out)
    return dbg


def assert_frame_parity(g: dict, o: dict, check_rgb_bits: bool = True) -> None:
    """Bit-exact binning, tolerance-bounded pixels (bit-exact expected under the pinned semantics)."""
    assert g["instance_count"] == o["instance_count"], (g["instance_count"], o["instance_count"])
    assert g["sorted_count"] == o["sorted_count"]
    np.testing.assert_array_equal(g["tiles_touched"], o["tiles_touched"])
    vis = o["tiles_touched"] > 0
    np.testing.assert_array_equal(g["meta"].reshape(-1, 4)[vis], o["meta"].reshape(-1, 4)[vis])
    np.testing.assert_array_equal(g["offsets"], o["offsets"])
    for name, width in (("conic_opacity", 4), ("pixel", 2), ("color", 4)):
        gv = g[name].reshape(-1, width)[vis]
        ov = o[name].reshape(-1, width)[vis]
        np.testing.assert_array_equal(gv.view(np.uint32), ov.view(np.uint32), err_msg=name)
    n = o["sorted_count"]
    np.testing.assert_array_equal(g["keys"][:n], o["keys"][:n])
    np.testing.assert_array_equal(g["vals"][:n], o["vals"][:n])
    np.testing.assert_array_equal(g["ranges"], o["ranges"])
    err = float(np.abs(g["rgb"].astype(np.float64) - o["rgb"]).max()) if g["rgb"].size else 0.0
    assert err <= RGB_TOL, f"rgb max-abs {err}"
    if check_rgb_bits:
        np.testing.assert_array_equal(g["rgb"].view(np.uint32), o["rgb"].view(np.uint32))
        np.testing.assert_array_equal(g["final_t"].view(np.uint32), o["final_t"].view(np.uint32))
    np.testing.assert_array_equal(g["n_contrib"], o["n_contrib"])
    np.testing.assert_array_equal(g["rgba8"], o["rgba8"])
