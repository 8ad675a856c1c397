"""Building blocks on the GPU vs the oracle: the radix sort (gs_sort_pairs), the decoupled-lookback
scan (gs_exclusive_scan), the pinned exps (gs_exp_f32, gs_raster_exp_f32) and the raster's
o * exp(power) (gs_raster_alpha_f32), through the C ABI."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _stable_ref(keys, vals, key_bits):
    mask = np.uint64((1 << key_bits) - 1)
    order = np.argsort(keys.astype(np.uint64) & mask, kind="stable")
    return keys[order], vals[order]


@pytest.mark.parametrize("n", [1, 2, 255, 256, 4095, 4096, 4097, 100_003, 3_000_000])
def test_sort_random_keys(gpu_ctx, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = gpu_ctx.sort_pairs(keys, vals, 32)
    rk, rv = _stable_ref(keys, vals, 32)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_array_equal(v, rv)


def test_sort_deep_aggregate_tree(gpu_ctx):
    """2^24 + 12,345 keys: 4,100 partitions of 4,096 keys, more than the 608 CTAs of a pass, so CTAs
    take several partitions each and the per-digit prefixes of the last partitions come through
    every level of the aggregate tree, a level-4 node (8^4 = 4,096 partitions) included."""
    n = (1 << 24) + 12_345
    rng = np.random.default_rng(24)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = gpu_ctx.sort_pairs(keys, vals, 32)
    rk, rv = _stable_ref(keys, vals, 32)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_array_equal(v, rv)


@pytest.mark.parametrize("digit_bits", [4, 8])
def test_sort_small_partitions(digit_bits):
    """The 2048-key partitions of the autotuner's smaller sort block: 1,465 partitions at 3M keys."""
    import webgs

    n = 3_000_000
    rng = np.random.default_rng(2048 + digit_bits)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    with webgs.Context(digit_bits=digit_bits, sort_block=2048) as ctx:
        k, v = ctx.sort_pairs(keys, vals, 32)
    rk, rv = _stable_ref(keys, vals, 32)
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_array_equal(v, rv)


def test_sort_matches_literal_reference_radix(gpu_ctx):
    rng = np.random.default_rng(5)
    n = 70_000
    keys = (rng.integers(0, 300, n).astype(np.uint32) << 16) | rng.integers(0, 50, n).astype(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    k, v = gpu_ctx.sort_pairs(keys, vals, 32)
    ok, ov = oracle.radix_sort_pairs(keys, vals, 4)
    np.testing.assert_array_equal(k, ok)
    np.testing.assert_array_equal(v, ov)


def test_sort_all_equal_and_partial_bits(gpu_ctx):
    n = 50_000
    keys = np.full(n, 0xABCD1234, np.uint32)
    vals = np.arange(n, dtype=np.uint32)[::-1].copy()
    k, v = gpu_ctx.sort_pairs(keys, vals, 32)
    np.testing.assert_array_equal(v, vals)  # stability: input order kept
    rng = np.random.default_rng(9)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    k, v = gpu_ctx.sort_pairs(keys, np.arange(n, dtype=np.uint32), 20)
    rk, rv = _stable_ref(keys, np.arange(n, dtype=np.uint32), 20)
    np.testing.assert_array_equal(v, rv)


@pytest.mark.parametrize("n", [0, 1, 7, 2048, 2049, 1_000_001])
def test_exclusive_scan(gpu_ctx, n):
    rng = np.random.default_rng(n)
    data = rng.integers(0, 70, n).astype(np.uint32)
    out, tot = gpu_ctx.exclusive_scan(data)
    ref, rtot = oracle.exclusive_scan(data)
    np.testing.assert_array_equal(out, ref)
    assert tot == rtot


def test_pinned_exp_bitwise(gpu_ctx):
    rng = np.random.default_rng(0)
    x = np.concatenate([
        rng.uniform(-110, 95, 2_000_000).astype(np.float32),
        rng.uniform(-6, 0, 2_000_000).astype(np.float32),
        np.array([0.0, -0.0, 88.7, 88.8, 89.0, -103.9, -104.0, -104.1, np.inf, -np.inf, np.nan, 1e-30, -1e-30],
                 np.float32),
    ])
    g = gpu_ctx.exp(x)
    o = oracle.expf(x)
    np.testing.assert_array_equal(g.view(np.uint32), o.view(np.uint32))


def test_raster_exp_bitwise(gpu_ctx):
    """The raster's exp (its own pinned definition on [-5.6, 0]) on the device equals the oracle's."""
    rng = np.random.default_rng(1)
    x = np.concatenate([np.linspace(-5.6, 0.0, 1_000_001, dtype=np.float32),
                        rng.uniform(-5.6, 0.0, 2_000_000).astype(np.float32),
                        np.array([0.0, -0.0, -5.6, -1e-30, -1e-8, -0.3465736, -0.3465736 * 3], np.float32)])
    g = gpu_ctx.exp(x, raster=True)
    o = oracle.raster_expf(x)
    np.testing.assert_array_equal(g.view(np.uint32), o.view(np.uint32))


def test_raster_alpha_bitwise(gpu_ctx):
    """o * exp(power) as the raster forms it (2^n added to the exponent field of o * p) equals the
    oracle's o * raster_expf(power) bit for bit, for every power the raster evaluates: at or above the
    opacity's cut-off ln((1/255)/o) - 1e-3 (an opacity below about 1/255 has a positive cut-off and is
    never evaluated). NaN opacities or powers give 0.99 after the clamp, as the oracle's NaN does."""
    rng = np.random.default_rng(7)
    n = 3_000_000
    lo = np.float32(1.0 / 255.0) * np.float32(1.01)
    o = rng.uniform(float(lo), 1.0, n).astype(np.float32)
    o[:1000] = 1.0
    o[1000:2000] = lo
    cut = (np.log((1.0 / 255.0) / o.astype(np.float64)) - 1e-3).astype(np.float32)
    x = (cut.astype(np.float64) * rng.uniform(0.0, 1.0, n)).astype(np.float32)  # in (cut, 0]
    x[2000:3000] = np.float32(0.0)
    x[3000:4000] = np.float32(-0.0)
    x[4000:5000] = (cut[4000:5000].astype(np.float64) * (1.0 - 1e-6)).astype(np.float32)
    y = gpu_ctx.raster_alpha(o, x)
    ref = o * oracle.raster_expf(x)
    np.testing.assert_array_equal(y.view(np.uint32), ref.view(np.uint32))
    nan = np.float32(np.nan)
    on = np.array([nan, 0.5, nan, 0.0], np.float32)
    xn = np.array([-1.0, nan, nan, nan], np.float32)
    yn = np.fmin(np.float32(0.99), gpu_ctx.raster_alpha(on, xn))
    rn = np.fmin(np.float32(0.99), on * oracle.raster_expf(xn))
    np.testing.assert_array_equal(yn, rn)
    assert (yn == np.float32(0.99)).all()
