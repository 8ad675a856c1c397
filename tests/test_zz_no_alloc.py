"""gs_exclusive_scan_static: the exclusive scan for callers that must not allocate device memory.

Its scratch is a fixed device array inside libwebgs.so instead of context allocations, because some
callers cannot allocate on their hot path (cudaMalloc/cudaFree may synchronize the device, which a
real-time frame loop cannot afford; hosts with their own memory arenas forbid a library from
allocating). This file is collected last, so a stopped run has already exercised everything else.
Checked through the C ABI against gs_exclusive_scan and numpy's cumsum (integer results: equal), on
two calls in a row, in place, without a total pointer, at n = 0, 1 and the 2^24 maximum, across the
wrap of the lookback words' sequence tags, and with the device's free memory unchanged by a call.
"""
import numpy as np
import pytest

import webgs

pytestmark = pytest.mark.gpu

MAX_N = 1 << 24


def _cumsum_excl(data: np.ndarray) -> tuple[np.ndarray, int]:
    if data.size == 0:
        return np.zeros(0, np.uint32), 0
    c = np.cumsum(data.astype(np.uint64))
    excl = np.concatenate([[0], c[:-1]]).astype(np.uint64)
    return (excl & 0xFFFFFFFF).astype(np.uint32), int(c[-1] & 0xFFFFFFFF)


def _device(data: np.ndarray):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(data.astype(np.uint32).view(np.int32).copy()).cuda()


def _host(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


def _static_scan(data: np.ndarray, in_place: bool = False, with_total: bool = True):
    """Runs the scan on copies of `data` on the device; returns (out, total or None, input after)."""
    torch = pytest.importorskip("torch")
    lib = webgs.library()
    d_in = _device(data) if data.size else torch.zeros(1, dtype=torch.int32, device="cuda")
    d_out = d_in if in_place else torch.empty_like(d_in)
    d_tot = torch.full((1,), -1, dtype=torch.int32, device="cuda") if with_total else None
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    rc = lib.gs_exclusive_scan_static(d_in.data_ptr(), d_out.data_ptr(), data.size,
                                      d_tot.data_ptr() if with_total else None, stream.cuda_stream)
    assert rc == 0, webgs._abi.STATUS_NAMES.get(rc, rc)
    torch.cuda.synchronize()
    out = _host(d_out)[:data.size]
    return out, (int(_host(d_tot)[0]) if with_total else None), _host(d_in)[:data.size]


def test_static_scan_matches_context_scan_twice():
    rng = np.random.default_rng(2024)
    with webgs.Context() as ctx:
        for n in (1_234_567, 40_001):  # two calls in a row share (and reuse) the scratch array
            data = rng.integers(0, 200, n).astype(np.uint32)
            ref, ref_total = ctx.exclusive_scan(data)
            out, total, unchanged = _static_scan(data)
            np.testing.assert_array_equal(out, ref)
            assert total == ref_total
            np.testing.assert_array_equal(unchanged, data)


@pytest.mark.parametrize("n", [0, 1, 2048, 2049])
def test_static_scan_small_sizes(n):
    data = np.random.default_rng(n).integers(0, 1 << 20, n).astype(np.uint32)
    out, total, _ = _static_scan(data)
    ref, ref_total = _cumsum_excl(data)
    np.testing.assert_array_equal(out, ref)
    assert total == ref_total


def test_static_scan_in_place_and_without_total():
    rng = np.random.default_rng(7)
    data = rng.integers(0, 1000, 300_001).astype(np.uint32)
    ref, ref_total = _cumsum_excl(data)
    out, total, after = _static_scan(data, in_place=True)
    np.testing.assert_array_equal(out, ref)
    np.testing.assert_array_equal(after, ref)  # in place: the input buffer holds the result
    assert total == ref_total
    out, total, _ = _static_scan(data, with_total=False)
    np.testing.assert_array_equal(out, ref)
    assert total is None


def test_static_scan_at_its_maximum_size():
    """n = 2^24 fills every one of the 8192 lookback words of the fixed scratch."""
    data = np.random.default_rng(11).integers(0, 256, MAX_N).astype(np.uint32)
    ref, ref_total = _cumsum_excl(data)
    for _ in range(2):
        out, total, _ = _static_scan(data)
        np.testing.assert_array_equal(out, ref)
        assert total == ref_total


def test_static_scan_across_the_sequence_wrap():
    """The lookback words carry 30-bit sequence tags that repeat every 2^26 calls. Tag-0 words of
    another input are planted (a call right after a wrap), a one-partition call leaves them in place,
    and the call that wraps again must clear them before its lookback reads them."""
    lib = webgs.library()
    rng = np.random.default_rng(12)
    planted = rng.integers(0, 5000, MAX_N).astype(np.uint32)
    small = rng.integers(0, 5000, 1000).astype(np.uint32)
    data = rng.integers(0, 200, MAX_N).astype(np.uint32)
    pytest.importorskip("torch").cuda.synchronize()
    assert lib.gs_debug_set_sequence(None, 0xFFFFFFF0) == 0  # next call: tags 0..15
    for d in (planted, small, data):
        if d is small:
            assert lib.gs_debug_set_sequence(None, (1 << 30) - 32) == 0  # next: 2^30 - 16, then 0 again
        out, total, _ = _static_scan(d)
        ref, ref_total = _cumsum_excl(d)
        np.testing.assert_array_equal(out, ref)
        assert total == ref_total


def test_static_scan_allocates_no_device_memory():
    torch = pytest.importorskip("torch")
    lib = webgs.library()
    data = np.random.default_rng(3).integers(0, 100, 2_000_000).astype(np.uint32)
    d_in = _device(data)
    d_out = torch.empty_like(d_in)
    d_tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    args = (d_in.data_ptr(), d_out.data_ptr(), data.size, d_tot.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    assert lib.gs_exclusive_scan_static(*args) == 0  # warm-up: module loaded, symbol looked up
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert lib.gs_exclusive_scan_static(*args) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    ref, ref_total = _cumsum_excl(data)
    np.testing.assert_array_equal(_host(d_out), ref)
    assert int(_host(d_tot)[0]) == ref_total


def test_static_scan_rejects_sizes_beyond_its_scratch():
    lib = webgs.library()
    assert lib.gs_exclusive_scan_static(None, None, MAX_N + 1, None, None) == webgs._abi.GS_ERR_INVALID
    assert lib.gs_exclusive_scan_static(None, None, 5, None, None) == webgs._abi.GS_ERR_INVALID
