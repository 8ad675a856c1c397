"""gs_exclusive_scan_static: the exclusive scan for callers that must not allocate device memory.

Its scratch is a fixed device array inside libwebgs.so instead of context allocations, because some
callers cannot allocate on their hot path (cudaMalloc/cudaFree may synchronize the device, which a
real-time frame loop cannot afford; hosts with their own memory arenas forbid a library from
allocating). This file is collected last, so a stopped run has already exercised everything else.
Checked through the C ABI against gs_exclusive_scan on two calls in a row (integer results: equal).
"""
import ctypes as C

import numpy as np
import pytest

import webgs

pytestmark = pytest.mark.gpu

MAX_N = 1 << 24


def _static_scan(lib, data: np.ndarray):
    torch = pytest.importorskip("torch")
    d_in = torch.from_numpy(data.astype(np.int64)).to(torch.int32).cuda()
    d_out = torch.empty_like(d_in)
    d_tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    rc = lib.gs_exclusive_scan_static(d_in.data_ptr(), d_out.data_ptr(), data.size, d_tot.data_ptr(),
                                      stream.cuda_stream)
    assert rc == 0, webgs._abi.STATUS_NAMES.get(rc, rc)
    torch.cuda.synchronize()
    out = d_out.cpu().numpy().view(np.uint32)
    return out, int(d_tot.cpu().numpy().view(np.uint32)[0]), d_in.cpu().numpy().view(np.uint32)


def test_static_scan_matches_context_scan_twice():
    lib = webgs.library()
    rng = np.random.default_rng(2024)
    with webgs.Context() as ctx:
        for n in (1_234_567, 40_001):  # two calls in a row share (and reuse) the scratch array
            data = rng.integers(0, 200, n).astype(np.uint32)
            ref, ref_total = ctx.exclusive_scan(data)
            out, total, unchanged = _static_scan(lib, data)
            np.testing.assert_array_equal(out, ref)
            assert total == ref_total
            np.testing.assert_array_equal(unchanged, data)


def test_static_scan_rejects_sizes_beyond_its_scratch():
    lib = webgs.library()
    assert lib.gs_exclusive_scan_static(None, None, MAX_N + 1, None, None) == webgs._abi.GS_ERR_INVALID
