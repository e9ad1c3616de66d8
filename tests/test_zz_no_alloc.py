"""The allocation-free prefix sum (gb_scan_i32_noalloc) against the workspace-based gb_scan_i32.

gb_scan_i32_noalloc serves callers that must not allocate device memory (a host arena that owns
all device memory, or offsets built during a stream capture): its scratch is a fixed device array
inside the library.  This file is collected last on purpose; it must pass both alone in a fresh
process and after the other GPU tests.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lib():
    import warp_gb300._native as N

    L = N.lib()
    L.gb_scan_i32_noalloc.restype = ctypes.c_int
    L.gb_scan_i32_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                      ctypes.c_void_p]
    L.gb_scan_i32_noalloc_max_n.restype = ctypes.c_int64
    L.gb_scan_i32_noalloc_max_n.argtypes = []
    return N, L


def _reference_scan(N, L, data, inclusive, stream):
    out = torch.empty_like(data)
    ws = torch.empty(max(int(L.gb_scan_i32_workspace_bytes(data.numel())), 256), dtype=torch.uint8, device="cuda")
    N.check(L.gb_scan_i32(data.data_ptr(), out.data_ptr(), data.numel(), inclusive, ws.data_ptr(), ws.numel(),
                          stream), "gb_scan_i32")
    return out


def test_scan_noalloc_matches_workspace_scan_on_two_calls_in_a_row(cuda):
    N, L = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2026)
    # two calls in a row for each case: the second must not see the first one's scratch contents
    for n, inclusive in [(10_000_019, 1), (10_000_019, 1), (4097, 0), (4097, 0), (123, 1), (70_000_000, 0)]:
        data = torch.from_numpy(rng.integers(0, 8, n).astype(np.int32)).cuda()
        ref = _reference_scan(N, L, data, inclusive, stream)
        out = torch.full_like(data, -1)
        N.check(L.gb_scan_i32_noalloc(data.data_ptr(), out.data_ptr(), n, inclusive, stream), "gb_scan_i32_noalloc")
        torch.cuda.synchronize()
        assert torch.equal(out, ref), (n, inclusive)
    # in place, as gb_scan_i32 allows
    data = torch.from_numpy(rng.integers(0, 8, 5_000_000).astype(np.int32)).cuda()
    ref = _reference_scan(N, L, data, 0, stream)
    N.check(L.gb_scan_i32_noalloc(data.data_ptr(), data.data_ptr(), data.numel(), 0, stream), "in place")
    torch.cuda.synchronize()
    assert torch.equal(data, ref)


def test_scan_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    N, L = _lib()
    limit = int(L.gb_scan_i32_noalloc_max_n())
    assert limit == 1 << 28
    dummy = torch.zeros(4, dtype=torch.int32, device="cuda")
    # rejected before anything touches the (too small) arrays
    rc = L.gb_scan_i32_noalloc(dummy.data_ptr(), dummy.data_ptr(), limit + 1, 1,
                               torch.cuda.current_stream().cuda_stream)
    assert rc != 0
    assert b"exceeds the fixed scratch" in L.gb_last_error()
