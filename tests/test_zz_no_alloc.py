"""The allocation-free prefix sum (gb_scan_i32_noalloc) against numpy.cumsum and gb_scan_i32.

gb_scan_i32_noalloc serves callers that cannot allocate device memory (an application whose own
arena owns all device memory and lets no library call cudaMalloc): its scratch is a fixed device
array inside the library.  This file is collected last on purpose; it must pass both alone in a
fresh process and after the other GPU tests.
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


def _workspace_scan(N, L, data, inclusive, stream):
    out = torch.empty_like(data)
    ws = torch.empty(max(int(L.gb_scan_i32_workspace_bytes(data.numel())), 256), dtype=torch.uint8, device="cuda")
    N.check(L.gb_scan_i32(data.data_ptr(), out.data_ptr(), data.numel(), inclusive, ws.data_ptr(), ws.numel(),
                          stream), "gb_scan_i32")
    return out


def _numpy_scan(host, inclusive):
    inc = np.cumsum(host, dtype=np.int64)
    ref = inc if inclusive else np.concatenate([[0], inc[:-1]])
    return ref.astype(np.int32)  # the sums wrap like int32 additions do on the GPU


def test_scan_noalloc_matches_cumsum_on_two_calls_in_a_row(cuda):
    N, L = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2026)
    # two calls in a row for each case: the second must not see the first one's scratch contents
    for n, inclusive in [(10_000_019, 1), (10_000_019, 1), (4097, 0), (4097, 0), (123, 1), (70_000_000, 0)]:
        host = rng.integers(0, 8, n).astype(np.int32)
        data = torch.from_numpy(host).cuda()
        out = torch.full_like(data, -1)
        N.check(L.gb_scan_i32_noalloc(data.data_ptr(), out.data_ptr(), n, inclusive, stream), "gb_scan_i32_noalloc")
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), _numpy_scan(host, inclusive)), (n, inclusive)
        assert torch.equal(out, _workspace_scan(N, L, data, inclusive, stream)), (n, inclusive)
    # in place, as gb_scan_i32 allows
    host = rng.integers(0, 8, 5_000_000).astype(np.int32)
    data = torch.from_numpy(host).cuda()
    N.check(L.gb_scan_i32_noalloc(data.data_ptr(), data.data_ptr(), data.numel(), 0, stream), "in place")
    torch.cuda.synchronize()
    assert np.array_equal(data.cpu().numpy(), _numpy_scan(host, 0))


def test_scan_noalloc_at_its_limit(cuda):
    """n = 2^28 exactly (the documented maximum) runs, twice in a row, and matches numpy."""
    N, L = _lib()
    limit = int(L.gb_scan_i32_noalloc_max_n())
    assert limit == 1 << 28
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(7)
    host = rng.integers(0, 4, limit, dtype=np.int8).astype(np.int32)
    data = torch.from_numpy(host).cuda()
    out = torch.empty_like(data)
    for inclusive in (1, 0):
        N.check(L.gb_scan_i32_noalloc(data.data_ptr(), out.data_ptr(), limit, inclusive, stream), "at the limit")
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        ref = _numpy_scan(host, inclusive)
        assert np.array_equal(got, ref), inclusive
    del data, out
    torch.cuda.empty_cache()


def test_scan_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    N, L = _lib()
    limit = int(L.gb_scan_i32_noalloc_max_n())
    dummy = torch.zeros(4, dtype=torch.int32, device="cuda")
    # rejected before anything touches the (too small) arrays
    rc = L.gb_scan_i32_noalloc(dummy.data_ptr(), dummy.data_ptr(), limit + 1, 1,
                               torch.cuda.current_stream().cuda_stream)
    assert rc != 0
    assert b"exceeds the fixed scratch" in L.gb_last_error()
