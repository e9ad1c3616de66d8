"""The drop-in boundary: arrays that only expose __cuda_array_interface__, Warp's current stream,
outputs in the caller's array type, and the C entry point bound through ctypes exactly as a
maintainer would bind it next to Warp's own declarations (warp/_src/context.py:7444-7466)."""

import ctypes
import sys
import types

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


class CAIArray:
    """A minimal device array that is not a torch tensor: only __cuda_array_interface__ (v3)."""

    def __init__(self, t: torch.Tensor):
        self._t = t  # keeps the memory alive; the library sees only the interface below
        self.__cuda_array_interface__ = {"data": (t.data_ptr(), False), "shape": tuple(t.shape),
                                         "typestr": _typestr(t.dtype),
                                         "strides": None, "version": 3, "stream": None}


def _typestr(dt):
    return {torch.float32: "<f4", torch.float64: "<f8", torch.int32: "<i4"}[dt]


def _fake_warp(stream: torch.cuda.Stream):
    """A stand-in for the warp module: get_stream / from_torch and an array type defined in a module
    named warp (what the library keys on)."""
    mod = types.ModuleType("warp")

    class array:  # noqa: N801 -- the name of Warp's array type
        def __init__(self, t):
            self.tensor = t
            self.__cuda_array_interface__ = t.__cuda_array_interface__

    array.__module__ = "warp"

    class Stream:
        def __init__(self, s):
            self.cuda_stream = s.cuda_stream

    mod.array = array
    mod.get_stream = lambda device=None: Stream(stream)
    mod.from_torch = lambda t: array(t)
    return mod


def _poisson(res=(12, 10, 8)):
    from warp_gb300 import problems

    s = problems.diffusion(res, sigma=1.0, seed=3)
    nnz = s.A.nnz_sync()
    return s.A, (s.A.offsets.cpu().numpy(), s.A.columns[:nnz].cpu().numpy(), s.A.values[:nnz].cpu().numpy())


def test_bsr_mv_runs_on_warps_current_stream_and_returns_a_warp_array(cuda, monkeypatch):
    from warp_gb300 import sparse

    A, host = _poisson()
    n = A.nrow
    xh = np.random.default_rng(0).standard_normal(n).astype(np.float32)
    x = torch.zeros(n, device="cuda")
    xsrc = torch.from_numpy(xh).cuda()
    torch.cuda.synchronize()
    ws = torch.cuda.Stream()
    wp = _fake_warp(ws)
    monkeypatch.setitem(sys.modules, "warp", wp)
    # the producer writes x on Warp's stream behind a ~20 ms spin: a call ordered on any other stream
    # would read the zeros
    with torch.cuda.stream(ws):
        torch.cuda._sleep(40_000_000)
        x.copy_(xsrc)
    y = sparse.bsr_mv(A, wp.array(x))
    assert type(y) is wp.array
    torch.cuda.synchronize()
    exp = oracle.bsr_mv_f64(*host, xh.astype(np.float64))
    np.testing.assert_allclose(y.tensor.cpu().numpy(), exp, rtol=1e-5, atol=1e-5 * np.abs(exp).max())


def test_scoped_stream_orders_the_call_on_the_given_stream(cuda):
    import warp_gb300
    from warp_gb300 import sparse

    A, host = _poisson()
    n = A.nrow
    xh = np.random.default_rng(1).standard_normal(n).astype(np.float32)
    x = torch.zeros(n, device="cuda")
    xsrc = torch.from_numpy(xh).cuda()
    y = torch.zeros(n, device="cuda")
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        torch.cuda._sleep(40_000_000)
        x.copy_(xsrc)
    with warp_gb300.ScopedStream(s):
        out = sparse.bsr_mv(A, CAIArray(x), CAIArray(y))
    assert isinstance(out, CAIArray)  # the caller's output array, written in place
    torch.cuda.synchronize()
    exp = oracle.bsr_mv_f64(*host, xh.astype(np.float64))
    np.testing.assert_allclose(y.cpu().numpy(), exp, rtol=1e-5, atol=1e-5 * np.abs(exp).max())


def test_assembly_and_solve_from_interface_only_arrays(cuda):
    """bsr_set_from_triplets and cg driven with arrays that are not torch tensors."""
    from warp_gb300 import sparse
    from warp_gb300.optim import linear
    from oracle import fem_q1

    r, c, v = fem_q1.assemble_triplets((9, 7), coef=1.0)
    nn = 10 * 8
    v = v + np.where(r == c, 1.0, 0.0).astype(np.float32)  # shift: SPD without boundary conditions
    A = sparse.bsr_zeros(nn, nn, torch.float32)
    sparse.bsr_set_from_triplets(A, CAIArray(torch.from_numpy(r).cuda()), CAIArray(torch.from_numpy(c).cuda()),
                                 CAIArray(torch.from_numpy(v).cuda()))
    o = oracle.bsr_from_triplets(nn, nn, r, c, v)
    nnz = A.nnz_sync()
    np.testing.assert_array_equal(A.offsets.cpu().numpy(), o["offsets"])
    np.testing.assert_array_equal(A.columns[:nnz].cpu().numpy(), o["columns"])
    np.testing.assert_array_equal(A.values[:nnz].cpu().numpy(), o["values"])
    b = torch.from_numpy(np.random.default_rng(2).uniform(-1, 1, nn).astype(np.float32)).cuda()
    x = torch.zeros(nn, device="cuda")
    it, err, atol = linear.cg(A, CAIArray(b), CAIArray(x), tol=1e-6, atol=0.0, maxiter=500,
                              M=linear.preconditioner(A, "diag"))
    assert err <= atol
    rel = np.linalg.norm(b.cpu().numpy() - oracle.bsr_mv_f64(o["offsets"], o["columns"], o["values"],
                                                             x.cpu().numpy().astype(np.float64)))
    assert rel <= 4e-6 * np.linalg.norm(b.cpu().numpy())


def test_ctypes_binding_of_the_triplet_entry_point(cuda):
    """Binds gb_bsr_matrix_from_triplets_device with the argument types a maintainer adds beside
    Warp's ctypes declarations and calls it with raw pointers from interface-only arrays."""
    import warp_gb300._native as N

    gb = ctypes.CDLL(N.LIB_PATH)
    gb.gb_bsr_matrix_from_triplets_device.argtypes = [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,      # block_size, scalar_size, rows, cols, nnz
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,        # tpl_nnz, rows, columns, values
        ctypes.c_uint64, ctypes.c_int,                                             # zero mask, masked
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,        # run ends, run ids, offsets, row_counts
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,                         # columns, nnz host ptr, nnz event
        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]                         # workspace, bytes, stream
    gb.gb_bsr_matrix_from_triplets_device.restype = ctypes.c_int
    gb.gb_bsr_from_triplets_workspace_bytes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    gb.gb_bsr_from_triplets_workspace_bytes.restype = ctypes.c_size_t
    rng = np.random.default_rng(11)
    nrow, ncol, n = 300, 250, 5000
    rows = rng.integers(-2, nrow + 2, n).astype(np.int32)
    cols = rng.integers(-2, ncol + 2, n).astype(np.int32)
    vals = rng.random(n).astype(np.float32)
    vals[rng.random(n) < 0.1] = 0.0
    dev = lambda a: CAIArray(torch.from_numpy(a).cuda())  # noqa: E731
    d_rows, d_cols, d_vals = dev(rows), dev(cols), dev(vals)
    d_runend, d_runidx = dev(np.zeros(n, np.int32)), dev(np.zeros(n, np.int32))
    d_off, d_bcols = dev(np.zeros(nrow + 1, np.int32)), dev(np.zeros(n, np.int32))
    ws = dev(np.zeros(int(gb.gb_bsr_from_triplets_workspace_bytes(n, nrow, ncol)) // 4 + 64, np.int32))
    nnz_host = (ctypes.c_int * 1)()
    p = lambda a: a.__cuda_array_interface__["data"][0]  # noqa: E731
    stream = torch.cuda.current_stream().cuda_stream
    rc = gb.gb_bsr_matrix_from_triplets_device(1, 4, nrow, ncol, n, None, p(d_rows), p(d_cols), p(d_vals),
                                               0x7FFFFFFF, 0, p(d_runend), p(d_runidx), p(d_off), None, p(d_bcols),
                                               ctypes.addressof(nnz_host), None, p(ws),
                                               ws.__cuda_array_interface__["shape"][0] * 4, stream)
    assert rc == 0, gb.gb_last_error
    torch.cuda.synchronize()
    ref = oracle.ref_bsr_from_triplets(nrow, ncol, rows, cols, vals) or oracle.bsr_from_triplets(nrow, ncol, rows,
                                                                                                 cols, vals)
    nb = int(nnz_host[0])
    assert nb == ref["nnz"]
    np.testing.assert_array_equal(d_off._t.cpu().numpy(), ref["offsets"])
    np.testing.assert_array_equal(d_bcols._t.cpu().numpy()[:nb], ref["columns"])
    np.testing.assert_array_equal(d_runend._t.cpu().numpy()[:nb], ref["tpl_block_offsets"])
