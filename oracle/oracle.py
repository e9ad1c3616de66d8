"""ctypes bindings to the C oracle (``liboracle.so``) and the compiled reference routine
(``_ref/libref_sparse.so``).  Test infrastructure only (see the package docstring)."""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(reference_root: str | None = None) -> None:
    """Compile ``liboracle.so`` (and ``_ref/`` when the Warp sources are present)."""
    cmd = ["make", "-s", "-C", _HERE]
    if reference_root is not None:
        cmd.append(f"REF_ROOT={reference_root}")
    subprocess.run(cmd, check=True)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_bsr_from_triplets.restype = ctypes.c_int64
        L.orc_bsr_from_triplets.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            _i32p, _i32p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
            _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p,
        ]
        L.orc_bsr_accumulate_f32.restype = None
        L.orc_bsr_accumulate_f32.argtypes = [ctypes.c_int, ctypes.c_int64, _i32p, _i32p, _f32p, _f32p]
        L.orc_bsr_mv_f32.restype = None
        L.orc_bsr_mv_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p, _f32p, _f32p,
                                     _f32p, ctypes.c_float, ctypes.c_float]
        L.orc_bsr_mv_f64.restype = None
        L.orc_bsr_mv_f64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p, _f32p, _f64p,
                                     _f64p, ctypes.c_double, ctypes.c_double]
        L.orc_bsr_abs_mv_f64.restype = None
        L.orc_bsr_abs_mv_f64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p, _f32p,
                                         _f64p, _f64p]
        L.orc_inverse_diagonal_f32.restype = None
        L.orc_inverse_diagonal_f32.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p, _f32p, _f32p]
        L.orc_pcg_f32.restype = ctypes.c_int
        L.orc_pcg_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, _f32p, _f32p,
                                  _f32p, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, _f64p, _f64p]
        L.orc_bicgstab_f32.restype = ctypes.c_int
        L.orc_bicgstab_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, _f32p, _f32p,
                                       _f32p, ctypes.c_double, ctypes.c_double, ctypes.c_int, _f64p, _f64p]
        L.orc_pcg_sample_seconds.restype = ctypes.c_double
        L.orc_pcg_sample_seconds.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, _f32p,
                                             _f32p, _f32p, ctypes.c_int, ctypes.c_int]
        L.orc_pcg_f64.restype = ctypes.c_int
        L.orc_pcg_f64.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f32p, _f32p, _f32p,
                                  _f64p, ctypes.c_double, ctypes.c_int, ctypes.c_int, _f64p]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_max_threads.argtypes = []
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's compiled host routine, or None when ``_ref/`` was not built."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libref_sparse.so")
        if not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        R.wp_bsr_matrix_from_triplets_host.restype = None
        R.wp_bsr_matrix_from_triplets_host.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            _i32p, _i32p, _i32p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_bool,
            _i32p, _i32p, _i32p, _i32p, _i32p, _i32p, ctypes.c_void_p,
        ]
        _REF = R
    return _REF


ZERO_MASK_F32 = 0x7FFFFFFF


def bsr_from_triplets(nrow, ncol, rows, cols, values=None, block_shape=(1, 1), prune_numerical_zeros=True,
                      masked_topology=None):
    """Oracle triplet->BSR (restates the reference device path; stable ordering).

    Returns dict(offsets, columns, values, tpl_block_offsets, tpl_block_indices, nnz)."""
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    n = rows.shape[0]
    bs = block_shape[0] * block_shape[1]
    vals = None if values is None else np.ascontiguousarray(values, dtype=np.float32).reshape(n, bs)
    tbo = np.zeros(max(n, 1), np.int32)
    tbi = np.zeros(max(n, 1), np.int32)
    offsets = np.zeros(nrow + 1, np.int32)
    columns = np.zeros(max(n, 1), np.int32)
    mo = mrc = mc = None
    if masked_topology is not None:
        mo, mrc, mc = (None if a is None else np.ascontiguousarray(a, np.int32) for a in masked_topology)
    mask = ZERO_MASK_F32 if (prune_numerical_zeros and vals is not None) else 0
    nb = lib().orc_bsr_from_triplets(
        bs, 4 if vals is not None else 0, nrow, ncol, n, _ptr(rows, _i32p), _ptr(cols, _i32p),
        vals.ctypes.data if vals is not None else None, mask, 1 if masked_topology is not None else 0,
        _ptr(mo, _i32p), _ptr(mrc, _i32p), _ptr(mc, _i32p),
        _ptr(tbo, _i32p), _ptr(tbi, _i32p), _ptr(offsets, _i32p), _ptr(columns, _i32p))
    out = dict(offsets=offsets, columns=columns[:nb].copy(), tpl_block_offsets=tbo[:nb].copy(),
               tpl_block_indices=tbi[:n].copy(), nnz=int(nb))
    if vals is not None:
        bv = np.zeros((max(nb, 1), bs), np.float32)
        lib().orc_bsr_accumulate_f32(bs, nb, _ptr(tbo, _i32p), _ptr(tbi, _i32p), _ptr(vals, _f32p), _ptr(bv, _f32p))
        out["values"] = bv[:nb].reshape(nb, *block_shape) if bs > 1 else bv[:nb, 0].copy()
    return out


def ref_bsr_from_triplets(nrow, ncol, rows, cols, values=None, block_size=1, prune_numerical_zeros=True):
    """Run the reference's own compiled host routine (sparse.cpp:267-413).

    Returns dict(offsets, columns, tpl_block_offsets, tpl_block_indices, nnz) or None when the
    reference library was not built here.  The host routine uses an unstable std::sort, so its
    ``tpl_block_indices`` order inside a run is unspecified; offsets/columns/run ends are not."""
    R = ref_lib()
    if R is None:
        return None
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    n = rows.shape[0]
    vals = None if values is None else np.ascontiguousarray(values, dtype=np.float32).reshape(n, block_size)
    tbo = np.zeros(max(n, 1), np.int32)
    tbi = np.zeros(max(n, 1), np.int32)
    offsets = np.zeros(nrow + 1, np.int32)
    columns = np.zeros(max(n, 1), np.int32)
    nnz_out = np.zeros(1, np.int32)
    mask = ZERO_MASK_F32 if (prune_numerical_zeros and vals is not None) else 0
    R.wp_bsr_matrix_from_triplets_host(
        block_size, 4 if vals is not None else 0, nrow, ncol, n, None, _ptr(rows, _i32p), _ptr(cols, _i32p),
        vals.ctypes.data if vals is not None else None, mask, False, _ptr(tbo, _i32p), _ptr(tbi, _i32p),
        _ptr(offsets, _i32p), None, _ptr(columns, _i32p), _ptr(nnz_out, _i32p), None)
    nb = int(nnz_out[0])
    return dict(offsets=offsets, columns=columns[:nb].copy(), tpl_block_offsets=tbo[:nb].copy(),
                tpl_block_indices=tbi[:n].copy(), nnz=nb)


def ref_bsr_compress(offsets, row_counts, columns, values, block_size=1, prune_numerical_zeros=True,
                     make_compact=True):
    """Run the reference's own compiled in-place compression (sparse.cpp:521-610,
    wp_bsr_compress_inplace_host, float32 values).  Returns dict(offsets, row_counts, columns, values,
    nnz) or None when the reference library was not built here."""
    R = ref_lib()
    if R is None:
        return None
    nrow = len(offsets) - 1
    off = np.array(offsets, np.int32)
    rc = None if row_counts is None else np.array(row_counts, np.int32)
    cols = np.array(columns, np.int32)
    vals = np.array(values, np.float32).reshape(len(cols), block_size)
    nnz = np.zeros(1, np.int32)
    R.wp_bsr_compress_inplace_host.restype = None
    R.wp_bsr_compress_inplace_host.argtypes = [
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_bool, ctypes.c_uint64,
        ctypes.c_bool, _i32p, _i32p, _i32p, ctypes.c_void_p, ctypes.c_bool, _i32p, ctypes.c_void_p]
    R.wp_bsr_compress_inplace_host(nrow, block_size, 4, 0, len(cols), bool(prune_numerical_zeros), 0,
                                   bool(make_compact), _ptr(off, _i32p), None if rc is None else _ptr(rc, _i32p),
                                   _ptr(cols, _i32p), vals.ctypes.data, True, _ptr(nnz, _i32p), None)
    n = int(nnz[0]) if make_compact else len(cols)
    return dict(offsets=off, row_counts=rc, columns=cols[:n].copy(), values=vals[:n].copy(), nnz=n)


def bsr_compress_rows(offsets, row_counts, columns, values, block_size=1, prune_numerical_zeros=True):
    """Restatement (pure Python, small inputs) of the reference's per-row in-place compression
    (warp/native/sparse_util.h:82-139) followed by compaction: per active row, zero blocks dropped
    when pruning (all scalars == 0), stable insertion sort by column, runs of equal columns summed
    in order (float32 arithmetic).  Returns compact (offsets, columns, values)."""
    nrow = len(offsets) - 1
    cols = [int(c) for c in columns]
    vals = np.array(values, np.float32).reshape(len(cols), block_size).copy()
    out_off, out_cols, out_vals = [0], [], []
    for r in range(nrow):
        beg = int(offsets[r])
        end = beg + int(row_counts[r]) if row_counts is not None else int(offsets[r + 1])
        blk = [(cols[b], vals[b].copy()) for b in range(beg, end)]
        if prune_numerical_zeros:
            blk = [(c if (c < 0 or np.any(v != 0)) else -1, v) for c, v in blk]
        order = sorted(range(len(blk)), key=lambda i: blk[i][0])  # stable
        blk = [blk[i] for i in order if blk[i][0] >= 0]
        i = 0
        while i < len(blk):
            c, acc = blk[i][0], blk[i][1].copy()
            i += 1
            while i < len(blk) and blk[i][0] == c:
                acc = (acc + blk[i][1]).astype(np.float32)
                i += 1
            out_cols.append(c)
            out_vals.append(acc)
        out_off.append(len(out_cols))
    return (np.array(out_off, np.int32), np.array(out_cols, np.int32),
            np.array(out_vals, np.float32).reshape(-1, block_size))


def bsr_mv_f32(offsets, columns, values, x, y=None, alpha=1.0, beta=0.0, block_shape=(1, 1)):
    br, bc = block_shape
    nrow = len(offsets) - 1
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1)
    y = np.zeros(nrow * br, np.float32) if y is None else np.array(y, np.float32).reshape(-1)
    lib().orc_bsr_mv_f32(br, bc, nrow, _ptr(offsets, _i32p), None, _ptr(columns, _i32p), _ptr(values, _f32p),
                         _ptr(x, _f32p), _ptr(y, _f32p), alpha, beta)
    return y


def bsr_mv_f64(offsets, columns, values, x, y=None, alpha=1.0, beta=0.0, block_shape=(1, 1)):
    br, bc = block_shape
    nrow = len(offsets) - 1
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    y = np.zeros(nrow * br, np.float64) if y is None else np.array(y, np.float64).reshape(-1)
    lib().orc_bsr_mv_f64(br, bc, nrow, _ptr(offsets, _i32p), None, _ptr(columns, _i32p), _ptr(values, _f32p),
                         _ptr(x, _f64p), _ptr(y, _f64p), alpha, beta)
    return y


def bsr_abs_mv_f64(offsets, columns, values, x, block_shape=(1, 1)):
    br, bc = block_shape
    nrow = len(offsets) - 1
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    y = np.zeros(nrow * br, np.float64)
    lib().orc_bsr_abs_mv_f64(br, bc, nrow, _ptr(offsets, _i32p), None, _ptr(columns, _i32p), _ptr(values, _f32p),
                             _ptr(x, _f64p), _ptr(y, _f64p))
    return y


def inverse_diagonal_f32(offsets, columns, values, block_size=1):
    nrow = len(offsets) - 1
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    out = np.zeros(nrow * block_size, np.float32)
    lib().orc_inverse_diagonal_f32(block_size, nrow, _ptr(offsets, _i32p), None, _ptr(columns, _i32p),
                                   _ptr(values, _f32p), _ptr(out, _f32p))
    return out


def _tol_pair(tol, atol, eps=1.0e-8):
    """Restates _get_tolerances (warp/_src/optim/linear.py:2018-2032) for fp32."""
    default_tol = eps ** 0.75
    min_tol = eps ** 2.25
    if tol is None and atol is None:
        tol = atol = default_tol
    elif tol is None:
        tol = atol
    elif atol is None:
        atol = tol
    return tol, max(atol, min_tol)


def pcg_f32(offsets, columns, values, b, x0=None, inv_diag=None, tol=None, atol=None, maxiter=0,
            block_shape=(1, 1), nthreads=1):
    br, bc = block_shape
    nrow = len(offsets) - 1
    n = nrow * br
    if not maxiter:
        maxiter = n
    tol, atol = _tol_pair(tol, atol)
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    b = np.ascontiguousarray(b, np.float32).reshape(-1)
    x = np.zeros(n, np.float32) if x0 is None else np.array(x0, np.float32).reshape(-1)
    dinv = None if inv_diag is None else np.ascontiguousarray(inv_diag, np.float32).reshape(-1)
    rr = np.zeros(1)
    at = np.zeros(1)
    it = lib().orc_pcg_f32(br, bc, nrow, _ptr(offsets, _i32p), _ptr(columns, _i32p), _ptr(values, _f32p),
                           _ptr(dinv, _f32p), _ptr(b, _f32p), _ptr(x, _f32p), tol, atol, int(maxiter), nthreads,
                           _ptr(rr, _f64p), _ptr(at, _f64p))
    return x, int(it), float(np.sqrt(rr[0])), float(np.sqrt(at[0]))


def bicgstab_f32(offsets, columns, values, b, x0=None, inv_diag=None, tol=None, atol=None, maxiter=0,
                 block_shape=(1, 1)):
    br, bc = block_shape
    nrow = len(offsets) - 1
    n = nrow * br
    if not maxiter:
        maxiter = n
    tol, atol = _tol_pair(tol, atol)
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    b = np.ascontiguousarray(b, np.float32).reshape(-1)
    x = np.zeros(n, np.float32) if x0 is None else np.array(x0, np.float32).reshape(-1)
    dinv = None if inv_diag is None else np.ascontiguousarray(inv_diag, np.float32).reshape(-1)
    rr = np.zeros(1)
    at = np.zeros(1)
    it = lib().orc_bicgstab_f32(br, bc, nrow, _ptr(offsets, _i32p), _ptr(columns, _i32p), _ptr(values, _f32p),
                                _ptr(dinv, _f32p), _ptr(b, _f32p), _ptr(x, _f32p), tol, atol, int(maxiter),
                                _ptr(rr, _f64p), _ptr(at, _f64p))
    return x, int(it), float(np.sqrt(rr[0])), float(np.sqrt(at[0]))


def pcg_sample_seconds(offsets, columns, values, inv_diag, b, iters, nthreads, block_shape=(1, 1)):
    """Time ``iters`` Jacobi-PCG iterations of the oracle on ``nthreads`` host threads."""
    br, bc = block_shape
    nrow = len(offsets) - 1
    x = np.zeros(nrow * br, np.float32)
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    b = np.ascontiguousarray(b, np.float32).reshape(-1)
    dinv = np.ascontiguousarray(inv_diag, np.float32).reshape(-1)
    return float(lib().orc_pcg_sample_seconds(br, bc, nrow, _ptr(offsets, _i32p), _ptr(columns, _i32p),
                                              _ptr(values, _f32p), _ptr(dinv, _f32p), _ptr(b, _f32p),
                                              _ptr(x, _f32p), int(iters), int(nthreads)))


def pcg_f64(offsets, columns, values, b, inv_diag=None, tol=1e-8, maxiter=10000, nthreads=1, block_shape=(1, 1),
            x0=None):
    """FP64-vector Jacobi-PCG to ``tol`` relative residual; returns (x, iterations, rel_residual)."""
    br, bc = block_shape
    nrow = len(offsets) - 1
    offsets = np.ascontiguousarray(offsets, np.int32)
    columns = np.ascontiguousarray(columns, np.int32)
    values = np.ascontiguousarray(values, np.float32)
    b = np.ascontiguousarray(b, np.float32).reshape(-1)
    x = np.zeros(nrow * br) if x0 is None else np.array(x0, np.float64).reshape(-1)
    dinv = None if inv_diag is None else np.ascontiguousarray(inv_diag, np.float32).reshape(-1)
    rel = np.zeros(1)
    it = lib().orc_pcg_f64(br, bc, nrow, _ptr(offsets, _i32p), _ptr(columns, _i32p), _ptr(values, _f32p),
                           _ptr(dinv, _f32p), _ptr(b, _f32p), _ptr(x, _f64p), float(tol), int(maxiter),
                           int(nthreads), _ptr(rel, _f64p))
    return x, int(it), float(rel[0])


def max_threads() -> int:
    return int(lib().orc_max_threads())


def bsr_to_dense(offsets, columns, values, ncol, block_shape=(1, 1)):
    br, bc = block_shape
    nrow = len(offsets) - 1
    D = np.zeros((nrow * br, ncol * bc), np.float64)
    vals = np.asarray(values, np.float64).reshape(-1, br, bc)
    for r in range(nrow):
        for k in range(offsets[r], offsets[r + 1]):
            c = columns[k]
            D[r * br:(r + 1) * br, c * bc:(c + 1) * bc] += vals[k]
    return D


def triplets_to_dense(nrow, ncol, rows, cols, values, block_shape=(1, 1)):
    br, bc = block_shape
    D = np.zeros((nrow * br, ncol * bc), np.float64)
    vals = np.asarray(values, np.float64).reshape(-1, br, bc)
    for i in range(len(rows)):
        r, c = rows[i], cols[i]
        if 0 <= r < nrow and 0 <= c < ncol:
            D[r * br:(r + 1) * br, c * bc:(c + 1) * bc] += vals[i]
    return D
