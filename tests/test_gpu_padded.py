"""Padded BSR topology (reference warp/_src/sparse.py:1232-1420, :574-690): bsr_set_from_triplets with
topology="padded" writes the triplets' compact rows into the destination's row capacity, and rows that
do not fit are left empty and raise BSR_STATUS_ROW_CAPACITY_EXCEEDED (sticky status)."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _triplets(nrow, ncol, n, bs, seed):
    rng = np.random.default_rng(seed)
    rows = rng.integers(-1, nrow + 1, n).astype(np.int32)
    cols = rng.integers(-1, ncol + 1, n).astype(np.int32)
    vals = rng.standard_normal((n, bs)).astype(np.float32)
    vals[rng.random(n) < 0.1] = 0.0
    return rows, cols, vals


@pytest.mark.parametrize("bdim", [1, 3])
def test_padded_rows_hold_the_compact_rows(cuda, bdim):
    from warp_gb300 import sparse

    nrow, ncol, n = 200, 150, 1500
    bs = bdim * bdim
    rows, cols, vals = _triplets(nrow, ncol, n, bs, 3)
    o = oracle.bsr_from_triplets(nrow, ncol, rows, cols, vals, block_shape=(bdim, bdim))
    counts = np.diff(o["offsets"])
    cap = int(counts.max()) + 2
    bt = torch.float32 if bdim == 1 else ((3, 3), torch.float32)
    P = sparse.bsr_zeros(nrow, ncol, bt, row_capacity=cap)
    assert P.nnz == nrow * cap and P.row_counts is not None
    vd = torch.from_numpy(vals if bdim == 1 else vals.reshape(n, 3, 3)).cuda()
    sparse.bsr_set_from_triplets(P, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(),
                                 vd.reshape(n) if bdim == 1 else vd, topology="padded")
    assert P.status_sync() == sparse.BSR_STATUS_SUCCESS
    off = P.offsets.cpu().numpy()
    np.testing.assert_array_equal(off, np.arange(nrow + 1) * cap)
    np.testing.assert_array_equal(P.row_counts.cpu().numpy(), counts)
    pc = P.columns.cpu().numpy()
    pv = P.values.cpu().numpy().reshape(-1, bs)
    ov = np.asarray(o["values"]).reshape(-1, bs)
    for r in range(nrow):
        b, c = o["offsets"][r], counts[r]
        np.testing.assert_array_equal(pc[off[r]:off[r] + c], o["columns"][b:b + c])
        np.testing.assert_array_equal(pv[off[r]:off[r] + c], ov[b:b + c])
        assert not pv[off[r] + c:off[r + 1]].any()  # unused slots hold zeros
    # the padded matrix computes the same product as the compact one
    x = torch.randn(ncol * bdim, device="cuda")
    y = sparse.bsr_mv(P, x)
    exp = oracle.bsr_mv_f64(o["offsets"], o["columns"], ov.reshape(-1), x.cpu().numpy().astype(np.float64),
                            block_shape=(bdim, bdim))
    np.testing.assert_allclose(y.cpu().numpy().reshape(-1), exp, rtol=1e-5, atol=1e-5 * np.abs(exp).max())


def test_rows_over_capacity_are_emptied_and_raise_the_status(cuda):
    from warp_gb300 import sparse

    nrow, ncol, n = 64, 64, 600
    rows, cols, vals = _triplets(nrow, ncol, n, 1, 4)
    o = oracle.bsr_from_triplets(nrow, ncol, rows, cols, vals)
    counts = np.diff(o["offsets"])
    # per-row capacities: enough for even rows, one short for odd rows that have blocks
    caps = np.where(np.arange(nrow) % 2 == 0, counts, np.maximum(counts - 1, 0)).astype(np.int32)
    P = sparse.bsr_zeros(nrow, ncol, torch.float32, row_capacity=torch.from_numpy(caps).cuda())
    sparse.bsr_set_from_triplets(P, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(),
                                 torch.from_numpy(vals.reshape(n)).cuda(), topology="padded")
    over = (np.arange(nrow) % 2 == 1) & (counts > 0)
    assert over.any()
    assert P.status_sync() == sparse.BSR_STATUS_ROW_CAPACITY_EXCEEDED
    rc = P.row_counts.cpu().numpy()
    np.testing.assert_array_equal(rc[over], 0)
    np.testing.assert_array_equal(rc[~over], counts[~over])
    # sticky until cleared
    P.clear_status()
    assert P.status_sync() == sparse.BSR_STATUS_SUCCESS
    # emptying keeps the row capacity
    sparse.bsr_set_zero(P, topology="padded")
    np.testing.assert_array_equal(P.offsets.cpu().numpy()[1:], np.cumsum(caps))
    assert not P.row_counts.any()
