"""``bsr_mm``: BSR x BSR products through the triplet assembly (reference: ``sparse.py:4200-4624``).

z := alpha * x @ y + beta * z.  The product terms x[r,k] y[k,c] (and, when beta != 0, the
existing blocks of z) are emitted as triplets whose payload names the factor blocks; the
radix-sort assembly gives the output topology and each output block's run of terms in a stable
order; ``gb_spgemm_values`` sums the runs.  The result topology is the union of the product
pattern and z's pattern (explicit zeros are kept, as in the reference).  With ``masked=True`` (or
``topology="masked"``) z keeps its topology: the product terms go through the masked triplet
assembly, which keeps the terms that land on z's existing blocks, and z := alpha * (their sums) +
beta * z on those blocks (reference ``sparse.py:4200-4260``).
"""

from __future__ import annotations

import torch

from . import _arrays as A
from . import _native as N
from . import sparse

N.register("gb_spgemm_count", N._c_int, [N._c_int, N._vp, N._vp, N._vp, N._c_int, N._vp, N._vp])
N.register("gb_spgemm_emit", N._c_int, [N._c_int, N._vp, N._vp, N._vp, N._vp, N._c_int, N._vp, N._c_int, N._vp,
                                        N._vp, N._c_int, N._c_int, N._vp, N._vp, N._vp, N._vp])
N.register("gb_spgemm_values", N._c_int, [N._c_int, N._c_int, N._vp, N._vp, N._vp, N._vp, N._c_int, N._c_int,
                                          N._c_int, N._vp, N._vp, N._vp, N._c_dbl, N._c_dbl, N._vp, N._c_int, N._vp])


@A.on_caller_stream
def bsr_mm(x: sparse.BsrMatrix, y: sparse.BsrMatrix, z: sparse.BsrMatrix | None = None, alpha: float = 1.0,
           beta: float = 0.0, masked: bool = False, topology: str | None = None) -> sparse.BsrMatrix:
    if x.ncol != y.nrow:
        raise ValueError(f"Incompatible shapes: x has {x.ncol} block columns, y has {y.nrow} block rows")
    if x.block_shape[1] != y.block_shape[0]:
        raise ValueError("Incompatible block shapes")
    if x.scalar_type != y.scalar_type:
        raise ValueError("x and y must have the same scalar type")
    if topology is None:
        topology = "masked" if masked else "compact"
    elif topology not in ("compact", "masked"):
        raise NotImplementedError(f"bsr_mm topology {topology!r} is not supported (compact or masked)")
    masked = topology == "masked"
    if masked and z is None:
        raise ValueError("masked bsr_mm needs the destination matrix z")
    br, bk = x.block_shape
    bc = y.block_shape[1]
    dt = x.scalar_type
    block_type = dt if (br, bc) == (1, 1) else ((br, bc), dt)
    if z is None:
        z = sparse.bsr_zeros(x.nrow, y.ncol, block_type)
        beta = 0.0
    if (z.nrow, z.ncol) != (x.nrow, y.ncol) or z.block_shape != (br, bc):
        raise ValueError("Incompatible z")
    L = N.lib()
    stream = A.stream()
    xn = x.nnz_sync()
    yn = y.nnz_sync()
    zn = z.nnz_sync() if (beta != 0.0 and not masked) else 0
    count = A.empty(max(xn, 1), torch.int32)
    N.check(L.gb_spgemm_count(x.nrow, A.ptr(x.offsets), A.ptr(x.columns), A.ptr(y.offsets), xn, A.ptr(count),
                              stream), "spgemm_count")
    start = A.empty(max(xn, 1), torch.int32)
    ws = A.workspace(L.gb_scan_i32_workspace_bytes(max(xn, 1)))
    if xn > 0:
        N.check(L.gb_scan_i32(A.ptr(count), A.ptr(start), xn, 0, ws.data_ptr(), ws.numel(), stream), "scan")
        nprod = int(start[xn - 1].item()) + int(count[xn - 1].item())
    else:
        nprod = 0
    if masked:
        return _masked_product(x, y, z, alpha, beta, count, start, xn, nprod, L, stream)
    T = nprod + zn
    if T == 0:
        sparse.bsr_set_zero(z)
        return z
    rows = A.empty(T, torch.int32)
    cols = A.empty(T, torch.int32)
    pairs = A.empty((T, 2), torch.int32)
    N.check(L.gb_spgemm_emit(x.nrow, A.ptr(x.offsets), A.ptr(x.columns), A.ptr(y.offsets), A.ptr(y.columns), xn,
                             A.ptr(start), z.nrow, A.ptr(z.offsets) if zn else None, A.ptr(z.columns) if zn else None,
                             zn, nprod, A.ptr(rows), A.ptr(cols), A.ptr(pairs), stream), "spgemm_emit")
    out = sparse.BsrMatrix(x.nrow, y.ncol, (br, bc), dt)
    out.columns = A.empty(T, torch.int32)
    tbo = A.empty(T, torch.int32)
    tbi = A.empty(T, torch.int32)
    ws2 = A.workspace(L.gb_bsr_from_triplets_workspace_bytes(T, out.nrow, out.ncol))
    N.check(L.gb_bsr_matrix_from_triplets_device(1, 0, out.nrow, out.ncol, T, None, A.ptr(rows), A.ptr(cols), None,
                                                 0, 0, A.ptr(tbo), A.ptr(tbi), A.ptr(out.offsets), None,
                                                 A.ptr(out.columns), None, None, ws2.data_ptr(), ws2.numel(), stream),
            "spgemm_topology")
    nnz = int(out.offsets[out.nrow].item())
    vals = A.empty(out._values_shape(max(nnz, 1)), dt)
    N.check(L.gb_spgemm_values(A.gb_dtype(dt), out.nrow, A.ptr(out.offsets), A.ptr(tbo), A.ptr(tbi), A.ptr(pairs),
                               br, bk, bc, A.ptr(x.values), A.ptr(y.values), A.ptr(z.values) if zn else None,
                               float(alpha), float(beta), A.ptr(vals), nnz, stream), "spgemm_values")
    z.offsets, z.columns, z.values = out.offsets, out.columns[: max(nnz, 1)], vals
    z.row_counts = None
    z.nnz = nnz
    z._nnz_event = None
    z._nnz_exact = True
    z._topology_version += 1
    return z


def _masked_product(x, y, z, alpha, beta, count, start, xn, nprod, L, stream):
    """z := alpha x y + beta z on z's existing blocks only."""
    br, bk = x.block_shape
    bc = y.block_shape[1]
    dt = x.scalar_type
    z.nnz_sync()
    if beta != 1.0:
        z.values.mul_(beta) if beta != 0.0 else z.values.zero_()
    if nprod == 0:
        return z
    rows = A.empty(nprod, torch.int32)
    cols = A.empty(nprod, torch.int32)
    pairs = A.empty((nprod, 2), torch.int32)
    N.check(L.gb_spgemm_emit(x.nrow, A.ptr(x.offsets), A.ptr(x.columns), A.ptr(y.offsets), A.ptr(y.columns), xn,
                             A.ptr(start), z.nrow, None, None, 0, nprod, A.ptr(rows), A.ptr(cols), A.ptr(pairs),
                             stream), "spgemm_emit")
    # the masked assembly reads z's structure from its offsets / columns arguments and overwrites them
    # with the sub-structure of the blocks the terms hit: run it on copies
    sub_off = z.offsets.clone()
    mcols = torch.full((max(nprod, int(z.columns.shape[0])),), -1, dtype=torch.int32, device=z.device)
    mcols[: z.columns.shape[0]].copy_(z.columns)
    tbo = A.empty(nprod, torch.int32)
    tbi = A.empty(nprod, torch.int32)
    ws = A.workspace(L.gb_bsr_from_triplets_workspace_bytes(nprod, z.nrow, z.ncol))
    N.check(L.gb_bsr_matrix_from_triplets_device(1, 0, z.nrow, z.ncol, nprod, None, A.ptr(rows), A.ptr(cols), None,
                                                 0, 1, A.ptr(tbo), A.ptr(tbi), A.ptr(sub_off), A.ptr(z.row_counts),
                                                 A.ptr(mcols), None, None, ws.data_ptr(), ws.numel(), stream),
            "spgemm_topology(masked)")
    nsub = int(sub_off[z.nrow].item())
    if nsub == 0:
        return z
    sub_vals = A.empty(z._values_shape(nsub), dt)
    N.check(L.gb_spgemm_values(A.gb_dtype(dt), z.nrow, A.ptr(sub_off), A.ptr(tbo), A.ptr(tbi), A.ptr(pairs), br, bk,
                               bc, A.ptr(x.values), A.ptr(y.values), None, float(alpha), 0.0, A.ptr(sub_vals), nsub,
                               stream), "spgemm_values(masked)")
    sparse._scatter_sub_structure(z, sub_off, mcols, sub_vals, add=True)
    return z
