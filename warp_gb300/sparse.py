"""Block-sparse-row (BSR) matrices: the drop-in for ``warp.sparse`` on the FEM solve path.

Mirrors the reference interface (``warp/_src/sparse.py``): ``BsrMatrix`` (:103), ``bsr_zeros``
(:639), ``bsr_set_from_triplets`` (:1232), ``bsr_from_triplets``, ``bsr_mv`` (:4792),
``bsr_mm`` (:4200), ``bsr_get_diag`` (:2887), ``bsr_copy``, ``bsr_set_zero``.  Arrays are
exchanged through ``__cuda_array_interface__``; results are torch tensors.  Every numerical step
runs in the sm_103a library ``libwarp_gb300.so``.
"""

from __future__ import annotations

from typing import Any

import numpy as np
import torch

from . import _arrays as A
from . import _native as N

__all__ = [
    "BsrMatrix",
    "bsr_zeros",
    "bsr_set_zero",
    "bsr_set_from_triplets",
    "bsr_from_triplets",
    "bsr_mv",
    "bsr_mm",
    "bsr_get_diag",
    "bsr_copy",
    "bsr_scale",
    "bsr_compress",
]

# Zero masks for numerical-zero pruning, by scalar type (reference: sparse.py:991-1007).
_ZERO_MASK = {torch.float32: 0x7FFFFFFF, torch.float64: 0x7FFFFFFFFFFFFFFF, torch.float16: 0x7FFF,
              torch.bfloat16: 0x7FFF}


def _parse_block_type(block_type) -> tuple[tuple[int, int], torch.dtype]:
    """Accepts torch/numpy dtypes, strings, ``((br, bc), dtype)`` tuples and Warp matrix/scalar types."""
    if isinstance(block_type, tuple) and len(block_type) == 2 and isinstance(block_type[0], tuple):
        shape, dt = block_type
        return (int(shape[0]), int(shape[1])), _parse_scalar(dt)
    shape = getattr(block_type, "_shape_", None)
    if shape is not None and len(shape) == 2:
        return (int(shape[0]), int(shape[1])), _parse_scalar(getattr(block_type, "_wp_scalar_type_", torch.float32))
    return (1, 1), _parse_scalar(block_type)


def _parse_scalar(dt) -> torch.dtype:
    if isinstance(dt, torch.dtype):
        return dt
    if dt is float:
        return torch.float32
    name = getattr(dt, "__name__", None) or str(dt)
    name = name.replace("warp.types.", "").replace("<class '", "").replace("'>", "")
    table = {"float32": torch.float32, "float64": torch.float64, "float16": torch.float16,
             "bfloat16": torch.bfloat16, "f4": torch.float32, "f8": torch.float64}
    for k, v in table.items():
        if name.endswith(k):
            return v
    try:
        return {np.float32: torch.float32, np.float64: torch.float64}[np.dtype(dt).type]
    except Exception:
        raise TypeError(f"unsupported block type {block_type_repr(dt)}") from None


def block_type_repr(dt) -> str:
    return getattr(dt, "__name__", repr(dt))


BSR_STATUS_SUCCESS = 0
"""Sparse operation status code for success (reference ``sparse.py:82``)."""
BSR_STATUS_ROW_CAPACITY_EXCEEDED = 1
"""Sparse operation status code for insufficient padded row capacity (reference ``sparse.py:85``)."""


class BsrMatrix:
    """BSR matrix with the reference's attributes (``warp/_src/sparse.py:103-463``).

    Attributes:
        nrow, ncol: rows / columns of blocks.
        nnz: host-side upper bound of stored blocks (``nnz_sync()`` makes it exact).
        offsets: int32 tensor ``[nrow + 1]``.
        row_counts: ``None`` (compact topology) or int32 ``[nrow]`` active blocks per row (padded
            topology: row r owns ``[offsets[r], offsets[r + 1])`` and uses its first ``row_counts[r]``).
        columns: int32 tensor (capacity >= nnz).
        values: tensor ``[capacity]`` for 1x1 blocks or ``[capacity, br, bc]``.
    """

    def __init__(self, nrow: int, ncol: int, block_shape: tuple[int, int], scalar_type: torch.dtype):
        self.nrow = int(nrow)
        self.ncol = int(ncol)
        self._block_shape = (int(block_shape[0]), int(block_shape[1]))
        self._scalar_type = scalar_type
        self.offsets = A.zeros(self.nrow + 1, torch.int32)
        self.row_counts = None
        self.columns = A.empty(0, torch.int32)
        self.values = A.empty(self._values_shape(0), scalar_type)
        self.nnz = 0
        self._nnz_host = None
        self._nnz_event = None
        self._nnz_exact = True
        self._topology_version = 0
        self._status = None

    def _ensure_status(self) -> torch.Tensor:
        if self._status is None:
            self._status = A.zeros(1, torch.int32)
        return self._status

    def status_sync(self) -> int:
        """Sticky status of the sparse operations on this matrix (``BSR_STATUS_*``; reference
        ``sparse.py:265``): a padded construction that ran out of row capacity sets it."""
        if self._status is None:
            return BSR_STATUS_SUCCESS
        if torch.cuda.is_current_stream_capturing():
            raise RuntimeError("BsrMatrix.status_sync() cannot read the status during a CUDA graph capture")
        return int(self._status.item())

    def clear_status(self) -> None:
        if self._status is not None:
            self._status.zero_()

    def _values_shape(self, cap):
        return (cap,) if self._block_shape == (1, 1) else (cap, *self._block_shape)

    @property
    def block_shape(self) -> tuple[int, int]:
        return self._block_shape

    @property
    def block_size(self) -> int:
        return self._block_shape[0] * self._block_shape[1]

    @property
    def scalar_type(self) -> torch.dtype:
        return self.values.dtype

    @property
    def dtype(self):
        return self.values.dtype

    @property
    def shape(self) -> tuple[int, int]:
        return (self.nrow * self._block_shape[0], self.ncol * self._block_shape[1])

    @property
    def device(self):
        return self.offsets.device

    @property
    def scalar_values(self) -> torch.Tensor:
        return self.values.view(-1, *self._block_shape)

    @property
    def capacity(self) -> int:
        return min(int(self.columns.shape[0]), int(self.values.shape[0]))

    def nnz_sync(self) -> int:
        """Wait for the pending device->host nnz copy (or read ``offsets[nrow]``) and return it."""
        if self._nnz_exact and self._nnz_event is None:
            return self.nnz
        if torch.cuda.is_current_stream_capturing():
            raise RuntimeError("BsrMatrix.nnz_sync() cannot read the block count during a CUDA graph capture")
        self._nnz_exact = True
        if self._nnz_event is not None:
            self._nnz_event.synchronize()
            self.nnz = int(self._nnz_host[0])
            self._nnz_event = None
        else:
            self.nnz = int(self.offsets[self.nrow].item())
        return self.nnz

    def notify_nnz_changed(self, nnz: int | None = None) -> None:
        self._nnz_exact = nnz is not None
        if nnz is None:
            self._nnz_event = None
            self.nnz = max(self.nnz, self.capacity)
        else:
            self.nnz = int(nnz)
        self._topology_version += 1

    def uncompress_rows(self) -> torch.Tensor:
        counts = self.offsets[1:] - self.offsets[:-1]
        return torch.repeat_interleave(torch.arange(self.nrow, device=self.device, dtype=torch.int32),
                                       counts.long())

    def __matmul__(self, x):
        return bsr_mv(self, x)

    def numpy_dense(self) -> np.ndarray:
        """Dense host copy (tests / debugging)."""
        nnz = self.nnz_sync()
        off = A.to_numpy(self.offsets)
        cols = A.to_numpy(self.columns[:nnz])
        vals = A.to_numpy(self.values[:nnz].float() if self.values.dtype == torch.bfloat16 else self.values[:nnz])
        br, bc = self._block_shape
        D = np.zeros((self.nrow * br, self.ncol * bc), np.float64)
        vals = vals.reshape(-1, br, bc).astype(np.float64)
        rows = np.repeat(np.arange(self.nrow), np.diff(off[: self.nrow + 1]))
        for i in range(br):
            for j in range(bc):
                np.add.at(D, (rows * br + i, cols.astype(np.int64) * bc + j), vals[:, i, j])
        return D


def bsr_zeros(rows_of_blocks: int, cols_of_blocks: int, block_type=torch.float32, device=None, *,
              topology: str | None = None, row_capacity=None, nnz_capacity: int | None = None) -> BsrMatrix:
    """Empty BSR matrix (reference: ``sparse.py:639-690``).  ``row_capacity`` (an int, or an int32
    array of per-row capacities) gives the padded topology: every row owns that many block slots."""
    if topology is None:
        topology = "padded" if row_capacity is not None else "compact"
    elif topology not in ("compact", "padded"):
        raise ValueError(f"Unsupported topology policy: {topology}")
    shape, dt = _parse_block_type(block_type)
    bsr = BsrMatrix(rows_of_blocks, cols_of_blocks, shape, dt)
    _set_zero_topology(bsr, topology, row_capacity, nnz_capacity, preserve_row_capacity=False)
    return bsr


def _set_zero_topology(bsr: BsrMatrix, topology: str, row_capacity, nnz_capacity, preserve_row_capacity: bool):
    """Reference: ``_bsr_set_zero_topology`` (``sparse.py:574-636``)."""
    if nnz_capacity is not None and int(nnz_capacity) < 0:
        raise ValueError("nnz_capacity must be nonnegative")
    if row_capacity is not None and topology != "padded":
        raise ValueError("row_capacity requires topology='padded'")
    if topology == "padded":
        if row_capacity is not None:
            if isinstance(row_capacity, (int, np.integer)):
                rc = int(row_capacity)
                if rc < 0:
                    raise ValueError("row_capacity must be nonnegative")
                bsr.offsets = torch.arange(0, (bsr.nrow + 1) * rc, max(rc, 1), dtype=torch.int32,
                                           device=A.device())[: bsr.nrow + 1] if rc > 0 else A.zeros(bsr.nrow + 1,
                                                                                                   torch.int32)
                cap = bsr.nrow * rc
            else:
                caps = A.as_tensor(row_capacity)
                if caps.dim() != 1 or caps.shape[0] != bsr.nrow:
                    raise ValueError(f"row_capacity array must have shape ({bsr.nrow},), got {tuple(caps.shape)}")
                if caps.dtype != torch.int32:
                    raise TypeError("row_capacity array must have dtype int32")
                off = A.zeros(bsr.nrow + 1, torch.int32)
                torch.cumsum(caps, 0, out=off[1:])
                bsr.offsets = off
                cap = int(nnz_capacity) if nnz_capacity is not None else int(off[-1].item())
        elif preserve_row_capacity and bsr.row_counts is not None:
            cap = bsr.capacity
        else:
            bsr.offsets = A.zeros(bsr.nrow + 1, torch.int32)
            cap = 0
        cap = max(cap, int(nnz_capacity or 0))
        _ensure_fits(bsr, cap)
        bsr.row_counts = A.zeros(bsr.nrow, torch.int32)
        bsr._ensure_status()
        bsr.nnz = cap if row_capacity is not None or preserve_row_capacity else 0
    else:
        bsr.offsets = A.zeros(bsr.nrow + 1, torch.int32)
        bsr.row_counts = None
        bsr.nnz = 0
        if nnz_capacity:
            _ensure_fits(bsr, int(nnz_capacity))
    bsr._nnz_event = None
    bsr._nnz_exact = True
    bsr._topology_version += 1


@A.on_caller_stream
def bsr_set_zero(bsr: BsrMatrix, rows_of_blocks: int | None = None, cols_of_blocks: int | None = None, *,
                 topology: str = "compact", row_capacity=None, nnz_capacity: int | None = None):
    """Remove every block (reference: ``sparse.py:770-812``); ``topology="padded"`` keeps (or, with
    ``row_capacity``, sets) the row capacity and empties every row."""
    if topology not in ("compact", "padded", "masked"):
        raise ValueError(f"Unsupported topology policy: {topology}")
    if topology == "masked":
        bsr.values.zero_()
        return
    resized = rows_of_blocks is not None and int(rows_of_blocks) != bsr.nrow
    if rows_of_blocks is not None:
        bsr.nrow = int(rows_of_blocks)
    if cols_of_blocks is not None:
        bsr.ncol = int(cols_of_blocks)
    _set_zero_topology(bsr, topology, row_capacity, nnz_capacity,
                       preserve_row_capacity=(topology == "padded" and row_capacity is None and not resized))


def _ensure_fits(bsr: BsrMatrix, nnz: int) -> None:
    if bsr.columns.shape[0] < nnz:
        bsr.columns = A.empty(nnz, torch.int32)
    if bsr.values.shape[0] < nnz:
        bsr.values = A.empty(bsr._values_shape(nnz), bsr.values.dtype)


@A.on_caller_stream
def bsr_set_from_triplets(
    dest: BsrMatrix,
    rows,
    columns,
    values=None,
    count=None,
    prune_numerical_zeros: bool = True,
    masked: bool = False,
    topology: str | None = None,
) -> None:
    """Fill ``dest`` from COO triplets, discarding existing blocks (reference: ``sparse.py:1232-1519``).

    Invalid row/column indices are dropped; with ``prune_numerical_zeros`` blocks whose scalars
    are all (+/-)0 are dropped; duplicates are summed in triplet order.  The block count is
    copied to the host asynchronously (``dest.nnz`` is an upper bound until ``nnz_sync()``).
    """
    if topology is None:
        topology = "masked" if masked else "compact"
    elif topology not in ("compact", "masked", "padded"):
        raise ValueError(f"Unsupported topology policy: {topology}")
    elif masked and topology != "masked":
        raise ValueError("Cannot pass masked=True with a non-masked topology policy")
    masked = topology == "masked"

    rows = A.as_tensor(rows)
    columns = A.as_tensor(columns)
    if rows.shape[0] != columns.shape[0]:
        raise ValueError(f"Rows and columns arrays must have the same length, got {rows.shape[0]} and {columns.shape[0]}")
    if rows.dtype != torch.int32 or columns.dtype != torch.int32:
        raise TypeError("Rows and columns arrays must be of type int32")
    if count is not None:
        count = A.as_tensor(count)
        if tuple(count.shape) != (1,):
            raise ValueError(f"Count array must be a single-element array, got {tuple(count.shape)}")
        if count.dtype != torch.int32:
            raise TypeError("Count array must be of type int32")
    if values is not None:
        values = A.as_tensor(values)
        if values.shape[0] != rows.shape[0]:
            raise ValueError(f"Values and rows arrays must have the same length, got {values.shape[0]} and {rows.shape[0]}")
        if values.dtype != dest.scalar_type:
            raise ValueError(f"Scalar type of values array ({values.dtype}) should correspond to that of matrix ({dest.scalar_type})")
        if values.numel() != rows.shape[0] * dest.block_size:
            raise ValueError(f"Values array should hold {dest.block_size} scalars per triplet")
        if not values.is_contiguous():
            if prune_numerical_zeros:
                raise ValueError("Values array should be contiguous for numerical zero pruning")
            values = values.contiguous()

    nnz = int(rows.shape[0])
    if nnz == 0:
        if masked:
            dest.values.zero_()
            return
        bsr_set_zero(dest, topology="padded" if topology == "padded" else "compact")
        return
    if topology == "padded":
        _set_from_triplets_padded(dest, rows, columns, values, count, prune_numerical_zeros)
        return

    stream = A.stream()
    L = N.lib()
    if masked:
        _set_from_triplets_masked(dest, rows, columns, values, count, prune_numerical_zeros)
        return

    _ensure_fits(dest, nnz)
    scalar_size = dest.values.element_size() if values is not None else 0
    mask = _ZERO_MASK.get(dest.scalar_type, 0) if (prune_numerical_zeros and values is not None) else 0
    tbo = A.empty(nnz, torch.int32) if values is not None else None
    tbi = A.empty(nnz, torch.int32) if values is not None else None
    ws_bytes = L.gb_bsr_from_triplets_workspace_bytes(nnz, dest.nrow, dest.ncol)
    ws = A.workspace(ws_bytes)
    if dest._nnz_host is None:
        dest._nnz_host = torch.zeros(1, dtype=torch.int32, pin_memory=True)
    event = torch.cuda.Event()
    N.check(
        L.gb_bsr_matrix_from_triplets_device(
            dest.block_size, scalar_size, dest.nrow, dest.ncol, nnz, A.ptr(count), A.ptr(rows), A.ptr(columns),
            A.ptr(values), mask, 0, A.ptr(tbo), A.ptr(tbi), A.ptr(dest.offsets), None, A.ptr(dest.columns),
            dest._nnz_host.data_ptr(), None, ws.data_ptr(), ws.numel(), stream),
        "bsr_set_from_triplets")
    event.record()
    dest._nnz_event = event
    dest._nnz_exact = False
    dest.nnz = nnz
    dest.row_counts = None
    dest._topology_version += 1
    if values is not None:
        N.check(
            L.gb_bsr_accumulate_triplet_values(
                A.gb_dtype(dest.scalar_type), dest.block_size, dest.nrow, A.ptr(dest.offsets), A.ptr(tbo),
                A.ptr(tbi), A.ptr(values), A.ptr(dest.values), nnz, stream),
            "bsr_accumulate_triplet_values")
    # keep temporaries alive until the stream has consumed them
    dest._last_temporaries = (ws, tbo, tbi, rows, columns, values)


@A.on_caller_stream
def bsr_compress(src: BsrMatrix, prune_numerical_zeros: bool = True, inplace: bool = False,
                 topology: str | None = None) -> BsrMatrix:
    """Sort and coalesce the active blocks of every row (reference: ``sparse.py:1571-1640``).

    Active blocks are ``[offsets[r], offsets[r] + row_counts[r])`` (or ``offsets[r + 1]`` when
    ``row_counts`` is None); negative columns are inactive.  Zero blocks are dropped before
    coalescing when ``prune_numerical_zeros``; runs of equal columns are summed in their original
    order (the order the triplet path accumulates in).  ``topology="compact"`` (default) packs the
    rows into a compact CSR (new arrays; ``row_counts`` becomes None); ``"padded"`` keeps the row
    capacity and sets ``row_counts``.  Both ``inplace`` values run the same native in-place row pass.
    """
    if not isinstance(src, BsrMatrix):
        raise ValueError("bsr_compress() requires a BsrMatrix")
    if topology is None:
        topology = "compact"
    elif topology not in ("compact", "padded"):
        raise ValueError(f"Unsupported topology policy: {topology}")
    if src.nrow == 0:
        return src
    dt = A.gb_dtype(src.scalar_type)
    if dt not in (N.GB_F32, N.GB_F64):
        raise NotImplementedError("bsr_compress: float32 or float64 values")
    L = N.lib()
    stream = A.stream()
    counts = A.zeros(src.nrow + 1, torch.int32)
    mask = _ZERO_MASK[src.scalar_type] if prune_numerical_zeros else 0
    N.check(L.gb_bsr_compress_rows(src.block_size, dt, src.nrow, A.ptr(src.offsets), A.ptr(src.row_counts),
                                   A.ptr(src.columns), A.ptr(src.values), int(prune_numerical_zeros), mask,
                                   A.ptr(counts), stream), "bsr_compress_rows")
    if topology == "padded":
        src.row_counts = counts[: src.nrow]
        src._topology_version += 1
        return src
    cap = src.capacity
    new_off = A.empty(src.nrow + 1, torch.int32)
    new_cols = A.empty(cap, torch.int32)
    new_vals = A.empty(src._values_shape(cap), src.scalar_type)
    ws = A.workspace(L.gb_bsr_compact_workspace_bytes(src.nrow))
    N.check(L.gb_bsr_compact(src.block_size, dt, src.nrow, A.ptr(src.offsets), A.ptr(counts), A.ptr(src.columns),
                             A.ptr(src.values), A.ptr(new_off), A.ptr(new_cols), A.ptr(new_vals), A.ptr(ws),
                             ws.numel(), stream), "bsr_compact")
    src._last_temporaries = (src.offsets, src.columns, src.values, counts, ws)
    src.offsets, src.columns, src.values, src.row_counts = new_off, new_cols, new_vals, None
    src._nnz_host = torch.zeros(1, dtype=torch.int32, pin_memory=True)
    src._nnz_host.copy_(new_off[src.nrow:], non_blocking=True)
    event = torch.cuda.Event()
    event.record()
    src._nnz_event = event
    src._nnz_exact = False
    src.nnz = cap
    src._topology_version += 1
    return src


def _set_from_triplets_padded(dest, rows, columns, values, count, prune_numerical_zeros):
    """padded topology (reference ``sparse.py:1335-1420``): build the compact structure of the triplets,
    write each row into dest's existing row capacity (rows that do not fit are left empty and raise
    ``BSR_STATUS_ROW_CAPACITY_EXCEEDED``), then the block sums."""
    if dest.row_counts is None:
        # a compact matrix's rows become padded rows of their current extent
        dest.row_counts = A.zeros(dest.nrow, torch.int32)
    status = dest._ensure_status()
    tmp = BsrMatrix(dest.nrow, dest.ncol, dest.block_shape, dest.scalar_type)
    bsr_set_from_triplets(tmp, rows, columns, values, count, prune_numerical_zeros)
    L = N.lib()
    stream = A.stream()
    cap = dest.capacity
    block_map = A.empty(max(cap, 1), torch.int32) if values is not None else None
    N.check(L.gb_bsr_scatter_padded(dest.nrow, A.ptr(tmp.offsets), A.ptr(tmp.columns), A.ptr(dest.offsets),
                                    A.ptr(dest.row_counts), A.ptr(dest.columns), A.ptr(block_map), A.ptr(status),
                                    stream), "bsr_scatter_padded")
    if values is not None and cap > 0:
        total = int(dest.offsets[dest.nrow].item()) if not torch.cuda.is_current_stream_capturing() else cap
        N.check(L.gb_bsr_gather_blocks(A.gb_dtype(dest.scalar_type), dest.block_size, min(total, cap), A.ptr(block_map),
                                       A.ptr(tmp.values), A.ptr(dest.values), stream), "bsr_gather_blocks")
    dest._padded_temporaries = (tmp, block_map)
    dest._topology_version += 1


def _set_from_triplets_masked(dest, rows, columns, values, count, prune_numerical_zeros):
    """masked topology: keep dest's structure and sum only triplets that hit existing blocks."""
    nnz = int(rows.shape[0])
    L = N.lib()
    stream = A.stream()
    sub_off = A.empty(dest.nrow + 1, torch.int32)
    sub_cols = A.empty(nnz, torch.int32)
    tbo = A.empty(nnz, torch.int32)
    tbi = A.empty(nnz, torch.int32)
    ws = A.workspace(L.gb_bsr_from_triplets_workspace_bytes(nnz, dest.nrow, dest.ncol))
    scalar_size = dest.values.element_size() if values is not None else 0
    mask = _ZERO_MASK.get(dest.scalar_type, 0) if (prune_numerical_zeros and values is not None) else 0
    # the masked key pass reads dest's structure from the offsets/columns arguments, which are
    # also the outputs: run on copies so dest keeps its topology
    sub_off.copy_(dest.offsets)
    ncopy = min(nnz, int(dest.columns.shape[0]))
    mcols = torch.full((max(nnz, int(dest.columns.shape[0])),), -1, dtype=torch.int32, device=dest.device)
    mcols[: dest.columns.shape[0]].copy_(dest.columns)
    del ncopy, sub_cols
    N.check(
        L.gb_bsr_matrix_from_triplets_device(
            dest.block_size, scalar_size, dest.nrow, dest.ncol, nnz, A.ptr(count), A.ptr(rows), A.ptr(columns),
            A.ptr(values), mask, 1, A.ptr(tbo), A.ptr(tbi), A.ptr(sub_off), A.ptr(dest.row_counts),
            A.ptr(mcols), None, None, ws.data_ptr(), ws.numel(), stream),
        "bsr_set_from_triplets(masked)")
    # mcols now holds the sub-structure columns; sum run values and scatter into dest blocks
    dest.values.zero_()
    if values is None:
        return
    sub_vals = A.empty(dest._values_shape(nnz), dest.scalar_type)
    N.check(L.gb_bsr_accumulate_triplet_values(A.gb_dtype(dest.scalar_type), dest.block_size, dest.nrow,
                                               A.ptr(sub_off), A.ptr(tbo), A.ptr(tbi), A.ptr(values),
                                               A.ptr(sub_vals), nnz, stream), "accumulate(masked)")
    _scatter_sub_structure(dest, sub_off, mcols, sub_vals)


def _scatter_sub_structure(dest, sub_off, sub_cols, sub_vals, add: bool = False):
    """dest.values[block(r, c)] = sub_vals[k] (``add``: += ) for every block k = (r, c) of the
    sub-structure."""
    n_sub = int(sub_off[dest.nrow].item())
    if n_sub == 0:
        return
    counts = (sub_off[1:] - sub_off[:-1]).long()
    sub_rows = torch.repeat_interleave(torch.arange(dest.nrow, device=dest.device), counts)
    # position of (row, col) inside dest: dest columns are sorted per row
    keys_dest = dest.uncompress_rows().long() * dest.ncol + dest.columns[: int(dest.offsets[dest.nrow].item())].long()
    keys_sub = sub_rows * dest.ncol + sub_cols[:n_sub].long()
    pos = torch.searchsorted(keys_dest, keys_sub)
    if add:
        dest.values[pos] += sub_vals[:n_sub]
    else:
        dest.values[pos] = sub_vals[:n_sub]


@A.on_caller_stream
def bsr_from_triplets(rows_of_blocks: int, cols_of_blocks: int, rows, columns, values,
                      prune_numerical_zeros: bool = True) -> BsrMatrix:
    """Constructs a BSR matrix from triplets (reference: ``sparse.py`` ``bsr_from_triplets``)."""
    values = A.as_tensor(values)
    if values.dim() == 3:
        block_type = ((int(values.shape[1]), int(values.shape[2])), values.dtype)
    else:
        block_type = values.dtype
    Am = bsr_zeros(rows_of_blocks, cols_of_blocks, block_type)
    bsr_set_from_triplets(Am, rows, columns, values, prune_numerical_zeros=prune_numerical_zeros)
    return Am


@A.on_caller_stream
def bsr_copy(A_: BsrMatrix, scalar_type=None) -> BsrMatrix:
    out = BsrMatrix(A_.nrow, A_.ncol, A_.block_shape, A_.scalar_type if scalar_type is None else _parse_scalar(scalar_type))
    nnz = A_.nnz_sync()
    out.offsets = A_.offsets.clone()
    out.columns = A_.columns[:nnz].clone()
    out.values = A_.values[:nnz].to(out._scalar_type).clone()
    out.nnz = nnz
    out._nnz_exact = True
    return out


@A.on_caller_stream
def bsr_scale(x: BsrMatrix, alpha: float) -> BsrMatrix:
    x.values.mul_(alpha)
    return x


def _vec_view(v, n_scalars: int, dtype: torch.dtype, what: str) -> torch.Tensor:
    t = A.as_tensor(v)
    if t.dtype != dtype:
        raise ValueError(f"Incompatible '{what}' vector for bsr_mv: dtype {t.dtype}, expected {dtype}")
    if not t.is_contiguous():
        raise ValueError(f"'{what}' must be contiguous")
    if t.numel() != n_scalars:
        raise ValueError(f"Incompatible '{what}' vector for bsr_mv: {t.numel()} scalars, expected {n_scalars}")
    return t


@A.on_caller_stream
def bsr_mv(Am: BsrMatrix, x, y=None, alpha: float = 1.0, beta: float = 0.0, transpose: bool = False,
           work_buffer=None, tile_size: int = 0, _status: torch.Tensor | None = None):
    """``y := alpha * A x + beta * y`` (reference: ``sparse.py:4792-4913``).  Returns ``y`` (the
    caller's array when given; a new array of the caller's type -- ``wp.array`` for ``wp.array``
    inputs -- otherwise).  Runs on the caller's stream (Warp's current stream under Warp).

    ``x`` and ``y`` may alias (a work buffer then holds a copy of x).  ``tile_size`` > 0 sets the
    number of lanes cooperating on one block row (power of two <= 32).  Vectors may be float32 or
    float64 (fp64 vectors with fp32 values give an fp64 product).
    """
    br, bc = Am.block_shape
    nrow_out, ncol_in = (Am.ncol, Am.nrow) if transpose else (Am.nrow, Am.ncol)
    if transpose:
        br, bc = bc, br
    x_t = A.as_tensor(x)
    vec_dtype = x_t.dtype
    if vec_dtype not in (torch.float32, torch.float64):
        raise TypeError(f"bsr_mv: unsupported vector dtype {vec_dtype}")
    created = y is None
    if created:
        y_shape = (nrow_out,) if br == 1 else (nrow_out, br)
        y = A.empty(y_shape, vec_dtype)
        beta = 0.0
    y_t = A.as_tensor(y)
    x_t = _vec_view(x_t, ncol_in * bc, vec_dtype, "x")
    y_t = _vec_view(y_t, nrow_out * br, vec_dtype, "y")
    if x_t.data_ptr() == y_t.data_ptr():
        if work_buffer is None:
            work_buffer = torch.empty_like(y_t)
        wb = A.as_tensor(work_buffer)
        if wb.numel() < y_t.numel():
            raise ValueError(f"Work buffer size is insufficient, needs to be at least {y_t.numel()}, got {wb.numel()}")
        wb.view(-1)[: y_t.numel()].copy_(y_t.view(-1))
        x_t = wb.view(-1)[: y_t.numel()]
    if Am._nnz_event is not None and not torch.cuda.is_current_stream_capturing():
        Am.nnz_sync()  # exact block count for the tile heuristic (one-time host sync)
    vals = Am.values
    val_dtype = A.gb_dtype(vals.dtype)
    status = _status if _status is not None else _status_word()
    lanes = tile_size if tile_size > 0 else 0
    N.check(
        N.lib().gb_bsr_mv(
            Am.block_shape[0], Am.block_shape[1], Am.nrow, Am.ncol, max(int(Am.nnz), 0), Am.capacity,
            A.ptr(Am.offsets), A.ptr(Am.row_counts), A.ptr(Am.columns), A.ptr(vals), val_dtype, A.ptr(x_t),
            A.ptr(y_t), A.ptr(y_t), A.gb_dtype(vec_dtype), float(alpha), float(beta), 1 if transpose else 0, 0,
            lanes, -1, A.ptr(status), A.stream()),
        "bsr_mv")
    # a new output comes back in the caller's array type (wp.array for wp.array inputs)
    return A.like(x, y) if created else y


@A.on_caller_stream
def bsr_mv_into(Am: BsrMatrix, x, y, z, alpha: float = 1.0, beta: float = 0.0) -> None:
    """``z := alpha * A x + beta * y`` with distinct input ``y`` and output ``z`` (``y`` may be ``z``).

    This is the operator form the solvers use (``LinearOperator.matvec``); it avoids the extra
    copy the reference makes when ``z != y`` (``linear.py:161-164``).
    """
    br, bc = Am.block_shape
    x_t = _vec_view(x, Am.ncol * bc, A.as_tensor(x).dtype, "x")
    z_t = _vec_view(z, Am.nrow * br, x_t.dtype, "z")
    y_t = _vec_view(y, Am.nrow * br, x_t.dtype, "y") if (beta != 0.0 and y is not None) else z_t
    if x_t.data_ptr() == z_t.data_ptr():
        x_t = x_t.clone()
    N.check(
        N.lib().gb_bsr_mv(
            br, bc, Am.nrow, Am.ncol, max(int(Am.nnz), 0), Am.capacity, A.ptr(Am.offsets), A.ptr(Am.row_counts),
            A.ptr(Am.columns), A.ptr(Am.values), A.gb_dtype(Am.values.dtype), A.ptr(x_t), A.ptr(y_t), A.ptr(z_t),
            A.gb_dtype(x_t.dtype), float(alpha), float(beta), 0, 0, 0, -1, A.ptr(_status_word()), A.stream()),
        "bsr_mv")


_STATUS = {}


def _status_word() -> torch.Tensor:
    dev = torch.cuda.current_device()
    if dev not in _STATUS:
        _STATUS[dev] = A.zeros(4, torch.int32)
    return _STATUS[dev]


def device_status() -> int:
    """OR of the device status bits raised by kernels since the last ``clear_device_status()``."""
    return int(_status_word()[0].item())


def clear_device_status() -> None:
    _status_word().zero_()


@A.on_caller_stream
def bsr_get_diag(Am: BsrMatrix, out=None) -> torch.Tensor:
    """Diagonal blocks (zero where absent) (reference: ``sparse.py:2887``)."""
    br, bc = Am.block_shape
    shape = (Am.nrow,) if (br, bc) == (1, 1) else (Am.nrow, br, bc)
    out = A.empty(shape, Am.scalar_type) if out is None else A.as_tensor(out)
    N.check(N.lib().gb_bsr_get_diag(A.gb_dtype(Am.scalar_type), br, bc, Am.nrow, A.ptr(Am.offsets),
                                    A.ptr(Am.row_counts), A.ptr(Am.columns), A.ptr(Am.values), A.ptr(out),
                                    A.stream()), "bsr_get_diag")
    return out


@A.on_caller_stream
def bsr_mm(x: BsrMatrix, y: BsrMatrix, z: BsrMatrix | None = None, alpha: float = 1.0, beta: float = 0.0,
           masked: bool = False, work_arrays: Any = None, reuse_topology: bool = False, tile_size: int = 0,
           max_new_nnz: int | None = None, topology: Any = None) -> BsrMatrix:
    """``z := alpha * x @ y + beta * z`` (reference: ``sparse.py:4200-4624``).

    Implemented on the triplet assembly kernels: every product block x[r,k] y[k,c] becomes a
    triplet (r, c) that references the pair of factor blocks; the triplet sort gives the product
    topology and the per-run sums give the values (see ``warp_gb300.spgemm``).
    """
    from .spgemm import bsr_mm as _mm

    return _mm(x, y, z, alpha=alpha, beta=beta, masked=masked, topology=topology)
