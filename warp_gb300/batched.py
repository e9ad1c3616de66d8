"""Batched Jacobi-CG for thousands of independent sparse SPD systems in one persistent launch.

Reference: batched ``LinearOperator`` / ``cg`` (``warp/_src/optim/linear.py:33-133, 893-1121``):
``batch_offsets[B+1]`` partitions the scalar rows of a block-diagonal operator into B independent
subproblems, each with its own tolerance ``max(rtol ||b_i||, atol)`` and its own CG scalars; rows at
or beyond ``batch_offsets[B]`` are inactive.  Here the whole batch is one launch of
``gb_batched_pcg`` (each CTA -- or, for small subproblems, each warp -- runs one subproblem's CG to
its own convergence, pulling work from a largest-first queue), optionally captured in a CUDA graph.

The launch configuration (threads per CTA, lanes per matrix row, the size below which a single warp
solves a subproblem) is picked by ``autotune``, which times every candidate on the batch itself and
caches the winner per batch layout.
"""

from __future__ import annotations

import hashlib
import itertools

import numpy as np
import torch

from . import _arrays as A
from . import _native as N
from . import sparse

DEFAULT_CONFIG = {"threads": 512, "lanes_per_row": 2, "small_rows": 2048, "smem_rows": 0}
# smem_rows: CTA-mode subproblems of at most this many rows keep p, r, Ap in shared memory (16896 rows =
# 198 KB: every subproblem of a 128 x 128-cell batch fits, one CTA per SM; 8192: two CTAs per SM).  On
# the 4096-system workload it measured slower (194-454 ms against 161 ms: one or two CTAs per SM hide
# the matrix stream's latency worse than eight), so the default candidate set leaves it off.
CANDIDATES = {"threads": (128, 256, 512), "lanes_per_row": (1, 2, 4), "small_rows": (0, 1024, 4096),
              "smem_rows": (0,)}
_TUNED: dict = {}


def _layout_key(sizes: np.ndarray, nnz: int) -> str:
    h = hashlib.sha1(np.ascontiguousarray(sizes, np.int64).tobytes()).hexdigest()[:16]
    return f"{len(sizes)}:{nnz}:{h}"


class BatchedCG:
    """Persistent batched Jacobi-CG on a block-diagonal CSR (1x1 BSR, fp32) matrix.

    Args:
        Am: the block-diagonal matrix (global row / column indices).
        batch_offsets: [B+1] int array (device or host) of first rows; rows >= batch_offsets[B] inactive.
        inv_diag: Jacobi inverse diagonal (device fp32 [n]) or None.
        rtol, atol: per-subproblem tolerance max(rtol ||b_i||, atol) (already resolved by the caller).
        maxiter: per-subproblem iteration cap.
        config: launch configuration dict, "auto" (autotune on the first solve), or None (default).
        use_cuda_graph: capture the launch into a CUDA graph on the first solve and replay it.
    """

    method = "cg"

    def __init__(self, Am: sparse.BsrMatrix, batch_offsets, inv_diag=None, rtol: float = 1e-6, atol: float = 0.0,
                 maxiter: int = 0, config=None, use_cuda_graph: bool = True):
        if Am.block_shape != (1, 1) or Am.scalar_type != torch.float32 or Am.row_counts is not None:
            raise ValueError("batched CG: compact 1x1 float32 BSR matrix required")
        self.A = Am
        self.n = Am.nrow
        if isinstance(batch_offsets, torch.Tensor) or hasattr(batch_offsets, "__cuda_array_interface__"):
            offs = (batch_offsets if isinstance(batch_offsets, torch.Tensor) else A.as_tensor(batch_offsets)).reshape(-1)
        else:
            offs = torch.as_tensor(np.asarray(batch_offsets)).reshape(-1)
        host = offs.cpu().numpy().astype(np.int64)
        if host.size < 1 or np.any(np.diff(host) < 0) or host[0] < 0 or host[-1] > self.n:
            raise ValueError("batch_offsets must be non-decreasing, start >= 0 and end <= the row count")
        self.nbatch = int(host.size - 1)
        self.sizes = np.diff(host)
        self.batch_offsets = offs.to(device="cuda", dtype=torch.int32).contiguous()
        order = np.argsort(-self.sizes, kind="stable").astype(np.int32)
        self.order = A.from_numpy(order)
        self.inv_diag = inv_diag
        self.rtol, self.atol = float(rtol), float(atol)
        self.maxiter = int(maxiter) if maxiter else max(1, self.n // max(self.nbatch, 1))
        self.nnz = Am.nnz_sync()
        self.key = _layout_key(self.sizes, self.nnz)
        if config == "auto":
            self.config = _TUNED.get(self.key)
            self._autotune_pending = self.config is None
        else:
            self.config = dict(config) if config else dict(DEFAULT_CONFIG)
            self._autotune_pending = False
        self.use_cuda_graph = bool(use_cuda_graph)
        L = N.lib()
        self._ws = A.zeros(int(self._workspace_bytes(L)), torch.uint8)
        B = max(self.nbatch, 1)
        self.iters = A.zeros(B, torch.int32)
        self.rr = A.zeros(B, torch.float32)
        self.atol_sq = A.zeros(B, torch.float32)
        self.status = A.zeros(1, torch.int32)
        self._graph = None
        self._graph_key = None
        self.launches = 0

    def _workspace_bytes(self, L) -> int:
        return L.gb_batched_pcg_workspace_bytes(self.n)

    def _launch(self, b: torch.Tensor, x: torch.Tensor, cfg, stream) -> None:
        Am = self.A
        N.check(N.lib().gb_batched_pcg2(
            self.nbatch, A.ptr(self.batch_offsets), A.ptr(self.order), self.n, A.ptr(Am.offsets), A.ptr(Am.columns),
            A.ptr(Am.values), A.ptr(self.inv_diag), A.ptr(b), A.ptr(x), self.rtol, self.atol, self.maxiter, 0,
            int(cfg["threads"]), int(cfg["lanes_per_row"]), int(cfg["small_rows"]), int(cfg.get("smem_rows", 0)),
            int(cfg.get("grid", 0)),
            A.ptr(self.iters), A.ptr(self.rr), A.ptr(self.atol_sq), A.ptr(self._ws), self._ws.numel(),
            A.ptr(self.status), stream), "batched_pcg")
        self.launches += 2  # queue reset + the persistent kernel

    @A.on_caller_stream
    def solve(self, b, x) -> None:
        """x <- the batched solve of A x = b (x is the initial guess); stream-ordered, no host sync
        once tuned."""
        b = A.as_tensor(b).reshape(-1)
        x = A.as_tensor(x).reshape(-1)
        if b.numel() != self.n or x.numel() != self.n:
            raise ValueError("b and x must have one entry per matrix row")
        if self._autotune_pending:
            self.config = autotune(self, b, x)
            self._autotune_pending = False
        stream = A.stream()
        if not self.use_cuda_graph or torch.cuda.is_current_stream_capturing():
            self._launch(b, x, self.config, stream)
            return
        key = (b.data_ptr(), x.data_ptr(), tuple(sorted(self.config.items())))
        if self._graph is None or self._graph_key != key:
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                with torch.cuda.graph(g, stream=side):
                    self._launch(b, x, self.config, torch.cuda.current_stream().cuda_stream)
            torch.cuda.current_stream().wait_stream(side)
            self._graph, self._graph_key = g, key
        self._graph.replay()
        self.launches += 2

    def results(self):
        """(max iterations over subproblems [1], r.r [B], atol^2 [B]) as device tensors."""
        return self.iters.max().reshape(1), self.rr, self.atol_sq


class BatchedBiCGSTAB(BatchedCG):
    """Persistent batched BiCGSTAB (Jacobi or no preconditioner, right or left preconditioning) on the
    same block-diagonal layout: one CTA per subproblem, each to its own tolerance (reference: BiCGSTAB
    with ``batch_offsets``, ``warp/_src/optim/linear.py:1377-1574``).  ``config``: threads and lanes per
    row (the autotuner's CG table does not apply; default 256 threads, 1 lane per row)."""

    method = "bicgstab"

    def __init__(self, Am: sparse.BsrMatrix, batch_offsets, inv_diag=None, rtol: float = 1e-6, atol: float = 0.0,
                 maxiter: int = 0, left_precond: bool = False, config=None, use_cuda_graph: bool = True):
        self.left_precond = bool(left_precond)
        super().__init__(Am, batch_offsets, inv_diag, rtol, atol, maxiter,
                         config=dict(config) if isinstance(config, dict) else dict(DEFAULT_CONFIG),
                         use_cuda_graph=use_cuda_graph)

    def _workspace_bytes(self, L) -> int:
        return L.gb_batched_bicgstab_workspace_bytes(self.n)

    def _launch(self, b: torch.Tensor, x: torch.Tensor, cfg, stream) -> None:
        Am = self.A
        N.check(N.lib().gb_batched_bicgstab(
            self.nbatch, A.ptr(self.batch_offsets), A.ptr(self.order), self.n, A.ptr(Am.offsets), A.ptr(Am.columns),
            A.ptr(Am.values), A.ptr(self.inv_diag), A.ptr(b), A.ptr(x), self.rtol, self.atol, self.maxiter, 0,
            int(self.left_precond), int(cfg["threads"]), int(cfg["lanes_per_row"]), int(cfg.get("grid", 0)),
            A.ptr(self.iters), A.ptr(self.rr), A.ptr(self.atol_sq), A.ptr(self._ws), self._ws.numel(),
            A.ptr(self.status), stream), "batched_bicgstab")
        self.launches += 2


def autotune(solver: BatchedCG, b: torch.Tensor, x: torch.Tensor, candidates=None, repeats: int = 1, log=None):
    """Time every candidate configuration on the batch itself (same b, same initial x) with CUDA
    events and return the fastest; the result is cached per batch layout."""
    cands = candidates or CANDIDATES
    x0 = x.clone()
    best, best_ms = None, float("inf")
    stream = A.stream()
    for th, lpr, sm, sv in itertools.product(cands["threads"], cands["lanes_per_row"], cands["small_rows"],
                                             cands.get("smem_rows", (0,))):
        cfg = {"threads": th, "lanes_per_row": lpr, "small_rows": sm, "smem_rows": sv}
        x.copy_(x0)
        solver._launch(b, x, cfg, stream)  # warm-up (module load, caches)
        times = []
        for _ in range(repeats):
            x.copy_(x0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            solver._launch(b, x, cfg, stream)
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        ms = min(times)
        if log:
            log(f"  threads={th:4d} lanes/row={lpr} small_rows={sm:5d} smem_rows={sv:5d}: {ms:8.3f} ms")
        if ms < best_ms:
            best, best_ms = cfg, ms
    x.copy_(x0)
    best = dict(best, tuned_ms=best_ms)
    _TUNED[solver.key] = best
    return best


def as_block_csr(Aop) -> sparse.BsrMatrix:
    """A compact 1x1 fp32 BSR view of a batched operator: the BSR itself, or a CSR built once from a
    dense matrix or a diagonal (the reference's batched tests use both)."""
    bsr = getattr(Aop, "_bsr", None)
    if bsr is not None:
        if bsr.block_shape != (1, 1):
            raise NotImplementedError("batched CG: 1x1 BSR blocks only")
        return bsr
    src = getattr(Aop, "_source", None)
    if src is None:
        raise NotImplementedError("batched CG: BSR, dense or diagonal operators only")
    t = src.detach().to(torch.float32)
    if t.dim() == 2:
        nz = torch.nonzero(t, as_tuple=False)
        rows, cols = nz[:, 0].to(torch.int32), nz[:, 1].to(torch.int32)
        vals = t[nz[:, 0], nz[:, 1]].contiguous()
        n = t.shape[0]
    else:
        n = t.numel()
        rows = cols = torch.arange(n, dtype=torch.int32, device=t.device)
        vals = t.reshape(-1).contiguous()
    out = sparse.bsr_zeros(n, n, torch.float32)
    sparse.bsr_set_from_triplets(out, rows, cols, vals, prune_numerical_zeros=False)
    out.nnz_sync()
    return out


def q1_batch_2d(ncells, sigma: float = 1.0, corr_length: float = 0.1, seed: int = 0, return_fields: bool = False):
    """Block-diagonal system of independent Q1 diffusion problems on unit squares: subproblem i has
    ncells[i]^2 cells, a = exp(g) (g: squared-exponential GRF per cell), f ~ U[-1, 1] per node, zero
    Dirichlet boundary by projection.  Returns (BsrMatrix, b, batch_offsets)."""
    from . import fem

    ncells = np.asarray(ncells, np.int64)
    rows = (ncells + 1) ** 2
    nnz = (3 * ncells + 1) ** 2
    cells = ncells ** 2
    if rows.sum() >= 2 ** 31 or nnz.sum() >= 2 ** 31:
        raise ValueError("batch too large for int32 indices")
    row_off = np.concatenate([[0], np.cumsum(rows)]).astype(np.int32)
    nnz_off = np.concatenate([[0], np.cumsum(nnz)]).astype(np.int32)
    cell_off = np.concatenate([[0], np.cumsum(cells)]).astype(np.int32)
    rng = np.random.default_rng(seed)
    coef = np.empty(int(cells.sum()), np.float32)
    f = rng.uniform(-1.0, 1.0, int(rows.sum())).astype(np.float32)
    for i, n in enumerate(ncells):
        g = fem.gaussian_random_field((int(n), int(n)), corr_length, sigma, seed * 1_000_003 + i)
        coef[cell_off[i]:cell_off[i + 1]] = np.exp(g).reshape(-1)
    total = int(row_off[-1])
    Am = sparse.bsr_zeros(total, total, torch.float32)
    Am.offsets = A.empty(total + 1, torch.int32)
    Am.columns = A.empty(int(nnz_off[-1]), torch.int32)
    Am.values = A.empty(int(nnz_off[-1]), torch.float32)
    Am.nnz = int(nnz_off[-1])
    b = A.empty(total, torch.float32)
    dev = [A.from_numpy(v) for v in (ncells.astype(np.int32), row_off, nnz_off, cell_off, coef, f)]
    N.check(N.lib().gb_q1_batched_assemble_2d(len(ncells), *[A.ptr(t) for t in dev], total, A.ptr(Am.offsets),
                                              A.ptr(Am.columns), A.ptr(Am.values), A.ptr(b), A.stream()),
            "q1_batched_assemble_2d")
    torch.cuda.current_stream().synchronize()
    if return_fields:
        return Am, b, A.from_numpy(row_off), dict(coef=coef, f=f, cell_off=cell_off, row_off=row_off)
    return Am, b, A.from_numpy(row_off)


def shard(sizes, rank: int, world: int) -> np.ndarray:
    """Subproblems of ``rank`` when a batch is split over ``world`` GPUs (no collective on the data
    path: every rank computes the same deterministic split from the sizes alone).  Greedy
    largest-first assignment to the least-loaded rank by the estimated work rows^1.5 (Jacobi-CG
    iterations grow like the grid width); returns the rank's subproblem ids in increasing order."""
    sizes = np.asarray(sizes, np.float64)
    if world <= 1:
        return np.arange(len(sizes))
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    order = np.argsort(-sizes, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(sizes), np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += sizes[i] ** 1.5
    return np.nonzero(owner == rank)[0]
