"""Iterative linear solvers: the drop-in for ``warp.optim.linear`` on the FEM solve path.

Mirrors ``warp/_src/optim/linear.py``: ``LinearOperator`` (:33), ``aslinearoperator`` (:135),
``preconditioner`` (:236), ``cg`` (:1035) / ``CG`` (:893), ``bicgstab`` (:1577) / ``BiCGSTAB``
(:1377), with the same arguments, tolerance rules (:2010-2083) and return conventions:

* ``check_every > 0``: returns ``(iterations, residual_norm, absolute_tolerance)`` (host numbers);
* ``check_every == 0``: returns device arrays ``(iterations[1], residual_norm_sq[1],
  atol_sq[1])`` and performs no host synchronisation -- the whole solve is one CUDA graph with a
  device-side while loop (and may itself be captured by the caller);
* ``run=False``: returns the pre-allocated solver functor.

BSR operators with 1x1 or 3x3 float32 (or bfloat16-valued) blocks and the Jacobi / identity
preconditioner take the fused native path of ``libwarp_gb300.so`` (three kernels per CG
iteration, single-pass grid reductions, conditional-while CUDA graph).  Any other
``LinearOperator`` (dense, user-defined matvec, batched) runs the generic path, whose vector
updates and dot products are also library kernels.

Additions beyond the reference: ``solve_refined`` (FP32 Krylov inside FP64 iterative
refinement, FP64 true residual and solution) and ``fcg`` (flexible CG with a nonlinear
preconditioner and a Jacobi-CG fallback), used by the learned preconditioner.
"""

from __future__ import annotations

import ctypes
import math
from typing import Callable

import numpy as np
import torch

from .. import _arrays as A
from .. import _native as N
from .. import sparse

__all__ = [
    "FCG",
    "fcg",
    "LinearOperator",
    "aslinearoperator",
    "preconditioner",
    "cg",
    "bicgstab",
    "CG",
    "BiCGSTAB",
    "CR",
    "cr",
    "GMRES",
    "gmres",
    "solve_refined",
]


class LinearOperator:
    """Linear operator for the iterative solvers (reference: ``linear.py:33-133``).

    ``matvec(x, y, z, alpha, beta)`` computes ``z = alpha * A x + beta * y``.
    """

    def __init__(self, shape, dtype, device, matvec: Callable, batch_offsets=None, max_batch_length=None):
        if max_batch_length is not None:
            if batch_offsets is None:
                raise ValueError("max_batch_length requires batch_offsets")
            if max_batch_length < 0:
                raise ValueError("max_batch_length must be non-negative")
        self._shape = tuple(shape)
        self._dtype = dtype
        self._device = device
        self._matvec = matvec
        self._batch_offsets = batch_offsets
        self._max_batch_length = max_batch_length
        self._bsr = None  # set for BSR operators (fused path)
        self._inv_diag = None  # set for Jacobi preconditioners (fused path)
        self._source = None  # the dense matrix / diagonal of array operators (batched path)

    @property
    def shape(self):
        return self._shape

    @property
    def dtype(self):
        return self._dtype

    @property
    def device(self):
        return self._device

    @property
    def matvec(self):
        return self._matvec

    @property
    def scalar_type(self):
        return self._dtype

    @property
    def batch_offsets(self):
        return self._batch_offsets

    @property
    def batch_count(self) -> int:
        return 1 if self._batch_offsets is None else int(self._batch_offsets.shape[0]) - 1

    @property
    def max_batch_length(self):
        return self._max_batch_length


def _flat(t) -> torch.Tensor:
    return A.as_tensor(t).reshape(-1)


def aslinearoperator(Am, batch_offsets=None, max_batch_length=None) -> LinearOperator | None:
    """Cast a BSR matrix, dense 2-D array or diagonal 1-D array (reference: ``linear.py:135-233``)."""
    if Am is None or isinstance(Am, LinearOperator):
        return Am
    stream_of = A.stream
    if isinstance(Am, sparse.BsrMatrix):

        def bsr_mv(x, y, z, alpha, beta):
            sparse.bsr_mv_into(Am, x, y, z, alpha, beta)

        op = LinearOperator(Am.shape, Am.scalar_type, Am.device, bsr_mv, batch_offsets, max_batch_length)
        op._bsr = Am
        return op
    t = A.as_tensor(Am)
    if t.dim() == 2:
        m, n = t.shape
        tc = t.contiguous()

        def dense_mv(x, y, z, alpha, beta):
            N.check(N.lib().gb_dense_mv(A.gb_dtype(tc.dtype), m, n, A.ptr(tc), A.ptr(_flat(x)), A.ptr(_flat(y)),
                                        A.ptr(_flat(z)), float(alpha), float(beta), stream_of()), "dense_mv")

        op = LinearOperator(tuple(t.shape), t.dtype, t.device, dense_mv, batch_offsets, max_batch_length)
        op._source = tc
        return op
    if t.dim() in (1, 2) or t.dim() >= 1:
        td = t.reshape(-1).contiguous()

        def diag_mv(x, y, z, alpha, beta):
            N.check(N.lib().gb_diag_mv(A.gb_dtype(td.dtype), td.numel(), A.ptr(td), A.ptr(_flat(x)),
                                       A.ptr(_flat(y)), A.ptr(_flat(z)), float(alpha), float(beta), stream_of()),
                    "diag_mv")

        op = LinearOperator((td.numel(), td.numel()), t.dtype, t.device, diag_mv, batch_offsets, max_batch_length)
        op._source = td
        op._inv_diag = td
        return op
    raise ValueError(f"Unable to create LinearOperator from {Am}")


@A.on_caller_stream
def preconditioner(Am, ptype: str = "diag") -> LinearOperator | None:
    """``"diag"`` (Jacobi), ``"diag_abs"`` or ``"id"`` (reference: ``linear.py:236-280``)."""
    if ptype == "id":
        return None
    if ptype not in ("diag", "diag_abs"):
        raise ValueError(f"Unsupported preconditioner type '{ptype}'")
    use_abs = 1 if ptype == "diag_abs" else 0
    if isinstance(Am, sparse.BsrMatrix):
        br, bc = Am.block_shape
        if br != bc:
            raise ValueError("Jacobi preconditioner needs square blocks")
        dt = Am.scalar_type if Am.scalar_type in (torch.float32, torch.float64) else torch.float32
        vals = Am.values if Am.values.dtype == dt else Am.values.to(dt)
        inv = A.empty(Am.nrow * br, dt)
        N.check(N.lib().gb_bsr_inverse_diagonal(A.gb_dtype(dt), br, Am.nrow, A.ptr(Am.offsets),
                                                A.ptr(Am.row_counts), A.ptr(Am.columns), A.ptr(vals), use_abs,
                                                A.ptr(inv), A.stream()), "preconditioner")
        return aslinearoperator(inv)
    t = A.as_tensor(Am)
    if t.dim() == 2:
        d = torch.diagonal(t).clone()
        d = d.abs() if use_abs else d
        inv = torch.where(d == 0, torch.ones_like(d), 1.0 / d)
        return aslinearoperator(inv.contiguous())
    raise ValueError("Unsupported source matrix type for building diagonal preconditioner")


@A.on_caller_stream
def refresh_preconditioner(M: LinearOperator, Am, ptype: str = "diag") -> None:
    """Recompute a Jacobi preconditioner in place after ``Am``'s values changed (same structure)."""
    inv = M._inv_diag
    br = Am.block_shape[0]
    N.check(N.lib().gb_bsr_inverse_diagonal(A.gb_dtype(inv.dtype), br, Am.nrow, A.ptr(Am.offsets),
                                            A.ptr(Am.row_counts), A.ptr(Am.columns), A.ptr(Am.values),
                                            1 if ptype == "diag_abs" else 0, A.ptr(inv), A.stream()),
            "refresh_preconditioner")


# -------------------------------------------------------------------------------------------
# tolerance rules (reference: linear.py:2010-2032)
# -------------------------------------------------------------------------------------------
def _dtype_epsilon(dtype) -> float:
    if dtype == torch.float64:
        return 1.0e-16
    if dtype == torch.float16:
        return 1.0e-4
    return 1.0e-8


def _get_tolerances(dtype, tol, atol):
    eps = _dtype_epsilon(dtype)
    default_tol = eps ** (3 / 4)
    min_tol = eps ** (9 / 4)
    if tol is None and atol is None:
        tol = atol = default_tol
    elif tol is None:
        tol = atol
    elif atol is None:
        atol = tol
    return tol, max(atol, min_tol)


class _DevScalar:
    """A device scalar exposed through ``__cuda_array_interface__`` (views into solver state)."""

    def __init__(self, ptr: int, typestr: str, keep):
        self.__cuda_array_interface__ = {"shape": (1,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None, "stream": None}
        self._keep = keep


# -------------------------------------------------------------------------------------------
# solver state
# -------------------------------------------------------------------------------------------
class LinearSolverState:
    """Pre-allocated solver (reference: ``linear.py:722-878``)."""

    _kind = None

    def __init__(self, A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
                 use_cuda_graph=True):
        self._A = aslinearoperator(A_)
        self._M = aslinearoperator(M)
        self._b = A.as_tensor(b)
        self._x = A.as_tensor(x)
        self._tol = tol
        self._atol = atol
        self._callback = callback
        self._check_every = int(check_every)
        self._use_cuda_graph = bool(use_cuda_graph)
        self._scalar_type = self._A.scalar_type
        self._batch_count = self._A.batch_count
        n = self._b.numel()
        if maxiter is None or maxiter == 0:
            maxiter = n // self._batch_count
        self._maxiter = int(maxiter)
        self._native = None
        self._ws = None
        self.persistent_active = False
        self._fused = self._fused_eligible(self._A, self._M, self._b, self._x)
        if self._fused:
            self._create_native()

    # -- fused path -----------------------------------------------------------------------
    def _fused_eligible(self, Aop, Mop, b, x) -> bool:
        bsr = getattr(Aop, "_bsr", None)
        if bsr is None or Aop.batch_offsets is not None:
            return False
        if bsr.block_shape not in ((1, 1), (3, 3)) or bsr.row_counts is not None:
            return False
        if bsr.values.dtype not in (torch.float32, torch.bfloat16):
            return False
        if b.dtype != torch.float32 or x.dtype != torch.float32 or not b.is_contiguous() or not x.is_contiguous():
            return False
        if Mop is not None:
            inv = getattr(Mop, "_inv_diag", None)
            if inv is None or inv.dtype != torch.float32 or inv.numel() != b.numel():
                return False
        if bsr.columns.data_ptr() % 16 or bsr.values.data_ptr() % 16:
            return False
        return True

    def _create_native(self):
        bsr = self._A._bsr
        L = N.lib()
        nnz = bsr.nnz_sync()
        bdim = bsr.block_shape[0]
        vdt = A.gb_dtype(bsr.values.dtype)
        ws_bytes = L.gb_krylov_workspace_bytes(self._kind, bdim, bsr.nrow, nnz, vdt)
        self._ws = A.zeros(int(ws_bytes), torch.uint8)
        h = ctypes.c_void_p()
        N.check(L.gb_krylov_create(self._kind, bdim, bsr.nrow, nnz, bsr.capacity, vdt, 0, 0, 0,
                                   self._ws.data_ptr(), self._ws.numel(), ctypes.byref(h)), "krylov_create")
        self._native = h
        self._native_key = (bsr.nrow, nnz, bdim, vdt)
        active = ctypes.c_int(0)
        if self._kind == N.KRYLOV_CG:
            N.check(L.gb_krylov_set_persistent(h, 1 if getattr(self, "_persistent", True) else 0,
                                               ctypes.byref(active)), "krylov_set_persistent")
        self.persistent_active = bool(active.value)
        it = ctypes.c_void_p()
        rr = ctypes.c_void_p()
        at = ctypes.c_void_p()
        st = ctypes.c_void_p()
        N.check(L.gb_krylov_scalars(h, ctypes.byref(it), ctypes.byref(rr), ctypes.byref(at), ctypes.byref(st)))
        self._dev_iter = torch.as_tensor(_DevScalar(it.value, "<i4", self._ws), device="cuda")
        self._dev_rr = torch.as_tensor(_DevScalar(rr.value, "<f8", self._ws), device="cuda")
        self._dev_atol_sq = torch.as_tensor(_DevScalar(at.value, "<f8", self._ws), device="cuda")
        self._dev_status = torch.as_tensor(_DevScalar(st.value, "<i4", self._ws), device="cuda")
        self._host_i = torch.zeros(3, dtype=torch.int32, pin_memory=True)
        self._host_d = torch.zeros(3, dtype=torch.float64, pin_memory=True)

    def __del__(self):
        try:
            if self._native is not None:
                N.lib().gb_krylov_destroy(self._native)
                self._native = None
        except Exception:
            pass

    def _read(self):
        N.check(N.lib().gb_krylov_read(self._native, self._host_i.data_ptr(), self._host_d.data_ptr(), A.stream()))
        torch.cuda.current_stream().synchronize()
        it, cond, status = (int(v) for v in self._host_i.tolist())
        rr, atol_sq, bb = (float(v) for v in self._host_d.tolist())
        return it, cond, status, rr, atol_sq

    def _run_fused(self, Aop, b, x, Mop, x_is_zero=False):
        bsr = Aop._bsr
        L = N.lib()
        key = (bsr.nrow, bsr.nnz if bsr._nnz_exact and bsr._nnz_event is None else bsr.nnz_sync(),
               bsr.block_shape[0], A.gb_dtype(bsr.values.dtype))
        if key != self._native_key:
            raise ValueError("operator shape changed since the solver was created")
        rtol, atol = _get_tolerances(torch.float32, self._tol, self._atol)
        dinv = None if Mop is None else Mop._inv_diag
        stream = A.stream()
        N.check(L.gb_krylov_set_operands(self._native, A.ptr(bsr.offsets), None, A.ptr(bsr.columns),
                                         A.ptr(bsr.values), A.ptr(dinv), A.ptr(b), A.ptr(x), 1 if x_is_zero else 0,
                                         float(rtol), float(atol), self._maxiter,
                                         1 if getattr(self, "_is_left_preconditioner", False) else 0, stream),
                "krylov_set_operands")
        self._keep = (b, x, dinv, bsr)
        if self._check_every == 0:
            mode = 0 if self._use_cuda_graph else None
            if mode == 0:
                N.check(L.gb_krylov_launch(self._native, 0, 0, stream), "krylov_launch")
            else:
                N.check(L.gb_krylov_launch(self._native, 4, 0, stream), "krylov_launch")
                for _ in range(self._maxiter):
                    N.check(L.gb_krylov_launch(self._native, 3, 0, stream), "krylov_launch")
            return self._dev_iter, self._dev_rr, self._dev_atol_sq
        # host-checked loop
        graph = self._use_cuda_graph
        N.check(L.gb_krylov_launch(self._native, 1 if graph else 4, 0, stream), "krylov_launch")
        it, cond, status, rr, atol_sq = self._read()
        atol_v = math.sqrt(atol_sq)
        if self._callback is not None:
            self._callback(0, math.sqrt(rr), atol_v)
        chunk = max(1, self._check_every)
        while cond and it < self._maxiter:
            n = min(chunk, self._maxiter - it)
            if graph:
                N.check(L.gb_krylov_launch(self._native, 2, n, stream), "krylov_launch")
            else:
                for _ in range(n):
                    N.check(L.gb_krylov_launch(self._native, 3, 0, stream), "krylov_launch")
            it, cond, status, rr, atol_sq = self._read()
            if self._callback is not None:
                self._callback(it, math.sqrt(rr), atol_v)
        self.last_status = status
        return it, math.sqrt(rr), atol_v

    # -- public ---------------------------------------------------------------------------
    @A.on_caller_stream
    def __call__(self, A_=None, b=None, x=None, M=None):
        Aop = aslinearoperator(A_) if A_ is not None else self._A
        Mop = aslinearoperator(M) if M is not None else self._M
        b_t = A.as_tensor(b) if b is not None else self._b
        x_t = A.as_tensor(x) if x is not None else self._x
        if Aop is not self._A and tuple(Aop.shape) != tuple(self._A.shape):
            raise ValueError(f"Incompatible A.shape: expected {self._A.shape}, got {Aop.shape}")
        if b_t.shape != self._b.shape:
            raise ValueError(f"Incompatible b.shape: expected {tuple(self._b.shape)}, got {tuple(b_t.shape)}")
        if x_t.shape != self._x.shape:
            raise ValueError(f"Incompatible x.shape: expected {tuple(self._x.shape)}, got {tuple(x_t.shape)}")
        if self._A.batch_offsets is not None:
            if Aop is not self._A and Aop.batch_offsets is not self._A.batch_offsets:
                raise ValueError("A.batch_offsets must be the same array as at construction")
            return self._run_batched(Aop, b_t.reshape(-1), x_t.reshape(-1), Mop)
        if self._fused and self._fused_eligible(Aop, Mop, b_t, x_t):
            return self._run_fused(Aop, b_t, x_t, Mop)
        return self._run_generic(Aop, b_t.reshape(-1), x_t.reshape(-1), Mop)

    def _run_batched(self, Aop, b, x, Mop):
        raise NotImplementedError(f"{type(self).__name__}: batched operators (batch_offsets) are solved by cg and "
                                  "bicgstab")

    # -- generic path (any LinearOperator) ------------------------------------------------
    def _dots(self, pairs):
        L = N.lib()
        if not hasattr(self, "_dot_ws"):
            self._dot_ws = A.zeros(int(L.gb_dots_workspace_bytes()), torch.uint8)
            self._dot_out = A.zeros(4, torch.float64)
        xs = (ctypes.c_void_p * 4)(*[p[0].data_ptr() for p in pairs])
        ys = (ctypes.c_void_p * 4)(*[p[1].data_ptr() for p in pairs])
        dt = A.gb_dtype(pairs[0][0].dtype)
        N.check(L.gb_dots(dt, pairs[0][0].numel(), len(pairs), xs, ys, self._dot_out.data_ptr(),
                          self._dot_ws.data_ptr(), A.stream()), "dots")
        return [float(v) for v in self._dot_out[: len(pairs)].tolist()]

    def _axpby(self, alpha, x, beta, y, out):
        N.check(N.lib().gb_axpby(A.gb_dtype(x.dtype), x.numel(), float(alpha), x.data_ptr(), float(beta),
                                 y.data_ptr(), out.data_ptr(), A.stream()), "axpby")


class CG(LinearSolverState):
    """Pre-allocated Conjugate Gradient solver (reference: ``linear.py:893-1032``)."""

    _kind = N.KRYLOV_CG

    def __init__(self, A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
                 use_cuda_graph=True, restart=None, *, persistent: bool = True):
        """``persistent`` (not in the reference): on the fused path, run the iterations as one
        persistent cooperative launch (three phases per iteration separated by grid barriers) when
        the device holds the SpMV grid at once, else three kernels per iteration under a
        conditional graph node.  ``persistent_active`` tells which one runs."""
        self._persistent = bool(persistent)
        if restart is not None:
            if isinstance(restart, bool) or not isinstance(restart, int):
                raise TypeError("restart must be an integer or None")
            if restart < 1:
                raise ValueError("restart must be positive")
        self._restart = restart
        super().__init__(A_, b, x, tol, atol, maxiter, M, callback, check_every, use_cuda_graph)
        if restart is not None:
            self._fused = False

    def _run_batched(self, Aop, b, x, Mop):
        """Batched operator: the whole batch is one persistent launch (``warp_gb300.batched``);
        each subproblem converges to its own tolerance (reference: ``linear.py:893-1032``).  The
        callback, if any, sees the final state."""
        from .. import batched

        if self._restart is not None:
            raise NotImplementedError("batched CG with restart")
        if b.dtype != torch.float32 or x.dtype != torch.float32:
            raise NotImplementedError("batched CG: float32 systems")
        inv = None
        if Mop is not None:
            inv = getattr(Mop, "_inv_diag", None)
            if inv is None:
                raise NotImplementedError("batched CG: Jacobi ('diag') or no preconditioner")
        if getattr(self, "_batched", None) is None or self._batched_op is not Aop:
            csr = batched.as_block_csr(Aop)
            rtol, atol = _get_tolerances(torch.float32, self._tol, self._atol)
            cfg = "auto" if Aop.batch_count >= 256 else None
            self._batched = batched.BatchedCG(csr, Aop.batch_offsets, inv, rtol, atol, self._maxiter, config=cfg,
                                              use_cuda_graph=self._use_cuda_graph)
            self._batched_op = Aop
        self._batched.inv_diag = inv
        self._batched.solve(b, x)
        it, rr, atol_sq = self._batched.results()
        if self._check_every == 0:
            return it, rr, atol_sq
        it_h = int(it.item())
        err = math.sqrt(float(rr.max())) if rr.numel() else 0.0
        atol_v = math.sqrt(float(atol_sq.max())) if atol_sq.numel() else 0.0
        if self._callback is not None:
            self._callback(it_h, err, atol_v)
        return it_h, err, atol_v

    def _run_generic(self, Aop, b, x, Mop):
        dt = b.dtype
        rtol, atol = _get_tolerances(dt, self._tol, self._atol)
        n = b.numel()
        r = torch.empty_like(b)
        z = torch.empty_like(b) if Mop is not None else r
        p = torch.empty_like(b)
        Ap = torch.zeros_like(b)
        (bb,) = self._dots([(b, b)])
        atol_v = max(rtol * math.sqrt(bb), atol)
        atol_sq = atol_v * atol_v
        Aop.matvec(x, b, r, -1.0, 1.0)
        if Mop is not None:
            Mop.matvec(r, z, z, 1.0, 0.0)
        rr, rz = self._dots([(r, r), (r, z)])
        p.copy_(z)
        it = 0
        if self._callback is not None and self._check_every > 0:
            self._callback(0, math.sqrt(rr), atol_v)
        while not (rr <= atol_sq) and it < self._maxiter:
            Aop.matvec(p, Ap, Ap, 1.0, 0.0)
            (pAp,) = self._dots([(p, Ap)])
            alpha = rz / pAp if (rr > atol_sq and pAp != 0.0) else 0.0
            self._axpby(alpha, p, 1.0, x, x)
            self._axpby(-alpha, Ap, 1.0, r, r)
            if Mop is not None:
                Mop.matvec(r, z, z, 1.0, 0.0)
            rz_new, rr = self._dots([(r, z), (r, r)])
            beta = rz_new / rz if (rr > atol_sq and rz != 0.0) else 0.0
            self._axpby(1.0, z, beta, p, p)
            rz = rz_new
            it += 1
            if self._restart is not None and it % self._restart == 0:
                Aop.matvec(x, b, r, -1.0, 1.0)
                if Mop is not None:
                    Mop.matvec(r, z, z, 1.0, 0.0)
                rr, rz = self._dots([(r, r), (r, z)])
                p.copy_(z)
            if self._callback is not None and self._check_every > 0 and it % self._check_every == 0:
                self._callback(it, math.sqrt(rr), atol_v)
        if self._check_every == 0:
            return (torch.tensor([it], dtype=torch.int32, device=b.device),
                    torch.tensor([rr], dtype=torch.float64, device=b.device),
                    torch.tensor([atol_sq], dtype=torch.float64, device=b.device))
        return it, math.sqrt(rr), atol_v


def _generic_return(self, it, rr, atol_sq, device):
    if self._check_every == 0:
        return (torch.tensor([it], dtype=torch.int32, device=device),
                torch.tensor([rr], dtype=torch.float64, device=device),
                torch.tensor([atol_sq], dtype=torch.float64, device=device))
    return it, math.sqrt(rr), math.sqrt(atol_sq)


class CR(LinearSolverState):
    """Conjugate Residual (reference: ``linear.py:1124-1286``, kernels ``:2377-2423``): minimises the
    A-norm of the (preconditioned) residual for symmetric A; same tolerance rule and returns as
    ``CG``.  Runs on the generic path (library matvec / dot / axpby kernels, host-read scalars)."""

    def __init__(self, A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
                 use_cuda_graph=True, restart=None):
        if restart is not None and (isinstance(restart, bool) or not isinstance(restart, int) or restart < 1):
            raise ValueError("restart must be a positive integer")
        self._restart = restart
        super().__init__(A_, b, x, tol, atol, maxiter, M, callback, check_every, use_cuda_graph)

    def _fused_eligible(self, Aop, Mop, b, x) -> bool:
        return False

    def _run_generic(self, Aop, b, x, Mop):
        rtol, atol = _get_tolerances(b.dtype, self._tol, self._atol)
        r = torch.empty_like(b)
        z = torch.zeros_like(b) if Mop is not None else r
        Az = torch.zeros_like(b)
        y = torch.zeros_like(b) if Mop is not None else None
        (bb,) = self._dots([(b, b)])
        atol_v = max(rtol * math.sqrt(bb), atol)
        atol_sq = atol_v * atol_v

        def refresh():
            Aop.matvec(x, b, r, -1.0, 1.0)
            if Mop is not None:
                Mop.matvec(r, z, z, 1.0, 0.0)
            Aop.matvec(z, Az, Az, 1.0, 0.0)
            return self._dots([(r, r), (z, Az)])

        rr, zAz = refresh()
        p, Ap = z.clone(), Az.clone()
        it = 0
        if self._callback is not None and self._check_every > 0:
            self._callback(0, math.sqrt(rr), atol_v)
        while not (rr <= atol_sq) and it < self._maxiter:
            zAz_old = zAz
            yv = Ap
            if Mop is not None:
                Mop.matvec(Ap, y, y, 1.0, 0.0)
                yv = y
            (yAp,) = self._dots([(Ap, yv)])
            alpha = zAz_old / yAp if (rr > atol_sq and yAp > 0.0) else 0.0
            self._axpby(alpha, p, 1.0, x, x)
            self._axpby(-alpha, Ap, 1.0, r, r)
            if Mop is not None:
                self._axpby(-alpha, y, 1.0, z, z)
            it += 1
            if self._restart is not None and it % self._restart == 0:
                rr, zAz = refresh()
                p.copy_(z)
                Ap.copy_(Az)
            else:
                Aop.matvec(z, Az, Az, 1.0, 0.0)
                rr, zAz = self._dots([(r, r), (z, Az)])
                beta = zAz / zAz_old if (rr > atol_sq and zAz_old > 0.0) else 0.0
                self._axpby(1.0, z, beta, p, p)
                self._axpby(1.0, Az, beta, Ap, Ap)
            if self._callback is not None and self._check_every > 0 and it % self._check_every == 0:
                self._callback(it, math.sqrt(rr), atol_v)
        return _generic_return(self, it, rr, atol_sq, b.device)


class GMRES(LinearSolverState):
    """Restarted GMRES(k) (reference: ``linear.py:1653-1916``, least squares ``:2497-2560``): each
    cycle runs k Arnoldi steps (one-pass classical Gram-Schmidt against the basis, library multi-dot
    / multi-axpy kernels), solves the small least-squares problem by Givens QR with the pivot
    tolerance eps^2 (on the host, float64), updates x, and tests the true residual
    ||b - A x|| <= max(rtol ||b||, atol).  Left or right preconditioning; the iteration count
    advances by k per cycle, as in the reference."""

    def __init__(self, A_, b, x, tol=None, atol=None, restart=31, maxiter=0, M=None, callback=None, check_every=31,
                 use_cuda_graph=True, is_left_preconditioner=False):
        self._restart = int(restart)
        self._is_left_preconditioner = bool(is_left_preconditioner)
        super().__init__(A_, b, x, tol, atol, maxiter, M, callback, check_every, use_cuda_graph)
        self._restart = max(1, min(self._restart, self._maxiter))
        if self._check_every > 0:
            self._check_every = max(self._restart, self._check_every)

    def _fused_eligible(self, Aop, Mop, b, x) -> bool:
        return False

    def _run_generic(self, Aop, b, x, Mop):
        L = N.lib()
        dt = b.dtype
        gdt = A.gb_dtype(dt)
        rtol, atol = _get_tolerances(dt, self._tol, self._atol)
        pivot = _dtype_epsilon(dt) ** 2
        k = self._restart
        n = b.numel()
        left = self._is_left_preconditioner and Mop is not None
        V = torch.zeros((k + 1, n), dtype=dt, device=b.device)
        r = torch.empty_like(b)
        w = torch.zeros_like(b)
        tmp = torch.zeros_like(b)
        h_dev = A.zeros(k + 1, torch.float64)
        ws = A.workspace(int(L.gb_multi_dot_workspace_bytes(k + 1)))
        stream = A.stream()
        (bb,) = self._dots([(b, b)])
        atol_v = max(rtol * math.sqrt(bb), atol)
        atol_sq = atol_v * atol_v
        Aop.matvec(x, b, r, -1.0, 1.0)
        (rr,) = self._dots([(r, r)])
        it = 0
        if self._callback is not None and self._check_every > 0:
            self._callback(0, math.sqrt(rr), atol_v)
        while not (rr <= atol_sq) and it < self._maxiter:
            rh = r
            if left:
                Mop.matvec(r, w, w, 1.0, 0.0)
                rh = w
            (beta2,) = self._dots([(rh, rh)])
            beta = math.sqrt(beta2)
            self._axpby(1.0 / beta if beta2 != 0.0 else 1.0, rh, 0.0, rh, V[0])
            H = np.zeros((k + 1, k))
            for j in range(k):
                if Mop is not None:
                    if left:
                        Aop.matvec(V[j], tmp, tmp, 1.0, 0.0)
                        Mop.matvec(tmp, w, w, 1.0, 0.0)
                    else:
                        Mop.matvec(V[j], tmp, tmp, 1.0, 0.0)
                        Aop.matvec(tmp, w, w, 1.0, 0.0)
                else:
                    Aop.matvec(V[j], w, w, 1.0, 0.0)
                N.check(L.gb_multi_dot(gdt, n, j + 1, A.ptr(V), n, A.ptr(w), A.ptr(h_dev), A.ptr(ws), ws.numel(),
                                       stream), "multi_dot")
                N.check(L.gb_multi_axpy(gdt, n, j + 1, A.ptr(V), n, A.ptr(h_dev), -1.0, 1.0, A.ptr(w), stream),
                        "multi_axpy")
                H[: j + 1, j] = h_dev[: j + 1].cpu().numpy()
                (hh,) = self._dots([(w, w)])
                H[j + 1, j] = math.sqrt(hh)
                self._axpby(1.0 / math.sqrt(hh) if hh != 0.0 else 1.0, w, 0.0, w, V[j + 1])
            y = _gmres_least_squares(H, beta, pivot)
            coef = A.from_numpy(np.concatenate([y, np.zeros(k + 1 - len(y))]).astype(np.float64))
            if Mop is None or left:
                N.check(L.gb_multi_axpy(gdt, n, k, A.ptr(V), n, A.ptr(coef), 1.0, 1.0, A.ptr(x), stream), "update x")
            else:
                N.check(L.gb_multi_axpy(gdt, n, k, A.ptr(V), n, A.ptr(coef), 1.0, 0.0, A.ptr(w), stream), "update w")
                Mop.matvec(w, tmp, tmp, 1.0, 0.0)
                self._axpby(1.0, tmp, 1.0, x, x)
            Aop.matvec(x, b, r, -1.0, 1.0)
            (rr,) = self._dots([(r, r)])
            it += k
            if self._callback is not None and self._check_every > 0 and it % self._check_every < k:
                self._callback(it, math.sqrt(rr), atol_v)
        return _generic_return(self, it, rr, atol_sq, b.device)


def _gmres_least_squares(H: np.ndarray, beta: float, pivot: float) -> np.ndarray:
    """min ||beta e1 - H y|| for the (k+1) x k Hessenberg H by Givens rotations; stops at the first
    rotation whose pivot norm^2 is below ``pivot`` (the Arnoldi process ended early)."""
    H = H.copy()
    k = H.shape[1]
    g = np.zeros(k + 1)
    rhs = beta
    kk = k
    for i in range(k):
        a, b_ = H[i, i], H[i + 1, i]
        n2 = a * a + b_ * b_
        if n2 < pivot:
            kk = i
            break
        nrm = math.sqrt(n2)
        c, s = a / nrm, b_ / nrm
        Hi, Hj = H[i, i:].copy(), H[i + 1, i:].copy()
        H[i, i:] = c * Hi + s * Hj
        H[i + 1, i:] = c * Hj - s * Hi
        g[i] = c * rhs
        rhs = -s * rhs
    y = np.zeros(kk)
    for i in range(kk - 1, -1, -1):
        y[i] = (g[i] - H[i, i + 1:kk] @ y[i + 1:kk]) / H[i, i]
    return y


class BiCGSTAB(LinearSolverState):
    """Pre-allocated BiCGSTAB solver (reference: ``linear.py:1377-1574``)."""

    _kind = N.KRYLOV_BICGSTAB

    def __init__(self, A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
                 use_cuda_graph=True, is_left_preconditioner=False):
        self._is_left_preconditioner = bool(is_left_preconditioner)
        super().__init__(A_, b, x, tol, atol, maxiter, M, callback, check_every, use_cuda_graph)

    def _run_batched(self, Aop, b, x, Mop):
        """Batched operator: one persistent launch, one CTA per subproblem running its BiCGSTAB to its
        own tolerance (reference: ``linear.py:1377-1574`` with ``batch_offsets``)."""
        from .. import batched

        if b.dtype != torch.float32 or x.dtype != torch.float32:
            raise NotImplementedError("batched BiCGSTAB: float32 systems")
        inv = None
        if Mop is not None:
            inv = getattr(Mop, "_inv_diag", None)
            if inv is None:
                raise NotImplementedError("batched BiCGSTAB: Jacobi ('diag') or no preconditioner")
        if getattr(self, "_batched", None) is None or self._batched_op is not Aop:
            csr = batched.as_block_csr(Aop)
            rtol, atol = _get_tolerances(torch.float32, self._tol, self._atol)
            self._batched = batched.BatchedBiCGSTAB(csr, Aop.batch_offsets, inv, rtol, atol, self._maxiter,
                                                    left_precond=self._is_left_preconditioner,
                                                    use_cuda_graph=self._use_cuda_graph)
            self._batched_op = Aop
        self._batched.inv_diag = inv
        self._batched.solve(b, x)
        it, rr, atol_sq = self._batched.results()
        if self._check_every == 0:
            return it, rr, atol_sq
        it_h = int(it.item())
        err = math.sqrt(float(rr.max())) if rr.numel() else 0.0
        atol_v = math.sqrt(float(atol_sq.max())) if atol_sq.numel() else 0.0
        if self._callback is not None:
            self._callback(it_h, err, atol_v)
        return it_h, err, atol_v

    def _run_generic(self, Aop, b, x, Mop):
        dt = b.dtype
        rtol, atol = _get_tolerances(dt, self._tol, self._atol)
        r = torch.empty_like(b)
        v = torch.zeros_like(b)
        t = torch.zeros_like(b)
        y = torch.zeros_like(b) if Mop is not None else None
        z = torch.zeros_like(b) if Mop is not None else None
        (bb,) = self._dots([(b, b)])
        atol_v = max(rtol * math.sqrt(bb), atol)
        atol_sq = atol_v * atol_v
        Aop.matvec(x, b, r, -1.0, 1.0)
        (rr,) = self._dots([(r, r)])
        p = r.clone()
        r0 = r.clone()
        rho = rr
        it = 0
        left = self._is_left_preconditioner
        while not (rr <= atol_sq) and it < self._maxiter:
            yv = p
            if Mop is not None:
                Mop.matvec(p, y, y, 1.0, 0.0)
                yv = y
            Aop.matvec(yv, v, v, 1.0, 0.0)
            (r0v,) = self._dots([(r0, v)])
            alpha = rho / r0v if (rr > atol_sq and r0v != 0.0) else 0.0
            self._axpby(alpha, yv, 1.0, x, x)
            self._axpby(-alpha, v, 1.0, r, r)
            (rr,) = self._dots([(r, r)])
            zv = r
            if Mop is not None:
                Mop.matvec(r, z, z, 1.0, 0.0)
                zv = z
            Aop.matvec(zv, t, t, 1.0, 0.0)
            if Mop is not None and left:
                Mt = torch.empty_like(t)
                Mop.matvec(t, Mt, Mt, 1.0, 0.0)
                st, tt = self._dots([(zv, Mt), (Mt, Mt)])
            else:
                st, tt = self._dots([(r, t), (t, t)])
            omega = st / tt if (rr > atol_sq and tt != 0.0) else 0.0
            self._axpby(omega, zv, 1.0, x, x)
            self._axpby(-omega, t, 1.0, r, r)
            rr, rho_new = self._dots([(r, r), (r0, r)])
            active = rr > atol_sq and r0v != 0.0 and st != 0.0
            beta = rho_new * tt / (r0v * st) if active else 0.0
            beta_omega = rho_new / r0v if active else 0.0
            # p = r + beta p - beta_omega v
            self._axpby(beta, p, -beta_omega, v, p)
            self._axpby(1.0, r, 1.0, p, p)
            rho = rho_new
            it += 1
            if self._callback is not None and self._check_every > 0 and it % self._check_every == 0:
                self._callback(it, math.sqrt(rr), atol_v)
        if self._check_every == 0:
            return (torch.tensor([it], dtype=torch.int32, device=b.device),
                    torch.tensor([rr], dtype=torch.float64, device=b.device),
                    torch.tensor([atol_sq], dtype=torch.float64, device=b.device))
        return it, math.sqrt(rr), atol_v


def _fine_stencil(M, Aop):
    """(dims, S) of a multigrid preconditioner's fine level when it is Aop's matrix in stencil form."""
    levels = getattr(M, "levels", None)
    bsr = getattr(Aop, "_bsr", None)
    if not levels or bsr is None:
        return None
    lv = levels[0]
    if getattr(lv, "S", None) is None or lv.A is not bsr or bsr.block_shape != (1, 1) or len(lv.dims) != 3:
        return None
    return lv.dims, lv.S


class FCG(LinearSolverState):
    """Flexible CG, FCG(1) (Notay's truncated variant): each new direction z = M(r) is
    A-orthogonalised against the previous direction only, so M may change from one application to
    the next (a nonlinear / learned preconditioner).  Same interface and return conventions as
    ``CG``; ``M`` is an object with ``launch(stream, r_ptr, z_ptr)`` that enqueues z = M(r) on the
    given stream (e.g. ``MultigridPreconditioner``).  A stagnation rule (every
    ``stagnation_window`` iterations the residual norm must drop by ``stagnation_factor``) or a
    non-descent direction (z.r <= 0) stops the loop with a status bit so that the caller can fall
    back to Jacobi-CG.  No reference counterpart (Warp has CG/CR/BiCGSTAB/GMRES only).
    """

    _kind = N.KRYLOV_FCG

    def __init__(self, A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
                 use_cuda_graph=True, stagnation_window: int = 25, stagnation_factor: float = 0.9,
                 stencil=None):
        """``stencil``: optional ``(dims, S)`` -- the 27-point stencil form (``gb_st27_build``, fp32) of the
        same 1x1 matrix on a node grid of ``dims``; the product of every iteration then reads it
        (120 B per node) instead of the CSR form.  ``stencil="auto"`` takes it from a
        ``MultigridPreconditioner`` M whose fine level is this matrix in stencil form."""
        if M is None or not hasattr(M, "launch"):
            raise ValueError("FCG needs a preconditioner object with launch(stream, r_ptr, z_ptr)")
        self._precond_obj = M
        self._stag = (int(stagnation_window), float(stagnation_factor))
        super().__init__(A_, b, x, tol, atol, maxiter, None, callback, check_every, use_cuda_graph)
        if not self._fused:
            raise ValueError("FCG needs a BSR operator with 1x1/3x3 fp32 blocks and fp32 vectors")
        self._M = None
        self._install_precond(M)
        if stencil == "auto":
            stencil = _fine_stencil(M, self._A)
        self.stencil_product = stencil is not None
        if stencil is not None:
            dims, S = stencil
            self._stencil_keep = S
            N.check(N.lib().gb_krylov_set_stencil(self._native, int(dims[0]), int(dims[1]), int(dims[2]), A.ptr(S)),
                    "krylov_set_stencil")

    def _install_precond(self, M):
        import traceback

        def _cb(user, stream, r, z):
            try:
                M.launch(stream, r, z)
                return 0
            except Exception:  # reported through the solver's status
                traceback.print_exc()
                return 1

        self._cb = N.PRECOND_FN(_cb)
        N.check(N.lib().gb_krylov_set_precond(self._native, ctypes.cast(self._cb, ctypes.c_void_p), None,
                                              self._stag[0], self._stag[1]), "krylov_set_precond")
        self._precond_obj = M

    def _run_generic(self, Aop, b, x, Mop):
        raise ValueError("FCG runs on the fused path only")


@A.on_caller_stream
def fcg(A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10, use_cuda_graph=True,
        run=True, stagnation_window: int = 25, stagnation_factor: float = 0.9):
    """Flexible CG with a (possibly nonlinear) preconditioner object; see ``FCG``."""
    state = FCG(A_, b, x, tol=tol, atol=atol, maxiter=maxiter, M=M, callback=callback, check_every=check_every,
                use_cuda_graph=use_cuda_graph, stagnation_window=stagnation_window,
                stagnation_factor=stagnation_factor)
    if run:
        return state()
    return state


@A.on_caller_stream
def cg(A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10, use_cuda_graph=True,
       run=True, *, restart=None):
    """Preconditioned Conjugate Gradient (reference: ``linear.py:1035-1121``)."""
    state = CG(A_, b, x, tol=tol, atol=atol, maxiter=maxiter, M=M, callback=callback, check_every=check_every,
               use_cuda_graph=use_cuda_graph, restart=restart)
    if run:
        return state()
    return state


@A.on_caller_stream
def cr(A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10, use_cuda_graph=True,
       run=True, *, restart=None):
    """Conjugate Residual (reference: ``linear.py:1288-1374``)."""
    state = CR(A_, b, x, tol=tol, atol=atol, maxiter=maxiter, M=M, callback=callback, check_every=check_every,
               use_cuda_graph=use_cuda_graph, restart=restart)
    if run:
        return state()
    return state


@A.on_caller_stream
def gmres(A_, b, x, tol=None, atol=None, restart=31, maxiter=0, M=None, callback=None, check_every=31,
          use_cuda_graph=True, is_left_preconditioner=False, run=True):
    """Restarted GMRES(k) (reference: ``linear.py:1918-2008``)."""
    state = GMRES(A_, b, x, tol=tol, atol=atol, restart=restart, maxiter=maxiter, M=M, callback=callback,
                  check_every=check_every, use_cuda_graph=use_cuda_graph, is_left_preconditioner=is_left_preconditioner)
    if run:
        return state()
    return state


@A.on_caller_stream
def bicgstab(A_, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10, use_cuda_graph=True,
             is_left_preconditioner=False, run=True):
    """BiCGSTAB (reference: ``linear.py:1577-1650``)."""
    state = BiCGSTAB(A_, b, x, tol=tol, atol=atol, maxiter=maxiter, M=M, callback=callback,
                     check_every=check_every, use_cuda_graph=use_cuda_graph,
                     is_left_preconditioner=is_left_preconditioner)
    if run:
        return state()
    return state


# -------------------------------------------------------------------------------------------
# FP64 iterative refinement around the fused FP32 Krylov solver
# -------------------------------------------------------------------------------------------
class _DivergenceGuard:
    """Decides when iterative refinement's corrections diverge, from the true residual norms.

    ``step(rnorm)`` after each correction returns "ok", "save" (the residual grew: the caller keeps
    the iterate before this correction), "undo" (stop; take this correction back) or "restore"
    (stop; go back to the iterate saved at the previous "save").  Stops on a non-finite residual, a
    residual over 100x the previous one or over 1e3 x max(||b||, initial residual), and on two
    corrections in a row that each made the residual grow.
    """

    def __init__(self, r0: float, bnorm: float):
        self.prev = r0
        self.cap = 1e3 * max(bnorm, r0)
        self.grew = False

    def step(self, rnorm: float) -> str:
        prev, self.prev = self.prev, rnorm
        bad = not math.isfinite(rnorm) or rnorm > 100.0 * prev or rnorm > self.cap
        if rnorm > prev or bad:
            if self.grew:
                return "restore"
            if bad:
                return "undo"
            self.grew = True
            return "save"
        self.grew = False
        return "ok"


class RefinedSolver:
    """Mixed-precision solve: FP32 Jacobi-PCG (or BiCGSTAB) inner loop inside iterative refinement.

    Each outer step computes the true residual r = b - A x from the high-precision solution
    (FP64 storage; product in double-float arithmetic, since GB300's FP64 rate is a small fraction
    of FP32 -- ``residual="fp64"`` selects FP64 arithmetic instead), solves A d = r in FP32 with
    the fused graph solver from d = 0, and updates x += d in FP64.  Convergence is tested on
    ||b - A x|| / ||b|| in FP64.  The inner tolerance adapts: the first step uses ``inner_tol``,
    later steps ask only for the reduction still missing (x 1/4 margin), never below
    ``inner_tol``.  Default ``inner_tol``: 1e-4 for the flexible solver (two corrections of 1e-4 reach
    1e-8: at 96^3 8 instead of 9 learned-FCG iterations, at 128^3 elasticity 59 instead of 64), 1e-5 for
    the Krylov drop-ins (with 1e-4 the 96^3 Jacobi-CG took a third outer step).  ``inner_values`` (e.g. a bfloat16 copy) replaces the matrix values in the
    inner loop only.  ``persistent``: the inner CG as one persistent cooperative launch (``CG``).
    ``stencil_product``: with a multigrid preconditioner whose fine level holds this matrix in 27-point
    stencil form, the true residual (and, with ``method="fcg"``, the flexible solver's product) reads
    the stencil form.
    """

    def __init__(self, Am: sparse.BsrMatrix, M: LinearOperator | None = None, method: str = "cg",
                 inner_tol: float | None = None, inner_maxiter: int = 0, inner_values: torch.Tensor | None = None,
                 residual: str = "df32", use_cuda_graph: bool = True, persistent: bool = True,
                 stencil_product: bool = True):
        self.A = Am
        self.M = M
        self.n = Am.nrow * Am.block_shape[0]
        if inner_tol is None:
            inner_tol = 1e-4 if method == "fcg" else 1e-5
        self.inner_tol = float(inner_tol)
        self.inner_maxiter = int(inner_maxiter) if inner_maxiter else self.n
        self.residual_mode = residual
        self._r32 = A.zeros(self.n, torch.float32)
        self._d = A.zeros(self.n, torch.float32)
        self._x2 = A.zeros(2 * self.n, torch.float32)
        self._inner_A = Am
        if inner_values is not None:
            self._inner_A = sparse.BsrMatrix(Am.nrow, Am.ncol, Am.block_shape, inner_values.dtype)
            self._inner_A.offsets, self._inner_A.columns = Am.offsets, Am.columns
            self._inner_A.values, self._inner_A.nnz = inner_values, Am.nnz
        self.method = method
        self.fallbacks = 0
        self._jacobi = None
        # graph mode: each correction solve is one conditional-loop graph launch; otherwise eager
        # launches with a host check after every iteration (for per-kernel profiling)
        loop = dict(check_every=0, use_cuda_graph=True) if use_cuda_graph else dict(check_every=1,
                                                                                   use_cuda_graph=False)
        if method == "fcg":
            self.inner = FCG(self._inner_A, self._r32, self._d, tol=self.inner_tol, atol=0.0,
                             maxiter=self.inner_maxiter, M=M, stencil="auto" if stencil_product else None, **loop)
            # Jacobi-CG: the fallback when the flexible solve stagnates
            self._jacobi_M = preconditioner(self._inner_A, "diag")
            self._jacobi = CG(self._inner_A, self._r32, self._d, tol=self.inner_tol, atol=0.0,
                              maxiter=self.inner_maxiter, M=self._jacobi_M, persistent=persistent, **loop)
        elif method == "cg":
            self.inner = CG(self._inner_A, self._r32, self._d, tol=self.inner_tol, atol=0.0,
                            maxiter=self.inner_maxiter, M=M, persistent=persistent, **loop)
        else:
            self.inner = BiCGSTAB(self._inner_A, self._r32, self._d, tol=self.inner_tol, atol=0.0,
                                  maxiter=self.inner_maxiter, M=M, **loop)
        if not self.inner._fused:
            raise ValueError("solve_refined needs a BSR operator with 1x1/3x3 float32 blocks and a Jacobi or no "
                             "preconditioner")
        L = N.lib()
        nnz = Am.nnz_sync()
        self._res_ws = A.zeros(int(L.gb_residual_f64_workspace_bytes(Am.block_shape[0], Am.nrow, nnz,
                                                                      A.gb_dtype(Am.values.dtype))), torch.uint8)
        self._norms = A.zeros(2, torch.float64)
        self._dots_ws = A.zeros(int(L.gb_dots_workspace_bytes()), torch.uint8)  # arrival counter starts at 0
        self._status = A.zeros(1, torch.int32)
        self._host = torch.zeros(2, dtype=torch.float64, pin_memory=True)
        self._step_host = torch.zeros(2, dtype=torch.int32, pin_memory=True)
        self._host0 = torch.zeros(2, dtype=torch.float64, pin_memory=True)
        self._x_backup = None
        self.kernel_launches = 0
        # the true residual on the multigrid fine level's stencil form of the same matrix, when it has one
        self._res_stencil = (_fine_stencil(M, aslinearoperator(Am)) if stencil_product and residual == "df32"
                             else None)

    def residual(self, x64: torch.Tensor, b: torch.Tensor, sync: bool = True):
        """True residual (written as the fp32 right-hand side of the next correction solve)."""
        Am = self.A
        L = N.lib()
        if self.residual_mode == "fp64":
            N.check(L.gb_residual_f64(Am.block_shape[0], Am.nrow, Am.nnz, Am.capacity, A.ptr(Am.offsets), None,
                                      A.ptr(Am.columns), A.ptr(Am.values), A.gb_dtype(Am.values.dtype), A.ptr(x64),
                                      A.ptr(b), None, A.ptr(self._r32), A.ptr(self._norms), self._res_ws.data_ptr(),
                                      self._res_ws.numel(), A.ptr(self._status), A.stream()), "residual_f64")
        elif self._res_stencil is not None:
            dims, S = self._res_stencil
            N.check(L.gb_residual_df_st27(*dims, A.ptr(S), A.ptr(self._x2), A.ptr(b), None, A.ptr(self._r32),
                                          A.ptr(self._norms), self._res_ws.data_ptr(), self._res_ws.numel(),
                                          A.ptr(self._status), A.stream()), "residual_df_st27")
        else:
            N.check(L.gb_residual_df(Am.block_shape[0], Am.nrow, Am.nnz, Am.capacity, A.ptr(Am.offsets), None,
                                     A.ptr(Am.columns), A.ptr(Am.values), A.gb_dtype(Am.values.dtype),
                                     A.ptr(self._x2), A.ptr(b), None, A.ptr(self._r32), A.ptr(self._norms),
                                     self._res_ws.data_ptr(), self._res_ws.numel(), A.ptr(self._status), A.stream()),
                    "residual_df")
        self.kernel_launches += 1
        if not sync:
            return None
        self._host.copy_(self._norms, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        rr, bb = self._host.tolist()
        return math.sqrt(rr), math.sqrt(bb)

    @A.on_caller_stream
    def solve(self, b, x64=None, tol: float = 1e-8, max_outer: int = 50, callback=None):
        b = A.as_tensor(b).reshape(-1)
        if b.dtype != torch.float32:
            raise TypeError("right-hand side must be float32 (the system's scalar type)")
        if b.numel() != self.n:
            raise ValueError(f"Incompatible b.shape: expected ({self.n},), got {tuple(b.shape)}")
        L = N.lib()
        history = []
        inner_iters = 0
        outer = 0
        Aop = self.inner._A
        diverged = False
        rhs = self._r32
        if x64 is None:
            # x = 0: the residual is b itself, so the first correction solve takes b as its right-hand
            # side and needs no product and no host read first; only (b.b, b.b) is queued, and the
            # initial norms come back with the first step's
            x64 = A.zeros(self.n, torch.float64)
            self._x2.zero_()
            xs = (ctypes.c_void_p * 2)(A.ptr(b), A.ptr(b))
            N.check(L.gb_dots(N.GB_F32, self.n, 2, xs, xs, A.ptr(self._norms), A.ptr(self._dots_ws), A.stream()),
                    "initial_norms")
            self.kernel_launches += 1
            self._host0.copy_(self._norms, non_blocking=True)
            rhs = b
            rnorm = bnorm = None
            guard = None
        else:
            x64 = A.as_tensor(x64).reshape(-1)
            N.check(L.gb_update_solution(self.n, A.ptr(x64), A.ptr(self._x2), None, 0.0, A.stream()), "update")
            self.kernel_launches += 1
            rnorm, bnorm = self.residual(x64, b)
            history.append(rnorm / bnorm if bnorm > 0 else 0.0)
            guard = _DivergenceGuard(rnorm, bnorm)
        while (bnorm is None or (bnorm > 0 and rnorm > tol * bnorm)) and outer < max_outer:
            # ask the correction solve only for the reduction still missing (never below inner_tol)
            need = 0.25 * tol * (1.0 if bnorm is None else bnorm / rnorm)
            self.inner._tol = min(max(self.inner_tol, need), 0.5)
            self._d.zero_()
            self.inner._run_fused(Aop, rhs, self._d, self.inner._M, x_is_zero=True)
            rhs = self._r32  # the residual queued below is the next step's right-hand side
            # queue x += d and the new residual behind the correction solve, and read its iteration
            # count and status together with the residual norms (one host synchronisation per step)
            self._step_host[0:1].copy_(self.inner._dev_iter.reshape(1), non_blocking=True)
            self._step_host[1:2].copy_(self.inner._dev_status.reshape(1), non_blocking=True)
            N.check(L.gb_update_solution(self.n, A.ptr(x64), A.ptr(self._x2), A.ptr(self._d), 1.0, A.stream()),
                    "update_solution")
            self.kernel_launches += 1
            self.residual(x64, b, sync=False)
            self._host.copy_(self._norms, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            it, status = (int(v) for v in self._step_host.tolist())
            if bnorm is None:
                r0, bnorm = (math.sqrt(v) for v in self._host0.tolist())
                history.append(r0 / bnorm if bnorm > 0 else 0.0)
                guard = _DivergenceGuard(r0, bnorm)
                if bnorm == 0:  # b = 0: x = 0 is the solution (the correction solve had nothing to do)
                    x64.zero_()
                    self._x2.zero_()
                    rnorm = 0.0
                    break
            rnorm = math.sqrt(float(self._host[0]))
            if self.inner.persistent_active:
                # argument store, init and the persistent loop (one launch per host-checked chunk)
                self.kernel_launches += 3 if self.inner._check_every == 0 else 2 + it
            else:
                per_it = 3 if self.method != "fcg" else ((2 if self.inner.stencil_product else 4) +
                                                         getattr(self.inner._precond_obj, "kernels_per_apply", 0))
                self.kernel_launches += 2 + per_it * it  # argument store, init, kernels per iteration
            if self.method == "fcg" and status & (N.DEV_STAGNATION | N.DEV_BREAKDOWN | N.DEV_NONFINITE):
                # the flexible solve stalled: take its correction back, recompute the residual it was
                # solving for (the queued residual overwrote it) and finish the correction with plain
                # Jacobi-CG, starting from the flexible solve's d
                N.check(L.gb_update_solution(self.n, A.ptr(x64), A.ptr(self._x2), A.ptr(self._d), -1.0, A.stream()),
                        "undo_solution")
                self.residual(x64, b, sync=False)
                self.fallbacks += 1
                self._jacobi._tol = self.inner._tol
                self._jacobi._run_fused(Aop, self._r32, self._d, self._jacobi_M, x_is_zero=False)
                jt = int(self._jacobi._dev_iter.item())
                it += jt
                if self._jacobi.persistent_active:
                    self.kernel_launches += 3 if self._jacobi._check_every == 0 else 2 + jt
                else:
                    self.kernel_launches += 2 + 3 * jt
                N.check(L.gb_update_solution(self.n, A.ptr(x64), A.ptr(self._x2), A.ptr(self._d), 1.0, A.stream()),
                        "update_solution")
                self.kernel_launches += 2
                rnorm, _ = self.residual(x64, b)
            inner_iters += it
            outer += 1
            history.append(rnorm / bnorm)
            if callback is not None:
                callback(outer, it, rnorm / bnorm)
            verdict = guard.step(rnorm)
            if verdict == "save":
                # this correction made the residual grow: keep the iterate before it, in case the
                # next one grows too
                if self._x_backup is None:
                    self._x_backup = torch.empty_like(x64)
                torch.sub(x64, self._d.to(torch.float64), out=self._x_backup)
            elif verdict in ("undo", "restore"):
                # the corrections diverge (e.g. reduced-precision inner values far from the true
                # operator): return the last accepted iterate, not the one the bad correction made
                if verdict == "undo":
                    N.check(L.gb_update_solution(self.n, A.ptr(x64), A.ptr(self._x2), A.ptr(self._d), -1.0,
                                                 A.stream()), "undo_solution")
                else:
                    x64.copy_(self._x_backup)
                    N.check(L.gb_update_solution(self.n, A.ptr(x64), A.ptr(self._x2), None, 0.0, A.stream()),
                            "restore_solution")
                rnorm, _ = self.residual(x64, b)
                history.append(rnorm / bnorm)
                diverged = True
                break
            if it == 0:
                break
        if bnorm is None:  # max_outer = 0: only the initial residual was queued
            torch.cuda.current_stream().synchronize()
            rnorm, bnorm = (math.sqrt(v) for v in self._host0.tolist())
            history.append(rnorm / bnorm if bnorm > 0 else 0.0)
        return x64, dict(outer=outer, inner_iterations=inner_iters, rel_residual=history[-1], history=history,
                         converged=bool(rnorm <= tol * bnorm), diverged=diverged)


@A.on_caller_stream
def solve_refined(A_: sparse.BsrMatrix, b, x64=None, tol: float = 1e-8, M=None, method: str = "cg",
                  inner_tol: float | None = None, max_outer: int = 50, residual: str = "df32"):
    """FP64-accurate solve of ``A x = b`` with an FP32 Krylov inner loop; returns ``(x64, info)``.

    method: "cg" / "bicgstab" (M = Jacobi or None) or "fcg" (M = a preconditioner object)."""
    solver = RefinedSolver(A_, M=M, method=method, inner_tol=inner_tol, residual=residual)
    return solver.solve(b, x64=x64, tol=tol, max_outer=max_outer)
