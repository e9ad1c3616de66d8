"""Geometric multigrid V-cycle on Q1 grids: the global part of the flexible-CG preconditioner.

Warp's solvers offer only the Jacobi preconditioner (``warp/_src/optim/linear.py:236-329``); the
learned preconditioner of this package needs a carrier with global reach, since a 4-layer
3x3x3 convolution only sees 9 nodes.  This module provides it:

* hierarchy: vertex-centred 2:1 coarsening of the node grid (fine node 2I = coarse node I), per-cell
  coefficient coarsened by geometric mean (``gb_mg_coarsen_cells``), coarse operators
  rediscretised with the same Q1 assembly kernels and Dirichlet projection as the fine one;
* transfers: trilinear prolongation P and full weighting R = P^T (``gb_mg_prolong_add`` /
  ``gb_mg_restrict``), matrix-free, Dirichlet nodes masked;
* smoothing: damped Jacobi, the post-smoothing step fused with its residual product
  (``gb_bsr_jacobi_smooth``); the coarsest level (<= ``coarsest_nodes`` nodes) is solved with a
  dense inverse computed once at set-up;
* level operators in 27-point stencil form (``gb_st27_build``: 27 coefficient planes instead of CSR
  columns and offsets, about half the bytes per pass, staged by bulk copies), the first Jacobi step fused
  with the residual
  and the post-smoothing step fused with its residual (``gb_st27_apply``); a level whose CSR has
  entries outside the 27-neighbourhood keeps the CSR kernels;
* an optional learned fine-level smoother (``warp_gb300.learned``) replaces the first Jacobi step.

Every launch goes to the stream the caller passes, so the flexible solver can capture a whole
V-cycle into its CUDA graph.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _arrays as A
from . import _native as N
from . import fem, sparse


class _Level:
    pass


def _coarse_inverse(Am: sparse.BsrMatrix) -> np.ndarray:
    """float32 inverse of the coarsest level's matrix, computed in float64 on the host (set-up only)."""
    nnz = Am.nnz_sync()
    off = A.to_numpy(Am.offsets).astype(np.int64)
    cols = A.to_numpy(Am.columns[:nnz]).astype(np.int64)
    br, bc = Am.block_shape
    vals = A.to_numpy(Am.values[:nnz]).reshape(-1, br, bc).astype(np.float64)
    D = np.zeros((Am.nrow * br, Am.ncol * bc), np.float64)
    rows = np.repeat(np.arange(Am.nrow, dtype=np.int64), np.diff(off[: Am.nrow + 1]))
    ri = (rows[:, None, None] * br + np.arange(br)[None, :, None]).repeat(bc, axis=2).reshape(-1)
    ci = (cols[:, None, None] * bc + np.arange(bc)[None, None, :]).repeat(br, axis=1).reshape(-1)
    v = vals.reshape(-1)
    D[ri, ci] = v  # compact BSR: each (row, column) block once
    # symmetric to rounding: every stored entry matches its transposed position
    symmetric = D.shape[0] == D.shape[1] and (v.size == 0 or
                                              float(np.abs(D[ci, ri] - v).max()) <= 1e-12 * float(np.abs(v).max()))
    return _dense_inverse(D, symmetric).astype(np.float32)


def _dense_inverse(a: np.ndarray, symmetric: bool) -> np.ndarray:
    """Inverse of a dense float64 matrix: from its Cholesky factor when it is symmetric positive definite
    (half the work of an LU inverse; only the upper triangle is read), else by LU."""
    if symmetric and a.size:
        try:
            from scipy.linalg import lapack
        except ImportError:
            lapack = None
        if lapack is not None:
            c, info = lapack.dpotrf(a, lower=0, clean=1)
            if info == 0:
                inv, info = lapack.dpotri(c, lower=0, overwrite_c=1)
                if info == 0:
                    inv = np.triu(inv)
                    inv += np.triu(inv, 1).T  # dpotri fills the upper triangle
                    return inv
    return np.linalg.inv(a)


class MultigridPreconditioner:
    """z = V(r): symmetric V(1,1)-cycle (damped Jacobi, exact coarsest solve).

    Args:
        A: the fine system (compact BSR fp32, Dirichlet rows already projected): 1x1 blocks (diffusion) or
            3x3 blocks (Q1 vec3 linear elasticity).
        geo: the fem.Grid3D / Grid2D it was assembled on.
        coef: per-cell diffusion coefficient (1x1), or per-cell Young's modulus (3x3; the Lame parameters
            of every level follow from it and ``poisson``); host array or device tensor.
        faces: Dirichlet faces (default: the whole boundary).
        omega: Jacobi damping: a number for every level, or "auto" (the default) for 4 / (3 rho_l) per level
            with rho_l = rho(D^-1 A_l) estimated by power iteration at set-up (about 0.91 on the 96^3
            lognormal diffusion levels: 10 flexible-CG iterations there against 13 with a fixed 0.6; on Q1
            elasticity a fixed 0.6 amplifies the high-frequency error it should damp).  A learned smoother
            attached to the hierarchy sets the damping its network was trained with.
        coarsest_nodes: stop coarsening at or below this many nodes; that level is solved exactly with a
            dense inverse (computed on the host at set-up).  Default: at most 2200 unknowns -- 2200 nodes
            for 1x1 hierarchies (13^3 at 96^3), 733 for 3x3 (9^3 at 128^3): a 19 MB dense product per
            cycle and ~60 ms of set-up, which cut the flexible-CG iterations at 96^3 from 15 to 13 (12 to
            9 with the learned smoother) and at 128^3 elasticity from 90 to 78 against coarsest grids of
            7^3 / 5^3 nodes.  Pass 400 for the cheaper set-up when a hierarchy serves a single solve.
        stencil: apply the level operators in 27-point stencil form (else the CSR kernels; 1x1 only).
        poisson: Poisson ratio of the elasticity levels (3x3).
        fine_values: scalar type of the fine level's matrix values inside the V-cycle:
            ``torch.bfloat16`` keeps a bf16 copy (of the CSR values, or of the 27-point stencil
            coefficients) for the cycle's residual and smoothing passes, about half their matrix
            traffic, with fp32 accumulation; the flexible solver's own product keeps the fp32 matrix,
            so its tolerance and the FP64 refinement are unaffected (the cycle only has to be a good
            approximate inverse).
        block_jacobi: 3x3 hierarchies smooth with the inverses of the node blocks (block Jacobi; damping
            from rho(Db^-1 A)) instead of the diagonal entries: 77 -> 64 flexible-CG iterations on the 128^3
            elasticity configuration.

    Vectors of a 3x3 hierarchy hold 3 interleaved components per node; masks are per node.
    """

    def __init__(self, Am: sparse.BsrMatrix, geo, coef, faces=("x-", "x+", "y-", "y+", "z-", "z+"), omega=None,
                 coarsest_nodes: int | None = None, max_levels: int = 12, stencil: bool = True, poisson: float = 0.3,
                 fine_values: torch.dtype = torch.float32, block_jacobi: bool = True):
        if fine_values not in (torch.float32, torch.bfloat16):
            raise ValueError("fine_values: torch.float32 or torch.bfloat16")
        if Am.block_shape not in ((1, 1), (3, 3)) or Am.scalar_type != torch.float32:
            raise ValueError("multigrid preconditioner: fp32 BSR matrix with 1x1 or 3x3 blocks required")
        self.bdim = Am.block_shape[0]
        self.block_jacobi = bool(block_jacobi) and self.bdim == 3
        if coarsest_nodes is None:
            coarsest_nodes = 2200 // self.bdim
        if self.bdim == 3 and geo.dimension != 3:
            raise ValueError("multigrid preconditioner: 3x3 blocks need a Grid3D (vec3 elasticity)")
        self.poisson = float(poisson)
        if omega is None:
            omega = "auto"
        self.omega = omega if omega == "auto" else float(omega)
        self.faces = tuple(faces)
        self.smoother = None  # learned fine-level smoother (set by warp_gb300.learned)
        self.status = A.zeros(1, torch.int32)
        L = N.lib()
        stream = A.stream()
        levels = []
        coef_t = coef if isinstance(coef, torch.Tensor) else A.from_numpy(np.asarray(coef, np.float32).reshape(-1))
        coef_t = coef_t.reshape(-1).to(torch.float32).contiguous()
        cur_geo, cur_A, cur_coef = geo, Am, coef_t
        while True:
            lv = _Level()
            lv.geo = cur_geo
            lv.A = cur_A
            lv.nnz = cur_A.nnz_sync()
            lv.dims = tuple(r + 1 for r in cur_geo.res) + ((1,) if cur_geo.dimension == 2 else ())
            lv.n = cur_A.nrow
            lv.mask = A.empty(lv.n, torch.float32)
            nx, ny, nz = cur_geo._dims()
            bits = fem.BoundarySides(cur_geo, self.faces).face_bits()
            N.check(L.gb_grid_boundary_mask(cur_geo.dimension, nx, ny, nz, bits, 1, 1, A.ptr(lv.mask), stream), "mask")
            C = self.bdim
            lv.dinv = A.empty(lv.n * C, torch.float32)
            N.check(L.gb_bsr_inverse_diagonal(N.GB_F32, C, lv.n, A.ptr(cur_A.offsets), None, A.ptr(cur_A.columns),
                                              A.ptr(cur_A.values), 0, A.ptr(lv.dinv), stream), "dinv")
            lv.w = A.zeros(lv.n * C, torch.float32)
            lv.t = A.zeros(lv.n * C, torch.float32)
            # the values the cycle's CSR passes read (a bf16 copy on the fine level when asked)
            lv.vals = cur_A.values
            lv.vals_dtype = N.GB_F32
            if not levels and fine_values == torch.bfloat16:
                lv.vals = cur_A.values[: lv.nnz].to(torch.bfloat16).contiguous()
                lv.vals_dtype = N.GB_BF16
            levels.append(lv)
            res = cur_geo.res
            if lv.n <= coarsest_nodes or any(r % 2 for r in res) or len(levels) >= max_levels:
                break
            cres = tuple(r // 2 for r in res)
            ccoef = A.empty(int(np.prod(cres)), torch.float32)
            fx, fy, fz = (res[0], res[1], res[2]) if cur_geo.dimension == 3 else (res[0], res[1], 2)
            if cur_geo.dimension == 2:
                raise NotImplementedError("2-D hierarchy: use Grid3D problems")
            N.check(L.gb_mg_coarsen_cells(fx, fy, fz, A.ptr(cur_coef), A.ptr(ccoef), stream), "coarsen")
            cgeo = fem.Grid3D(res=cres, bounds_lo=cur_geo.bounds_lo, bounds_hi=cur_geo.bounds_hi)
            if self.bdim == 1:
                space = fem.make_polynomial_space(cgeo, degree=1)
                cA = fem.integrate(fem.diffusion_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                                   values={"nu": ccoef})
            else:
                space = fem.make_polynomial_space(cgeo, degree=1, dtype="vec3")
                nu = self.poisson
                lam = (ccoef * (nu / ((1.0 + nu) * (1.0 - 2.0 * nu)))).contiguous()
                mu = (ccoef * (1.0 / (2.0 * (1.0 + nu)))).contiguous()
                cA = fem.integrate(fem.linear_elasticity_form,
                                   fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                                   values={"lame": (lam, mu)})
            rhs = A.zeros(cgeo.node_count() * self.bdim, torch.float32)
            bd = fem.BoundarySides(cgeo, self.faces)
            P = fem.integrate(fem.boundary_projector_form,
                              fields={"u": fem.make_trial(space, bd), "v": fem.make_test(space, bd)}, assembly="nodal")
            fem.project_linear_system(cA, rhs, P)
            cur_geo, cur_A, cur_coef = cgeo, cA, ccoef
        # 3x3 levels: inverses of the node blocks for the block-Jacobi smoother
        for lv in levels:
            lv.dinvb = None
            if self.block_jacobi:
                lv.dinvb = A.empty(lv.n * 9, torch.float32)
                N.check(L.gb_bsr_block_inverse_diagonal3(lv.n, A.ptr(lv.A.offsets), None, A.ptr(lv.A.columns),
                                                         A.ptr(lv.A.values), A.ptr(lv.dinvb), stream), "block_inverse")
        # damping per level
        for lv in levels:
            lv.omega = self._auto_omega(lv) if self.omega == "auto" else self.omega
        # stencil planes of every level above the coarsest
        st_status = A.zeros(len(levels), torch.int32)
        for li, lv in enumerate(levels):
            lv.S = None
            if stencil and self.bdim == 1 and li < len(levels) - 1:
                lv.S = A.empty(int(L.gb_st27_bytes(*lv.dims)) // 4, torch.float32)
                N.check(L.gb_st27_build(*lv.dims, A.ptr(lv.A.offsets), A.ptr(lv.A.columns), A.ptr(lv.A.values),
                                        A.ptr(lv.S), st_status[li:].data_ptr(), stream), "st27_build")
        for li, bad in enumerate(st_status.tolist()):
            if bad:
                levels[li].S = None  # entries outside the 27-neighbourhood: keep the CSR kernels
        for li, lv in enumerate(levels):
            lv.Sb = None
            if li == 0 and lv.S is not None and fine_values == torch.bfloat16:
                lv.Sb = A.empty(int(L.gb_st27_bytes_bf16(*lv.dims)) // 2, torch.bfloat16)
                N.check(L.gb_st27_to_bf16(*lv.dims, A.ptr(lv.S), A.ptr(lv.Sb), stream), "st27_to_bf16")
        # coarsest level: dense inverse (set-up only; at most a few thousand unknowns)
        last = levels[-1]
        last.inv = A.from_numpy(_coarse_inverse(last.A))
        for lv in levels[1:]:  # right-hand side / correction buffers of the coarse levels
            lv.rhs = A.zeros(lv.n * self.bdim, torch.float32)
            lv.sol = A.zeros(lv.n * self.bdim, torch.float32)
        self.levels = levels
        torch.cuda.current_stream().synchronize()

    def _auto_omega(self, lv, iters: int = 30) -> float:
        """4 / (3 rho(D^-1 A)) with rho from power iteration on the level (set-up only).  Runs on the
        library's own kernels (SpMV, dot products, axpby), so the set-up launches no torch reduction
        (those are compiled for this GPU on first use, which took seconds on a fresh process)."""
        L = N.lib()
        stream = A.stream()
        m = lv.n * self.bdim
        rng = np.random.default_rng(7)
        x = A.from_numpy((rng.random(m) + 0.5).astype(np.float32))
        y = A.empty(m, torch.float32)
        z = A.empty(m, torch.float32)
        ws = A.zeros(int(L.gb_dots_workspace_bytes()), torch.uint8)
        out = A.zeros(4, torch.float64)
        host = torch.zeros(4, dtype=torch.float64, pin_memory=True)

        def norms(*vs) -> list[float]:
            ptrs = (ctypes.c_void_p * 4)(*[v.data_ptr() for v in vs])
            N.check(L.gb_dots(N.GB_F32, m, len(vs), ptrs, ptrs, out.data_ptr(), ws.data_ptr(), stream), "dots")
            host[: len(vs)].copy_(out[: len(vs)], non_blocking=True)
            torch.cuda.current_stream().synchronize()
            return [float(v) ** 0.5 for v in host[: len(vs)].tolist()]

        # a <- D^-1 A b with b = a, rescaled to unit norm every 8 steps (8 steps grow it by rho^8, far inside
        # fp32 range for these operators, rho ~ 2-5); three buffers so that no kernel reads and writes the
        # same vector; rho = |a| / |b| at the last step.  5 host reads per level.
        a, b, c = x, y, z
        nrm = norms(a)[0]
        rho = 1.0
        for it in range(iters):
            scale = 1.0 / max(nrm, 1e-30) if it % 8 == 0 else 1.0
            N.check(L.gb_axpby(N.GB_F32, m, scale, a.data_ptr(), 0.0, a.data_ptr(), b.data_ptr(), stream), "scale")
            sparse.bsr_mv(lv.A, b, c)
            if lv.dinvb is not None:
                N.check(L.gb_mg_block_jacobi0(lv.n, 1.0, lv.dinvb.data_ptr(), c.data_ptr(), a.data_ptr(), stream),
                        "dinv")
            else:
                N.check(L.gb_diag_mv(N.GB_F32, m, lv.dinv.data_ptr(), c.data_ptr(), None, a.data_ptr(), 1.0, 0.0,
                                     stream), "dinv")
            if it == iters - 1:
                na, nb = norms(a, b)
                rho = na / max(nb, 1e-30)
            elif (it + 1) % 8 == 0:
                nrm = norms(a)[0]
        return 4.0 / (3.0 * max(rho, 1e-30))

    @property
    def n(self) -> int:
        """Length of the vectors the preconditioner maps (nodes x components of the fine level)."""
        return self.levels[0].n * self.bdim

    @property
    def kernels_per_apply(self) -> int:
        """Kernel launches of one V-cycle: per level above the coarsest, the first smoothing step,
        residual, restriction, prolongation and post-smoothing (stencil form: the first two fused),
        plus the coarse solve."""
        count = 1
        for li, lv in enumerate(self.levels[:-1]):
            if li == 0 and self.smoother is not None:
                count += getattr(self.smoother, "kernels_per_apply", 1) + 4
            else:
                count += 4 if lv.S is not None else 5
        return count

    def describe(self) -> str:
        return " -> ".join(f"{'x'.join(str(d) for d in lv.dims)}" for lv in self.levels)

    # z = M r on `stream` (device pointers r, z of the fine level)
    def launch(self, stream, r_ptr: int, z_ptr: int) -> None:
        self._vcycle(0, int(r_ptr), int(z_ptr), stream)

    def _vcycle(self, li: int, r: int, z: int, stream) -> None:
        L = N.lib()
        lv = self.levels[li]
        if li == len(self.levels) - 1:
            m = lv.n * self.bdim
            N.check(L.gb_dense_mv(N.GB_F32, m, m, A.ptr(lv.inv), r, None, z, 1.0, 0.0, stream), "coarse")
            return
        nxt = self.levels[li + 1]
        w, t = A.ptr(lv.w), A.ptr(lv.t)
        Am = lv.A
        # pre-smoothing from zero (learned step on the fine level when available, else Jacobi) and
        # the residual t = r - A w
        if li == 0 and self.smoother is not None:
            self.smoother.launch(stream, r, w)
            if lv.S is not None:
                self._st27(lv, 0, w, r, None, None, t, stream)  # residual
            else:
                self._csr_residual(lv, w, r, t, stream)
        elif lv.S is not None:
            self._st27(lv, 1, None, r, A.ptr(lv.dinv), w, t, stream)  # first Jacobi step + residual
        elif lv.dinvb is not None:
            N.check(L.gb_mg_block_jacobi0(lv.n, lv.omega, A.ptr(lv.dinvb), r, w, stream), "block_jacobi0")
            self._csr_residual(lv, w, r, t, stream)
        else:
            N.check(L.gb_mg_jacobi0(lv.n * self.bdim, lv.omega, A.ptr(lv.dinv), r, w, stream), "jacobi0")
            self._csr_residual(lv, w, r, t, stream)
        fx, fy, fz = lv.dims
        cx, cy, cz = nxt.dims
        rc, zc = A.ptr(nxt.rhs), A.ptr(nxt.sol)  # the coarse level's own w/t are its work vectors
        N.check(L.gb_mg_restrict_c(self.bdim, fx, fy, fz, cx, cy, cz, t, A.ptr(lv.mask), A.ptr(nxt.mask), rc, stream),
                "restrict")
        self._vcycle(li + 1, rc, zc, stream)
        N.check(L.gb_mg_prolong_add_c(self.bdim, fx, fy, fz, cx, cy, cz, zc, A.ptr(lv.mask), 1.0, w, stream),
                "prolong")
        # post-smoothing fused with its residual: z = w + omega D^-1 (r - A w)
        if lv.S is not None:
            self._st27(lv, 2, w, r, A.ptr(lv.dinv), None, z, stream)  # smoothing step + residual
        elif lv.dinvb is not None:
            N.check(L.gb_bsr_block_jacobi_smooth3(lv.n, lv.nnz, lv.nnz, A.ptr(Am.offsets), A.ptr(Am.columns),
                                                  A.ptr(lv.vals), lv.vals_dtype, r, w, A.ptr(lv.dinvb), lv.omega, z,
                                                  A.ptr(self.status), stream), "block_smooth")
        else:
            N.check(L.gb_bsr_jacobi_smooth(self.bdim, lv.n, lv.nnz, lv.nnz, A.ptr(Am.offsets), A.ptr(Am.columns),
                                           A.ptr(lv.vals), lv.vals_dtype, r, w, A.ptr(lv.dinv), lv.omega, z,
                                           A.ptr(self.status), stream), "smooth")

    def _st27(self, lv, mode: int, w, r: int, dinv, w_out, out: int, stream) -> None:
        """One stencil pass of level lv (fp32 coefficients, or their bf16 copy on the fine level)."""
        L = N.lib()
        if lv.Sb is not None:
            N.check(L.gb_st27_apply_bf16(mode, *lv.dims, A.ptr(lv.Sb), w, r, dinv, lv.omega, w_out, out,
                                         A.ptr(self.status), stream), "st27_apply_bf16")
        else:
            N.check(L.gb_st27_apply(mode, *lv.dims, A.ptr(lv.S), w, r, dinv, lv.omega, w_out, out, A.ptr(self.status),
                                    stream), "st27_apply")

    def _csr_residual(self, lv, w: int, r: int, t: int, stream) -> None:
        Am = lv.A
        C = self.bdim
        N.check(N.lib().gb_bsr_mv(C, C, lv.n, lv.n, lv.nnz, lv.nnz, A.ptr(Am.offsets), None, A.ptr(Am.columns),
                                  A.ptr(lv.vals), lv.vals_dtype, w, r, t, N.GB_F32, -1.0, 1.0, 0, 0, 0, -1,
                                  A.ptr(self.status), stream), "residual")

    @A.on_caller_stream
    def apply(self, r: torch.Tensor, z: torch.Tensor | None = None) -> torch.Tensor:
        """Eager z = M r on the current stream (tests / diagnostics)."""
        z = torch.empty_like(r) if z is None else z
        self.launch(A.stream(), r.data_ptr(), z.data_ptr())
        return z
