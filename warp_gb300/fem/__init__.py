"""Q1 finite elements on regular grids: the drop-in for the ``warp.fem`` calls of the solve path.

Covers what the FEM linear-solve path uses from ``warp.fem`` (``warp/fem/__init__.py``):
``Grid2D`` / ``Grid3D`` (``warp/_src/fem/geometry/grid_2d.py``, ``grid_3d.py``),
``make_polynomial_space`` (degree 1, scalar or vec3), ``make_test`` / ``make_trial``, ``Cells``
/ ``BoundarySides`` domains, ``integrate`` (``warp/_src/fem/integrate.py:1895``) for the
diffusion, linear-elasticity, mass, linear (source) and boundary-projector forms, and
``project_linear_system`` (``warp/_src/fem/dirichlet.py:107-124``).

Warp compiles arbitrary Python integrands; this package has hand-written kernels for the forms
above instead, recognised by the integrand objects exported here.  ``integrate`` raises for any
other integrand.  Bilinear assembly writes COO triplets in the reference's dispatch order and
converts them with ``bsr_set_from_triplets`` (the radix-sort assembly kernels).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from .. import _arrays as A
from .. import _native as N
from .. import sparse
from . import q1

__all__ = [
    "Grid2D",
    "Grid3D",
    "Cells",
    "BoundarySides",
    "make_polynomial_space",
    "make_test",
    "make_trial",
    "integrate",
    "project_linear_system",
    "diffusion_form",
    "linear_elasticity_form",
    "mass_form",
    "linear_form",
    "boundary_projector_form",
    "gaussian_random_field",
]

_f32 = ctypes.c_float
N.register("gb_q1_triplet_count", N._c_i64, [N._c_int] * 4)
N.register("gb_q1_assemble_triplets", N._c_int,
           [N._c_int, N._c_int, N._c_int, N._c_int, N._c_int, N._vp, N._vp, N._vp, _f32, N._vp, _f32, N._vp, N._vp,
            N._vp, N._vp])
N.register("gb_q1_assemble_rhs", N._c_int,
           [N._c_int, N._c_int, N._c_int, N._c_int, N._c_int, N._vp, N._vp, _f32, _f32, _f32, N._vp, N._vp])
N.register("gb_grid_boundary_mask", N._c_int,
           [N._c_int, N._c_int, N._c_int, N._c_int, N._c_int, N._c_int, N._c_int, N._vp, N._vp])
N.register("gb_q1_bsr_nnz_max", N._c_i64, [N._c_int] * 4)
N.register("gb_q1_assemble_bsr_workspace_bytes", N._c_sz, [N._c_int] * 4)
N.register("gb_q1_assemble_bsr", N._c_int,
           [N._c_int, N._c_int, N._c_int, N._c_int, N._c_int, N._vp, N._vp, N._vp, _f32, N._vp, _f32, N._c_int, N._vp,
            N._vp, N._vp, N._vp, N._vp, N._c_sz, N._vp])
N.register("gb_dirichlet_project", N._c_int,
           [N._c_int, N._c_int, N._vp, N._vp, N._vp, N._vp, N._vp, N._vp, N._vp, N._c_int, N._vp])


class Grid2D:
    """Regular 2-D grid of ``res`` cells over ``[bounds_lo, bounds_hi]`` (reference grid_2d.py)."""

    dimension = 2

    def __init__(self, res=(1, 1), bounds_lo=(0.0, 0.0), bounds_hi=(1.0, 1.0)):
        self.res = tuple(int(r) for r in res)[:2]
        self.bounds_lo = tuple(float(v) for v in bounds_lo)[:2]
        self.bounds_hi = tuple(float(v) for v in bounds_hi)[:2]
        self.cell_size = tuple((self.bounds_hi[d] - self.bounds_lo[d]) / self.res[d] for d in range(2))

    @property
    def cell_dimension(self) -> int:
        return self.dimension

    def cell_count(self) -> int:
        return int(np.prod(self.res))

    def node_count(self) -> int:
        return int(np.prod([r + 1 for r in self.res]))

    def _dims(self):
        return (self.res[0], self.res[1], 0)


class Grid3D(Grid2D):
    """Regular 3-D grid of ``res`` cells (reference grid_3d.py)."""

    dimension = 3

    def __init__(self, res=(1, 1, 1), bounds_lo=(0.0, 0.0, 0.0), bounds_hi=(1.0, 1.0, 1.0)):
        self.res = tuple(int(r) for r in res)[:3]
        self.bounds_lo = tuple(float(v) for v in bounds_lo)[:3]
        self.bounds_hi = tuple(float(v) for v in bounds_hi)[:3]
        self.cell_size = tuple((self.bounds_hi[d] - self.bounds_lo[d]) / self.res[d] for d in range(3))

    def _dims(self):
        return self.res


@dataclass
class Cells:
    geometry: Any


@dataclass
class BoundarySides:
    """All boundary faces, or the faces selected by ``faces`` (e.g. ``("x-",)`` for the x=0 face)."""

    geometry: Any
    faces: tuple = ("x-", "x+", "y-", "y+", "z-", "z+")

    def face_bits(self) -> int:
        bits = 0
        for f in self.faces:
            d = "xyz".index(f[0])
            bits |= 1 << (2 * d + (1 if f[1] == "+" else 0))
        return bits


@dataclass
class FunctionSpace:
    geometry: Any
    degree: int
    dof_count: int  # components per node

    def node_count(self) -> int:
        return self.geometry.node_count()

    def make_field(self):
        return A.zeros(self.node_count() * self.dof_count, torch.float32)


def make_polynomial_space(geo, degree: int = 1, dtype=float, element_basis=None, **kwargs) -> FunctionSpace:
    """Q1 nodal space (``degree=1``), scalar (``dtype=float``) or 3-vector (``dtype`` of length 3)."""
    if degree != 1:
        raise NotImplementedError("only degree-1 (Q1) spaces are implemented")
    ncomp = int(getattr(dtype, "_length_", 0) or (3 if dtype in ("vec3", (3,)) else 1))
    if ncomp not in (1, 3):
        raise NotImplementedError("scalar or 3-component spaces only")
    return FunctionSpace(geo, degree, ncomp)


@dataclass
class _Field:
    space: FunctionSpace
    domain: Any
    role: str


def make_test(space: FunctionSpace, domain=None) -> _Field:
    return _Field(space, domain if domain is not None else Cells(space.geometry), "test")


def make_trial(space: FunctionSpace, domain=None) -> _Field:
    return _Field(space, domain if domain is not None else Cells(space.geometry), "trial")


@dataclass(frozen=True)
class Integrand:
    name: str
    kind: str  # "bilinear" or "linear"


diffusion_form = Integrand("diffusion", "bilinear")  # nu(s) * dot(grad u, grad v)
linear_elasticity_form = Integrand("elasticity", "bilinear")  # 2 mu eps(u):eps(v) + lambda div u div v
mass_form = Integrand("mass", "bilinear")  # u . v
linear_form = Integrand("linear", "linear")  # f . v
boundary_projector_form = Integrand("boundary_projector", "bilinear")  # u . v on boundary sides (nodal)


def _cell_array(v, ncells: int):
    """None + constant, or a device float32 per-cell array."""
    if v is None:
        return None, 1.0
    if isinstance(v, (int, float, np.floating)):
        return None, float(v)
    t = A.as_tensor(v) if not isinstance(v, np.ndarray) else A.from_numpy(v.astype(np.float32))
    t = t.reshape(-1).to(torch.float32).contiguous()
    if t.numel() != ncells:
        raise ValueError(f"per-cell coefficient must have {ncells} entries, got {t.numel()}")
    return t, 0.0


@A.on_caller_stream
def integrate(integrand: Integrand, domain=None, quadrature=None, fields=None, values=None, accumulate_dtype=None,
              output_dtype=None, output=None, device=None, temporary_store=None, kernel_options=None, assembly=None,
              add=False, bsr_options=None):
    """Assemble a bilinear form into a BSR matrix or a linear form into a vector.

    Signature of ``warp.fem.integrate`` (``warp/_src/fem/integrate.py:1895-1910``).  ``values``:
    ``nu`` (diffusion; scalar or per-cell), ``lame`` = (lambda, mu) (elasticity; scalars or
    per-cell arrays), ``f`` (linear form; nodal array or constant scalar/3-vector).
    """
    fields = fields or {}
    values = values or {}
    if not isinstance(integrand, Integrand):
        raise NotImplementedError(
            f"integrand {getattr(integrand, '__name__', integrand)!r} has no kernel here; supported: diffusion, "
            "elasticity, mass, linear and boundary-projector forms")
    test = fields.get("v")
    trial = fields.get("u")
    if test is None:
        raise ValueError("a test field 'v' is required")
    space = test.space
    geo = space.geometry
    dim = geo.dimension
    nx, ny, nz = geo._dims()
    ncomp = space.dof_count
    stream = A.stream()
    L = N.lib()
    h = tuple(float(v) for v in geo.cell_size)

    if integrand.kind == "linear":
        out = A.empty(geo.node_count() * ncomp, torch.float32) if output is None else A.as_tensor(output)
        M = A.from_numpy(q1.mass(dim, h))
        f = values.get("f", 1.0)
        if isinstance(f, (int, float)) or (isinstance(f, (tuple, list)) and len(f) <= 3):
            fc = [float(f)] * ncomp if isinstance(f, (int, float)) else [float(v) for v in f] + [0.0] * (3 - len(f))
            N.check(L.gb_q1_assemble_rhs(dim, nx, ny, nz, ncomp, A.ptr(M), None, fc[0], fc[1] if ncomp > 1 else 0.0,
                                         fc[2] if ncomp > 2 else 0.0, A.ptr(out), stream), "q1_rhs")
        else:
            ft = A.as_tensor(f) if not isinstance(f, np.ndarray) else A.from_numpy(f.astype(np.float32))
            ft = ft.reshape(-1).to(torch.float32).contiguous()
            N.check(L.gb_q1_assemble_rhs(dim, nx, ny, nz, ncomp, A.ptr(M), A.ptr(ft), 0.0, 0.0, 0.0, A.ptr(out),
                                         stream), "q1_rhs")
        out._keep = M
        return out

    if integrand.name == "boundary_projector" or assembly == "nodal":
        dom = test.domain
        bits = dom.face_bits() if isinstance(dom, BoundarySides) else 0x3F
        if dim == 2:
            bits &= 0xF
        mask = A.empty(geo.node_count() * ncomp, torch.float32)
        comp_mask = int(values.get("components", (1 << ncomp) - 1))
        N.check(L.gb_grid_boundary_mask(dim, nx, ny, nz, bits, ncomp, comp_mask, A.ptr(mask), stream), "mask")
        return _diagonal_matrix(mask, ncomp)

    if trial is None:
        raise ValueError("a bilinear form needs a trial field 'u'")
    ncells = geo.cell_count()
    if integrand.name == "diffusion":
        if ncomp != 1:
            raise NotImplementedError("diffusion form on scalar spaces")
        K0 = A.from_numpy(q1.stiffness(dim, h).astype(np.float32))
        K1 = None
        c0, c0c = _cell_array(values.get("nu", 1.0), ncells)
        c1, c1c = None, 0.0
    elif integrand.name == "mass":
        if ncomp != 1:
            raise NotImplementedError("mass form on scalar spaces")
        K0 = A.from_numpy(q1.mass(dim, h).astype(np.float32))
        K1 = None
        c0, c0c = _cell_array(values.get("rho", 1.0), ncells)
        c1, c1c = None, 0.0
    elif integrand.name == "elasticity":
        if ncomp != 3 or dim != 3:
            raise NotImplementedError("elasticity form on 3-D vector spaces")
        KL, KM = q1.elasticity(dim, h)
        K0, K1 = A.from_numpy(KL.astype(np.float32)), A.from_numpy(KM.astype(np.float32))
        lam, mu = values.get("lame", (1.0, 1.0))
        c0, c0c = _cell_array(lam, ncells)
        c1, c1c = _cell_array(mu, ncells)
    else:
        raise NotImplementedError(integrand.name)

    nnode = geo.node_count()
    block_type = torch.float32 if ncomp == 1 else ((3, 3), torch.float32)
    opts = dict(bsr_options or {})
    construction = opts.pop("construction", "auto")
    if construction not in ("triplets", "row_compress", "auto"):
        raise ValueError(f"Unsupported BSR construction policy: {construction}")
    prune = bool(opts.pop("prune_numerical_zeros", True))
    if add and output is not None:
        raise NotImplementedError("add=True is not supported")
    if construction == "auto":
        # the structure of a Q1 grid is known from the element: assemble the compact BSR directly (the
        # matrix the triplet construction gives, bit for bit, without writing or sorting triplets)
        mat = output if output is not None else sparse.bsr_zeros(nnode, nnode, block_type)
        cap = int(L.gb_q1_bsr_nnz_max(dim, nx, ny, nz))
        mat.offsets = A.empty(nnode + 1, torch.int32)
        mat.columns = A.empty(cap, torch.int32)
        mat.values = A.empty((cap,) if ncomp == 1 else (cap, ncomp, ncomp), torch.float32)
        mat.row_counts = None
        ws = A.workspace(int(L.gb_q1_assemble_bsr_workspace_bytes(dim, nx, ny, nz)))
        if mat._nnz_host is None:
            mat._nnz_host = torch.zeros(1, dtype=torch.int32, pin_memory=True)
        N.check(L.gb_q1_assemble_bsr(dim, nx, ny, nz, ncomp, A.ptr(K0), A.ptr(K1), A.ptr(c0), c0c, A.ptr(c1), c1c,
                                     int(prune), A.ptr(mat.offsets), A.ptr(mat.columns), A.ptr(mat.values),
                                     mat._nnz_host.data_ptr(), ws.data_ptr(), ws.numel(), stream), "q1_assemble_bsr")
        event = torch.cuda.Event()
        event.record()
        mat._nnz_event, mat._nnz_exact, mat.nnz = event, False, cap
        mat._topology_version += 1
        mat._keep_assembly = (K0, K1, c0, c1, ws)
        return mat
    T = int(L.gb_q1_triplet_count(dim, nx, ny, nz))
    rows = A.empty(T, torch.int32)
    cols = A.empty(T, torch.int32)
    vals = A.empty((T,) if ncomp == 1 else (T, ncomp, ncomp), torch.float32)
    N.check(L.gb_q1_assemble_triplets(dim, nx, ny, nz, ncomp, A.ptr(K0), A.ptr(K1), A.ptr(c0), c0c, A.ptr(c1), c1c,
                                      A.ptr(rows), A.ptr(cols), A.ptr(vals), stream), "q1_assemble")
    mat = output if (output is not None and not add) else sparse.bsr_zeros(nnode, nnode, block_type)
    if construction == "row_compress":
        # the candidates come out row by row (test node, ascending element, trial node): they already
        # are the padded row layout of integrate.py:1664-1712, so only a row-local compression remains
        status = A.zeros(1, torch.int32)
        offsets = A.empty(nnode + 1, torch.int32)
        N.check(L.gb_bsr_rows_to_offsets(T, A.ptr(rows), nnode, A.ptr(offsets), A.ptr(status), stream), "row offsets")
        mat.offsets, mat.columns, mat.values, mat.row_counts = offsets, cols, vals, None
        mat.nnz, mat._nnz_event, mat._nnz_exact = T, None, True
        sparse.bsr_compress(mat, prune_numerical_zeros=prune)
        if int(status.item()) != 0:
            raise RuntimeError("fem.integrate(row_compress): candidate rows are not grouped by test node")
    else:
        sparse.bsr_set_from_triplets(mat, rows, cols, vals, prune_numerical_zeros=prune)
    mat._keep_assembly = (K0, K1, c0, c1)
    return mat


def _diagonal_matrix(mask: torch.Tensor, ncomp: int) -> sparse.BsrMatrix:
    n = mask.numel() // ncomp
    idx = torch.arange(n, dtype=torch.int32, device=mask.device)
    if ncomp == 1:
        vals = mask.clone()
        P = sparse.bsr_zeros(n, n, torch.float32)
    else:
        vals = torch.zeros((n, ncomp, ncomp), dtype=torch.float32, device=mask.device)
        vals.diagonal(dim1=1, dim2=2).copy_(mask.view(n, ncomp))
        P = sparse.bsr_zeros(n, n, ((ncomp, ncomp), torch.float32))
    sparse.bsr_set_from_triplets(P, idx, idx, vals)
    P._dirichlet_mask = mask
    return P


@A.on_caller_stream
def project_linear_system(system_matrix: sparse.BsrMatrix, system_rhs, projector_matrix: sparse.BsrMatrix,
                          fixed_value=None, normalize_projector: bool = True) -> None:
    """``A <- (I-P) A (I-P) + P`` and ``b <- (I-P)(b - A P f) + P f`` in place, keeping A's structure.

    ``projector_matrix`` must be diagonal (as the nodal boundary projector is); normalisation maps
    each positive diagonal entry to 1 (reference: ``dirichlet.py:126-184``).
    """
    mask = getattr(projector_matrix, "_dirichlet_mask", None)
    if mask is None:
        diag = sparse.bsr_get_diag(projector_matrix)
        if diag.dim() == 3:
            off = diag.clone()
            off.diagonal(dim1=1, dim2=2).zero_()
            if bool((off != 0).any()):
                raise NotImplementedError("non-diagonal projector blocks are not supported")
            d = diag.diagonal(dim1=1, dim2=2).reshape(-1)
        else:
            d = diag.reshape(-1)
        mask = (d > 0).to(torch.float32) if normalize_projector else d.to(torch.float32)
    rhs = A.as_tensor(system_rhs).reshape(-1)
    fixed = None if fixed_value is None else A.as_tensor(fixed_value).reshape(-1).to(torch.float32)
    tmp = A.empty(rhs.numel(), torch.float32) if fixed is not None else None
    system_matrix.nnz_sync()
    N.check(N.lib().gb_dirichlet_project(system_matrix.block_shape[0], system_matrix.nrow,
                                         A.ptr(system_matrix.offsets), A.ptr(system_matrix.columns),
                                         A.ptr(system_matrix.values), A.ptr(mask), A.ptr(rhs), A.ptr(fixed),
                                         A.ptr(tmp), 1, A.stream()), "dirichlet_project")


def gaussian_random_field(shape, corr_length: float, sigma: float, seed: int, cell_size=None) -> np.ndarray:
    """Stationary Gaussian random field with a squared-exponential covariance, sampled on cell
    centres by spectral (FFT) synthesis on a periodic grid twice the size (input synthesis for the
    benchmark configurations; float64 host array with the requested standard deviation)."""
    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    ext = tuple(2 * s for s in shape)
    if cell_size is None:
        cell_size = tuple(1.0 / s for s in shape)
    freqs = np.meshgrid(*[np.fft.fftfreq(n, d=h) for n, h in zip(ext, cell_size)], indexing="ij")
    k2 = sum(f ** 2 for f in freqs)
    # spectral density of exp(-r^2 / (2 l^2)) ~ exp(-2 pi^2 l^2 k^2)
    spec = np.exp(-2.0 * np.pi ** 2 * corr_length ** 2 * k2)
    noise = rng.standard_normal(ext)
    field = np.real(np.fft.ifftn(np.fft.fftn(noise) * np.sqrt(spec)))
    field = field[tuple(slice(0, s) for s in shape)]
    field = (field - field.mean()) / (field.std() + 1e-300) * sigma
    return field
