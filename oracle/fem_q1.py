"""ORACLE (test infrastructure only): NumPy FP64 restatement of Q1 assembly on Grid2D/Grid3D.

Follows the reference's definitions:
  * node numbering x*(ny+1)*(nz+1) + y*(nz+1) + z  (warp/_src/fem/space/grid_3d_function_space.py:202-204)
  * cell numbering x*ny*nz + y*nz + z              (warp/_src/fem/geometry/grid_3d.py:269-271)
  * element-local node i*4 + j*2 + k               (warp/_src/fem/space/shape/cube_shape_function.py:103-113)
  * triplet index = (node-element pair) * NPE + trial node, pairs ordered by test node then
    ascending element (warp/_src/fem/field/virtual.py:1084-1115, integrate.py:1637)
  * diffusion nu grad u . grad v, isotropic elasticity 2 mu eps(u):eps(v) + lambda div u div v
    (warp/examples/fem/example_diffusion.py:31-36, example_elastic_shape_optimization.py:66-84)
  * Dirichlet projection A <- (I-P) A (I-P) + P, b <- (I-P)(b - A P f) + P f
    (warp/_src/fem/dirichlet.py:69-124)
Element matrices are built here from closed-form 1-D integrals (tensor products), independently
of the product code's quadrature tables.
"""

from __future__ import annotations

import numpy as np


def _1d(h: float):
    m = h / 6.0 * np.array([[2.0, 1.0], [1.0, 2.0]])      # int N_p N_q
    k = 1.0 / h * np.array([[1.0, -1.0], [-1.0, 1.0]])    # int N_p' N_q'
    c = np.array([[-0.5, -0.5], [0.5, 0.5]])               # int N_p' N_q
    return m, k, c


def _bits(dim: int, a: int):
    return [(a >> (dim - 1 - d)) & 1 for d in range(dim)]


def element_stiffness(dim: int, h) -> np.ndarray:
    ones = [_1d(h[d]) for d in range(dim)]
    npe = 2 ** dim
    K = np.zeros((npe, npe))
    for a in range(npe):
        ba = _bits(dim, a)
        for b in range(npe):
            bb = _bits(dim, b)
            s = 0.0
            for d in range(dim):
                t = 1.0
                for e in range(dim):
                    m, k, _ = ones[e]
                    t *= k[ba[e], bb[e]] if e == d else m[ba[e], bb[e]]
                s += t
            K[a, b] = s
    return K


def element_mass(dim: int, h) -> np.ndarray:
    ones = [_1d(h[d]) for d in range(dim)]
    npe = 2 ** dim
    M = np.zeros((npe, npe))
    for a in range(npe):
        ba = _bits(dim, a)
        for b in range(npe):
            bb = _bits(dim, b)
            t = 1.0
            for e in range(dim):
                t *= ones[e][0][ba[e], bb[e]]
            M[a, b] = t
    return M


def _grad_grad(dim, ones, ba, bb, i, j):
    """int d_i phi_a d_j phi_b as a product of 1-D integrals."""
    t = 1.0
    for e in range(dim):
        m, k, c = ones[e]
        da, db = (e == i), (e == j)
        if da and db:
            t *= k[ba[e], bb[e]]
        elif da:
            t *= c[ba[e], bb[e]]
        elif db:
            t *= c[bb[e], ba[e]]
        else:
            t *= m[ba[e], bb[e]]
    return t


def element_elasticity(dim: int, h):
    ones = [_1d(h[d]) for d in range(dim)]
    npe = 2 ** dim
    nd = npe * dim
    KL = np.zeros((nd, nd))
    KM = np.zeros((nd, nd))
    for a in range(npe):
        ba = _bits(dim, a)
        for b in range(npe):
            bb = _bits(dim, b)
            gg = sum(_grad_grad(dim, ones, ba, bb, d, d) for d in range(dim))
            for i in range(dim):
                for j in range(dim):
                    KL[a * dim + i, b * dim + j] = _grad_grad(dim, ones, ba, bb, i, j)
                    KM[a * dim + i, b * dim + j] = _grad_grad(dim, ones, ba, bb, j, i) + (gg if i == j else 0.0)
    return KL, KM


def _cells_nodes(res):
    dim = len(res)
    npe = 2 ** dim
    cell_coords = np.stack(np.meshgrid(*[np.arange(r) for r in res], indexing="ij"), -1).reshape(-1, dim)
    pitches = []
    for d in range(dim):
        p = 1
        for e in range(d + 1, dim):
            p *= res[e] + 1
        pitches.append(p)
    pitches = np.array(pitches)
    local = np.array([_bits(dim, a) for a in range(npe)])
    nodes = ((cell_coords[:, None, :] + local[None, :, :]) * pitches).sum(-1)  # [cells, npe]
    return cell_coords, nodes


def assemble_triplets(res, bounds_hi=None, coef=None, lame=None, ncomp=1):
    """Q1 triplets in the reference's order.  Returns rows, cols, values (float32, block [T,nc,nc])."""
    res = tuple(int(r) for r in res)
    dim = len(res)
    if bounds_hi is None:
        bounds_hi = (1.0,) * dim
    h = [bounds_hi[d] / res[d] for d in range(dim)]
    npe = 2 ** dim
    ncells = int(np.prod(res))
    _, nodes = _cells_nodes(res)
    cell_ids = np.arange(ncells)
    if ncomp == 1:
        K = element_stiffness(dim, h)
        c = np.ones(ncells) if coef is None else np.asarray(coef, np.float64).reshape(-1)
        if np.ndim(coef) == 0 and coef is not None:
            c = np.full(ncells, float(coef))
        c = np.asarray(c, np.float32).astype(np.float64)
        vals = c[:, None, None] * K[None]  # [cells, a, b]
    else:
        KL, KM = element_elasticity(dim, h)
        lam, mu = lame
        lam = np.broadcast_to(np.asarray(lam, np.float32).astype(np.float64).reshape(-1), (ncells,))
        mu = np.broadcast_to(np.asarray(mu, np.float32).astype(np.float64).reshape(-1), (ncells,))
        full = lam[:, None, None] * KL[None] + mu[:, None, None] * KM[None]  # [cells, nd, nd]
        vals = full.reshape(ncells, npe, ncomp, npe, ncomp).transpose(0, 1, 3, 2, 4)  # [cells, a, b, i, j]
    # (cell, a, b) -> triplet; order by (row node = nodes[cell,a], cell, b)
    rows = np.repeat(nodes[:, :, None], npe, axis=2)          # [cells, a, b]
    cols = np.repeat(nodes[:, None, :], npe, axis=1)
    cells = np.broadcast_to(cell_ids[:, None, None], rows.shape)
    bidx = np.broadcast_to(np.arange(npe)[None, None, :], rows.shape)
    order = np.lexsort((bidx.reshape(-1), cells.reshape(-1), rows.reshape(-1)))
    r = rows.reshape(-1)[order].astype(np.int32)
    cc = cols.reshape(-1)[order].astype(np.int32)
    if ncomp == 1:
        v = vals.reshape(-1)[order].astype(np.float32)
    else:
        v = vals.reshape(-1, ncomp, ncomp)[order].astype(np.float32)
    return r, cc, v


def assemble_rhs(res, f_nodal=None, f_const=None, ncomp=1, bounds_hi=None):
    """b = M f (consistent Q1 mass), f nodal [nodes*ncomp] or constant per component, in FP64."""
    res = tuple(int(r) for r in res)
    dim = len(res)
    if bounds_hi is None:
        bounds_hi = (1.0,) * dim
    h = [bounds_hi[d] / res[d] for d in range(dim)]
    M = element_mass(dim, h)
    _, nodes = _cells_nodes(res)
    nn = int(np.prod([r + 1 for r in res]))
    b = np.zeros((nn, ncomp))
    for c in range(ncomp):
        if f_nodal is not None:
            fe = np.asarray(f_nodal, np.float64).reshape(nn, ncomp)[:, c][nodes]  # [cells, npe]
        else:
            fe = np.full(nodes.shape, float(f_const[c]))
        contrib = fe @ M.T  # [cells, a]
        np.add.at(b[:, c], nodes.reshape(-1), contrib.reshape(-1))
    return b.reshape(-1)


def boundary_mask(res, faces=("x-", "x+", "y-", "y+", "z-", "z+"), ncomp=1):
    res = tuple(int(r) for r in res)
    dim = len(res)
    coords = np.stack(np.meshgrid(*[np.arange(r + 1) for r in res], indexing="ij"), -1).reshape(-1, dim)
    on = np.zeros(coords.shape[0], bool)
    for f in faces:
        d = "xyz".index(f[0])
        if d >= dim:
            continue
        on |= coords[:, d] == (0 if f[1] == "-" else res[d])
    return np.repeat(on.astype(np.float32), ncomp)


def project_dense(Adense: np.ndarray, b: np.ndarray, mask: np.ndarray, fixed: np.ndarray | None = None):
    P = np.diag(mask.astype(np.float64))
    I = np.eye(len(mask))
    f = np.zeros(len(mask)) if fixed is None else fixed
    b2 = (I - P) @ (b - Adense @ (P @ f)) + P @ f
    A2 = (I - P) @ Adense @ (I - P) + P
    return A2, b2


# ---------------------------------------------------------------------------------------------
# Whole systems for the CPU baseline (the --impl reference arm of bench.py builds its input here,
# without the product library)
# ---------------------------------------------------------------------------------------------
def gaussian_random_field(shape, corr_length: float, sigma: float, seed: int) -> np.ndarray:
    """Input synthesis of the benchmark fields: a stationary Gaussian random field with a
    squared-exponential covariance on cell centres, by spectral (FFT) synthesis on a periodic grid
    twice the size, normalised to standard deviation ``sigma``.  Same method and seed convention as
    the product's field generator (tests check that both give the same field)."""
    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    ext = tuple(2 * s for s in shape)
    h = tuple(1.0 / s for s in shape)
    freqs = np.meshgrid(*[np.fft.fftfreq(n, d=hh) for n, hh in zip(ext, h)], indexing="ij")
    k2 = sum(fq ** 2 for fq in freqs)
    spec = np.exp(-2.0 * np.pi ** 2 * corr_length ** 2 * k2)
    noise = rng.standard_normal(ext)
    field = np.real(np.fft.ifftn(np.fft.fftn(noise) * np.sqrt(spec)))
    field = field[tuple(slice(0, s) for s in shape)]
    return (field - field.mean()) / (field.std() + 1e-300) * sigma


def assemble_csr_stencil(res, coef) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Q1 diffusion matrix on a unit Grid3D as a CSR with every node's full 27-neighbourhood
    (the structure fem.integrate keeps on cubic cells), values summed in FP64 from the closed-form
    element matrix and rounded to fp32 once.  Returns (offsets, columns, values)."""
    res = tuple(int(r) for r in res)
    assert len(res) == 3
    nx, ny, nz = res
    mx, my, mz = nx + 1, ny + 1, nz + 1
    K = element_stiffness(3, [1.0 / r for r in res])
    c = np.asarray(coef, np.float32).astype(np.float64).reshape(nx, ny, nz)
    st = np.zeros((mx, my, mz, 3, 3, 3))  # st[node][dx+1][dy+1][dz+1]
    for a in range(8):
        ai, aj, ak = a >> 2, (a >> 1) & 1, a & 1
        for b in range(8):
            bi, bj, bk = b >> 2, (b >> 1) & 1, b & 1
            st[ai:ai + nx, aj:aj + ny, ak:ak + nz, bi - ai + 1, bj - aj + 1, bk - ak + 1] += c * K[a, b]
    node = np.arange(mx * my * mz).reshape(mx, my, mz)
    cols_full = np.full((mx, my, mz, 3, 3, 3), -1, np.int64)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                sl_dst = (slice(max(0, -dx), mx - max(0, dx)), slice(max(0, -dy), my - max(0, dy)),
                          slice(max(0, -dz), mz - max(0, dz)))
                sl_src = (slice(max(0, dx), mx + min(0, dx)), slice(max(0, dy), my + min(0, dy)),
                          slice(max(0, dz), mz + min(0, dz)))
                cols_full[sl_dst + (dx + 1, dy + 1, dz + 1)] = node[sl_src]
    valid = cols_full.reshape(-1, 27) >= 0
    counts = valid.sum(1)
    offsets = np.zeros(mx * my * mz + 1, np.int32)
    np.cumsum(counts, out=offsets[1:])
    columns = cols_full.reshape(-1, 27)[valid].astype(np.int32)
    values = st.reshape(-1, 27)[valid].astype(np.float32)
    return offsets, columns, values


def diffusion_system_3d(res, sigma: float, corr_length: float, seed: int):
    """The benchmark's 3-D diffusion system (-div(a grad u) = f, a = exp(GRF), f ~ U[-1, 1] per node,
    u = 0 on the boundary by projection), restated on the host.  Returns (offsets, columns, values,
    b) in fp32: the projection zeroes boundary rows and columns (structure kept) and sets their
    diagonal to 1 (warp/_src/fem/dirichlet.py:69-124)."""
    res = tuple(int(r) for r in res)
    rng = np.random.default_rng(seed)
    coef = np.exp(gaussian_random_field(res, corr_length, sigma, seed)).reshape(-1)
    nn = int(np.prod([r + 1 for r in res]))
    f = rng.uniform(-1.0, 1.0, nn).astype(np.float32)
    off, cols, vals = assemble_csr_stencil(res, coef.astype(np.float32))
    b = assemble_rhs(res, f_nodal=f)
    mask = boundary_mask(res) > 0
    rows = np.repeat(np.arange(nn), np.diff(off))
    keep = ~(mask[rows] | mask[cols])
    vals = np.where(keep, vals, np.float32(0.0)).astype(np.float32)
    vals[(rows == cols) & mask[rows]] = 1.0
    b = np.where(mask, 0.0, b).astype(np.float32)
    return off, cols, vals, b
