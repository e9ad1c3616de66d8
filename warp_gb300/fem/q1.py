"""Q1 reference-element matrices (host-side constants of the assembly kernels).

The bi/trilinear shape functions on the unit cell, integrated with the 2-point Gauss-Legendre
rule per axis (``warp/_src/fem/polynomial.py:194-216``; exact for products of Q1 functions and
their gradients), scaled to a cell of size ``h``.  These small tables (at most 24 x 24) are
computed once per grid spacing and uploaded; the per-cell coefficient scaling and the triplet
generation run on the GPU (``gb_q1_assemble_triplets``).

Element-local node order: ``a = i*4 + j*2 + k`` in 3-D and ``a = i*2 + j`` in 2-D
(``warp/_src/fem/space/shape/cube_shape_function.py:103-113``).
"""

from __future__ import annotations

import functools

import numpy as np

_GAUSS2 = (0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0))


def _local_nodes(dim: int) -> np.ndarray:
    if dim == 2:
        return np.array([[a >> 1, a & 1] for a in range(4)], dtype=np.int64)
    return np.array([[a >> 2, (a >> 1) & 1, a & 1] for a in range(8)], dtype=np.int64)


def _shape_and_grad(dim: int, xi: np.ndarray, h: np.ndarray):
    """phi[a] and grad phi[a] (physical coordinates) at reference point xi in [0,1]^dim."""
    nodes = _local_nodes(dim)
    npe = nodes.shape[0]
    phi = np.ones(npe)
    grad = np.ones((npe, dim))
    for a in range(npe):
        for d in range(dim):
            f = xi[d] if nodes[a, d] == 1 else 1.0 - xi[d]
            df = 1.0 if nodes[a, d] == 1 else -1.0
            phi[a] *= f
            for e in range(dim):
                grad[a, e] *= (df / h[d]) if e == d else f
    return phi, grad


def _quadrature(dim: int):
    pts = []
    for idx in np.ndindex(*([2] * dim)):
        pts.append(np.array([_GAUSS2[i] for i in idx]))
    w = 0.5 ** dim
    return pts, w


@functools.lru_cache(maxsize=64)
def stiffness(dim: int, h: tuple[float, ...]) -> np.ndarray:
    """K[a, b] = int_cell grad phi_a . grad phi_b  (unit diffusion coefficient)."""
    h = np.asarray(h, np.float64)
    vol = float(np.prod(h))
    pts, w = _quadrature(dim)
    npe = 2 ** dim
    K = np.zeros((npe, npe))
    for xi in pts:
        _, g = _shape_and_grad(dim, xi, h)
        K += w * vol * g @ g.T
    return K


@functools.lru_cache(maxsize=64)
def mass(dim: int, h: tuple[float, ...]) -> np.ndarray:
    """M[a, b] = int_cell phi_a phi_b."""
    h = np.asarray(h, np.float64)
    vol = float(np.prod(h))
    pts, w = _quadrature(dim)
    npe = 2 ** dim
    M = np.zeros((npe, npe))
    for xi in pts:
        phi, _ = _shape_and_grad(dim, xi, h)
        M += w * vol * np.outer(phi, phi)
    return M


@functools.lru_cache(maxsize=64)
def elasticity(dim: int, h: tuple[float, ...]) -> tuple[np.ndarray, np.ndarray]:
    """(K_lambda, K_mu) of the isotropic form 2 mu eps(u):eps(v) + lambda div u div v.

    Row (a, i) = test node a, component i; column (b, j) = trial node b, component j:
      K_lambda[(a,i),(b,j)] = int d_i phi_a d_j phi_b
      K_mu[(a,i),(b,j)]     = int d_j phi_a d_i phi_b + delta_ij grad phi_a . grad phi_b
    """
    h = np.asarray(h, np.float64)
    vol = float(np.prod(h))
    pts, w = _quadrature(dim)
    npe = 2 ** dim
    nd = npe * dim
    KL = np.zeros((nd, nd))
    KM = np.zeros((nd, nd))
    for xi in pts:
        _, g = _shape_and_grad(dim, xi, h)
        for a in range(npe):
            for b in range(npe):
                gg = float(g[a] @ g[b])
                for i in range(dim):
                    for j in range(dim):
                        KL[a * dim + i, b * dim + j] += w * vol * g[a, i] * g[b, j]
                        KM[a * dim + i, b * dim + j] += w * vol * (g[a, j] * g[b, i] + (gg if i == j else 0.0))
    return KL, KM


def lame_from_young(E, nu):
    """Lame parameters (lambda, mu) from Young's modulus and Poisson ratio."""
    E = np.asarray(E, np.float64)
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    return lam, mu
