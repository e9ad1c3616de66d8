"""Seeded synthetic FEM systems with the shapes of the benchmark workloads.

Every system is assembled on the GPU through the drop-in API (``fem.integrate`` ->
``bsr_set_from_triplets`` -> ``project_linear_system``); only the random coefficient / source
fields are drawn on the host (NumPy, seeded).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _arrays as A
from . import fem, sparse


@dataclass
class System:
    A: sparse.BsrMatrix
    b: torch.Tensor
    geo: object
    coef: np.ndarray
    description: str


def diffusion(res, sigma: float = 1.5, corr_length: float = 0.1, seed: int = 0, lognormal: bool = True,
              constant: float | None = None, field_cell_size: float | None = None, coef=None, f=None) -> System:
    """-div(a grad u) = f, Q1 on a unit Grid2D/Grid3D, a = exp(g) with g a squared-exponential GRF
    (correlation ``corr_length``, std ``sigma``) per cell, f ~ U[-1, 1] per node, u = 0 on the whole
    boundary imposed by projection.  ``field_cell_size`` samples the field as if the cells had that
    size (a sub-block of a finer grid: same correlation length in cells); ``coef`` gives the per-cell
    coefficient directly and ``f`` the nodal source."""
    res = tuple(int(r) for r in res)
    geo = fem.Grid2D(res=res) if len(res) == 2 else fem.Grid3D(res=res)
    rng = np.random.default_rng(seed)
    if coef is not None:
        coef = np.asarray(coef, np.float64).reshape(-1)
    elif constant is not None:
        coef = np.full(geo.cell_count(), float(constant))
    elif lognormal:
        cs = None if field_cell_size is None else (float(field_cell_size),) * len(res)
        g = fem.gaussian_random_field(res, corr_length, sigma, seed, cell_size=cs)
        coef = np.exp(g).reshape(-1)
    else:
        coef = np.ones(geo.cell_count())
    f = rng.uniform(-1.0, 1.0, geo.node_count()).astype(np.float32) if f is None else np.asarray(f, np.float32)
    space = fem.make_polynomial_space(geo, degree=1)
    Am = fem.integrate(fem.diffusion_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                       values={"nu": coef.astype(np.float32)})
    b = fem.integrate(fem.linear_form, fields={"v": fem.make_test(space)}, values={"f": A.from_numpy(f)})
    bd = fem.BoundarySides(geo)
    P = fem.integrate(fem.boundary_projector_form,
                      fields={"u": fem.make_trial(space, bd), "v": fem.make_test(space, bd)}, assembly="nodal")
    fem.project_linear_system(Am, b, P)
    Am.nnz_sync()
    return System(Am, b, geo, coef, f"Q1 diffusion {'x'.join(map(str, res))}, lognormal sigma={sigma} l={corr_length}")


def elasticity(res, sigma: float = 1.0, corr_length: float | None = None, seed: int = 0, poisson: float = 0.3,
               young: float = 1e3) -> System:
    """Isotropic linear elasticity, Q1 vec3 on a unit Grid3D, E = young * exp(N(0, sigma^2)) per cell
    (i.i.d., or a GRF with ``corr_length``), Poisson ratio ``poisson``, body force (0, -9.81, 0),
    x = 0 face clamped by projection."""
    res = tuple(int(r) for r in res)
    geo = fem.Grid3D(res=res)
    rng = np.random.default_rng(seed)
    if corr_length is None:
        g = rng.standard_normal(geo.cell_count()) * sigma
    else:
        g = fem.gaussian_random_field(res, corr_length, sigma, seed).reshape(-1)
    E = young * np.exp(g)
    lam, mu = fem.q1.lame_from_young(E, poisson)
    space = fem.make_polynomial_space(geo, degree=1, dtype="vec3")
    Am = fem.integrate(fem.linear_elasticity_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                       values={"lame": (lam.astype(np.float32), mu.astype(np.float32))})
    b = fem.integrate(fem.linear_form, fields={"v": fem.make_test(space)}, values={"f": (0.0, -9.81, 0.0)})
    bd = fem.BoundarySides(geo, ("x-",))
    P = fem.integrate(fem.boundary_projector_form,
                      fields={"u": fem.make_trial(space, bd), "v": fem.make_test(space, bd)}, assembly="nodal")
    fem.project_linear_system(Am, b, P)
    Am.nnz_sync()
    return System(Am, b, geo, E, f"Q1 elasticity {'x'.join(map(str, res))}, E lognormal sigma={sigma}")
