"""GPU parity of the Q1 assembly path: triplets, BSR structure/values, rhs, Dirichlet projection."""

import numpy as np
import pytest
import torch

import oracle
from oracle import fem_q1

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("res", [(64, 64), (7, 5), (9, 7, 5), (16, 16, 16)])
def test_diffusion_triplets_and_bsr(cuda, res):
    import warp_gb300._arrays as A
    import warp_gb300._native as N
    from warp_gb300 import fem

    dim = len(res)
    geo = fem.Grid2D(res=res) if dim == 2 else fem.Grid3D(res=res)
    rng = np.random.default_rng(sum(res))
    nu = np.exp(rng.standard_normal(geo.cell_count())).astype(np.float32)
    # raw triplets: rows/cols bit-exact, values within 1e-6 of the oracle (relative to the row max)
    space = fem.make_polynomial_space(geo, degree=1)
    K = fem.q1.stiffness(dim, geo.cell_size)
    Kd = torch.from_numpy(K.astype(np.float32)).cuda()
    nud = torch.from_numpy(nu).cuda()
    L = N.lib()
    T = int(L.gb_q1_triplet_count(dim, *geo._dims()))
    rows = torch.empty(T, dtype=torch.int32, device="cuda")
    cols = torch.empty(T, dtype=torch.int32, device="cuda")
    vals = torch.empty(T, dtype=torch.float32, device="cuda")
    N.check(L.gb_q1_assemble_triplets(dim, *geo._dims(), 1, Kd.data_ptr(), None, nud.data_ptr(), 0.0, None, 0.0,
                                      rows.data_ptr(), cols.data_ptr(), vals.data_ptr(), A.stream()))
    r, c, v = fem_q1.assemble_triplets(res, coef=nu)
    np.testing.assert_array_equal(rows.cpu().numpy(), r)
    np.testing.assert_array_equal(cols.cpu().numpy(), c)
    np.testing.assert_allclose(vals.cpu().numpy(), v, rtol=1e-6, atol=1e-6 * np.abs(v).max())
    # full integrate -> BSR.  Structure and values: bit-exact against the oracle's triplet->BSR of
    # the same triplets (same stable summation order).  On cubic cells the exact edge-neighbour
    # entries of the Q1 stiffness are 0; quadrature leaves them at rounding level (as the
    # reference's fp32 quadrature does), so pruning keeps the full (3m-2)^dim pattern.
    Am = fem.integrate(fem.diffusion_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                       values={"nu": nu})
    nn = geo.node_count()
    vg = vals.cpu().numpy()
    o = oracle.bsr_from_triplets(nn, nn, r, c, vg)
    nnz = Am.nnz_sync()
    assert nnz == o["nnz"]
    np.testing.assert_array_equal(Am.offsets.cpu().numpy(), o["offsets"])
    np.testing.assert_array_equal(Am.columns[:nnz].cpu().numpy(), o["columns"])
    np.testing.assert_array_equal(Am.values[:nnz].cpu().numpy(), o["values"])
    # values against the independent closed-form oracle within 1e-6 of the row maximum
    oe = oracle.bsr_from_triplets(nn, nn, r, c, v, prune_numerical_zeros=False)
    assert oe["nnz"] == nnz
    got = Am.values[:nnz].cpu().numpy()
    rowmax = np.maximum.reduceat(np.abs(oe["values"]), oe["offsets"][:-1])
    rowid = np.repeat(np.arange(nn), np.diff(oe["offsets"]))
    assert np.all(np.abs(got - oe["values"]) <= 1e-6 * rowmax[rowid])
    # a regular Q1 grid couples every node with its (up to) 3^dim neighbours
    m = [k + 1 for k in res]
    assert nnz == int(np.prod([3 * mk - 2 for mk in m]))


def test_elasticity_bsr_3x3(cuda):
    from warp_gb300 import fem

    res = (6, 5, 4)
    geo = fem.Grid3D(res=res)
    space = fem.make_polynomial_space(geo, degree=1, dtype="vec3")
    rng = np.random.default_rng(2)
    E = 1e3 * np.exp(rng.standard_normal(geo.cell_count()))
    lam, mu = fem.q1.lame_from_young(E, 0.3)
    Am = fem.integrate(fem.linear_elasticity_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                       values={"lame": (lam.astype(np.float32), mu.astype(np.float32))})
    r, c, v = fem_q1.assemble_triplets(res, ncomp=3, lame=(lam, mu))
    nn = geo.node_count()
    o = oracle.bsr_from_triplets(nn, nn, r, c, v.reshape(len(r), 9), block_shape=(3, 3), prune_numerical_zeros=False)
    nnz = Am.nnz_sync()
    assert nnz == o["nnz"] == int(np.prod([3 * (k + 1) - 2 for k in res]))
    np.testing.assert_array_equal(Am.offsets.cpu().numpy(), o["offsets"])
    np.testing.assert_array_equal(Am.columns[:nnz].cpu().numpy(), o["columns"])
    got = Am.values[:nnz].cpu().numpy()
    scale = np.abs(o["values"]).max()
    assert np.abs(got - o["values"]).max() <= 1e-6 * scale


@pytest.mark.parametrize("res,ncomp", [((10, 12), 1), ((6, 5, 7), 1), ((5, 4, 3), 3)])
def test_rhs_and_projection(cuda, res, ncomp):
    from warp_gb300 import fem

    dim = len(res)
    geo = fem.Grid2D(res=res) if dim == 2 else fem.Grid3D(res=res)
    space = fem.make_polynomial_space(geo, degree=1, dtype="vec3" if ncomp == 3 else float)
    nn = geo.node_count()
    rng = np.random.default_rng(1)
    fn = rng.uniform(-1, 1, nn * ncomp).astype(np.float32)
    b = fem.integrate(fem.linear_form, fields={"v": fem.make_test(space)}, values={"f": torch.from_numpy(fn).cuda()})
    exp = fem_q1.assemble_rhs(res, f_nodal=fn, ncomp=ncomp)
    np.testing.assert_allclose(b.cpu().numpy(), exp, rtol=1e-6, atol=1e-7 * np.abs(exp).max())
    if ncomp == 1:
        Am = fem.integrate(fem.diffusion_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)})
        faces = ("x-", "x+", "y-", "y+", "z-", "z+")
    else:
        Am = fem.integrate(fem.linear_elasticity_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                           values={"lame": (1.0, 0.5)})
        faces = ("x-",)
    dense = Am.numpy_dense()
    bd = fem.BoundarySides(geo, faces)
    P = fem.integrate(fem.boundary_projector_form, fields={"u": fem.make_trial(space, bd),
                                                           "v": fem.make_test(space, bd)}, assembly="nodal")
    fixed = rng.uniform(-1, 1, nn * ncomp).astype(np.float32)
    fem.project_linear_system(Am, b, P, torch.from_numpy(fixed).cuda())
    mask = fem_q1.boundary_mask(res, faces, ncomp)
    A2, b2 = fem_q1.project_dense(dense, exp, mask, fixed.astype(np.float64))
    np.testing.assert_allclose(Am.numpy_dense(), A2, rtol=1e-5, atol=1e-6 * np.abs(A2).max())
    np.testing.assert_allclose(b.cpu().numpy(), b2, rtol=1e-4, atol=1e-5 * np.abs(b2).max())
    # structure is preserved (explicit zeros kept)
    assert Am.nnz_sync() == (Am.offsets[-1].item())


@pytest.mark.parametrize("res,ncomp,zero_cells", [((9, 7), 1, False), ((6, 5, 7), 1, False), ((6, 5, 7), 1, True),
                                                  ((5, 4, 3), 3, False), ((5, 4, 3), 3, True), ((4, 6), 1, True)])
@pytest.mark.parametrize("prune", [True, False])
def test_direct_assembly_equals_triplet_construction(cuda, res, ncomp, zero_cells, prune):
    """fem.integrate's default (direct compact-BSR assembly, no triplets) returns the triplet
    construction's matrix bit for bit: offsets, columns, value bits -- including the pruning of
    all-zero triplets (cells with a zero coefficient) and prune_numerical_zeros=False."""
    from warp_gb300 import fem

    dim = len(res)
    geo = fem.Grid2D(res=res) if dim == 2 else fem.Grid3D(res=res)
    rng = np.random.default_rng(5)
    coef = np.exp(rng.standard_normal(geo.cell_count())).astype(np.float32)
    if zero_cells:
        coef[rng.random(coef.size) < 0.3] = 0.0
        coef[0] = -0.0
    if ncomp == 1:
        space = fem.make_polynomial_space(geo, degree=1)
        form, vals = fem.diffusion_form, {"nu": coef}
    else:
        space = fem.make_polynomial_space(geo, degree=1, dtype="vec3")
        form, vals = fem.linear_elasticity_form, {"lame": (coef * 1.7, coef)}
    fields = {"u": fem.make_trial(space), "v": fem.make_test(space)}
    mats = {c: fem.integrate(form, fields=fields, values=vals,
                             bsr_options={"construction": c, "prune_numerical_zeros": prune})
            for c in ("auto", "triplets")}
    d, t = mats["auto"], mats["triplets"]
    nnz = d.nnz_sync()
    assert nnz == t.nnz_sync()
    np.testing.assert_array_equal(d.offsets.cpu().numpy(), t.offsets.cpu().numpy())
    np.testing.assert_array_equal(d.columns[:nnz].cpu().numpy(), t.columns[:nnz].cpu().numpy())
    np.testing.assert_array_equal(d.values[:nnz].cpu().numpy().view(np.uint32), t.values[:nnz].cpu().numpy().view(np.uint32))
    if not prune:
        assert nnz == int(np.prod([3 * (k + 1) - 2 for k in res]))
