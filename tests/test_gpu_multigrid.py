"""GPU tests of the multigrid carrier of the learned preconditioner and of flexible CG."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _system(res=(32, 32, 32), sigma=1.0, seed=0):
    from warp_gb300 import problems

    return problems.diffusion(res, sigma=sigma, corr_length=0.1, seed=seed)


def _host(A):
    nnz = A.nnz_sync()
    return A.offsets.cpu().numpy(), A.columns[:nnz].cpu().numpy(), A.values[:nnz].cpu().numpy()


def test_transfers_are_adjoint(cuda):
    """<R t, zc> = <t, P zc> for the masked full-weighting / trilinear pair."""
    import warp_gb300._native as N
    from warp_gb300 import multigrid

    s = _system((16, 16, 16))
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    f, c = mg.levels[0], mg.levels[1]
    rng = np.random.default_rng(0)
    t = torch.from_numpy(rng.standard_normal(f.n).astype(np.float32)).cuda() * (1 - f.mask)
    zc = torch.from_numpy(rng.standard_normal(c.n).astype(np.float32)).cuda() * (1 - c.mask)
    rc = torch.zeros(c.n, device="cuda")
    pz = torch.zeros(f.n, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    N.check(N.lib().gb_mg_restrict(*f.dims, *c.dims, t.data_ptr(), f.mask.data_ptr(), c.mask.data_ptr(),
                                   rc.data_ptr(), st))
    N.check(N.lib().gb_mg_prolong_add(*f.dims, *c.dims, zc.data_ptr(), f.mask.data_ptr(), 1.0, pz.data_ptr(), st))
    lhs = float(torch.dot(rc.double(), zc.double()))
    rhs = float(torch.dot(t.double(), pz.double()))
    assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + 1e-30)
    # prolongation of a constant is the constant away from the masked boundary
    ones = torch.ones(c.n, device="cuda")
    pz.zero_()
    N.check(N.lib().gb_mg_prolong_add(*f.dims, *c.dims, ones.data_ptr(), None, 1.0, pz.data_ptr(), st))
    assert torch.allclose(pz, torch.ones_like(pz))


def test_vcycle_is_symmetric_positive(cuda):
    from warp_gb300 import multigrid

    s = _system((32, 32, 32), sigma=1.5, seed=3)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    assert len(mg.levels) >= 3, mg.describe()
    rng = np.random.default_rng(1)
    m = 1 - mg.levels[0].mask
    r1 = torch.from_numpy(rng.standard_normal(mg.n).astype(np.float32)).cuda() * m
    r2 = torch.from_numpy(rng.standard_normal(mg.n).astype(np.float32)).cuda() * m
    z1, z2 = mg.apply(r1), mg.apply(r2)
    a, b = float(torch.dot(z1.double(), r2.double())), float(torch.dot(r1.double(), z2.double()))
    assert abs(a - b) <= 1e-4 * max(abs(a), abs(b))
    assert float(torch.dot(z1.double(), r1.double())) > 0


@pytest.mark.parametrize("check_every", [0, 10])
def test_fcg_multigrid_converges_fast(cuda, check_every):
    from warp_gb300 import multigrid
    from warp_gb300.optim import linear

    s = _system((48, 48, 48), sigma=1.5, seed=5)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    x = torch.zeros_like(s.b)
    out = linear.fcg(s.A, s.b, x, tol=1e-6, atol=0.0, maxiter=500, M=mg, check_every=check_every)
    if check_every == 0:
        it, rr, at = int(out[0].item()), float(out[1].item()), float(out[2].item())
        assert rr <= at
    else:
        it, err, atol = out
        assert err <= atol
    off, cols, vals = _host(s.A)
    b = s.b.cpu().numpy()
    r = b.astype(np.float64) - oracle.bsr_mv_f64(off, cols, vals, x.cpu().numpy().astype(np.float64))
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 32e-6
    # Jacobi-CG on the same system needs many more iterations
    xj = torch.zeros_like(s.b)
    itj, _, _ = linear.cg(s.A, s.b, xj, tol=1e-6, atol=0.0, maxiter=5000, M=linear.preconditioner(s.A, "diag"))
    assert it * 4 < itj, (it, itj)


def test_refined_fcg_reaches_fp64_tolerance_and_falls_back(cuda):
    from warp_gb300 import multigrid
    from warp_gb300.optim import linear

    s = _system((32, 32, 32), sigma=1.5, seed=7)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    solver = linear.RefinedSolver(s.A, M=mg, method="fcg", inner_tol=1e-5)
    x64, info = solver.solve(s.b, tol=1e-8)
    assert info["converged"], info
    off, cols, vals = _host(s.A)
    b = s.b.cpu().numpy()
    r = b.astype(np.float64) - oracle.bsr_mv_f64(off, cols, vals, x64.cpu().numpy())
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-8

    # a preconditioner that returns -r is not a descent direction: FCG stops and the Jacobi-CG
    # fallback still delivers the solution
    class Bad:
        kernels_per_apply = 1

        def launch(self, stream, r, z):
            import warp_gb300._native as N

            N.check(N.lib().gb_axpby(N.GB_F32, mg.n, -1.0, r, 0.0, r, z, stream))

    bad = linear.RefinedSolver(s.A, M=Bad(), method="fcg", inner_tol=1e-5)
    x64b, infob = bad.solve(s.b, tol=1e-8)
    assert infob["converged"] and bad.fallbacks >= 1


def test_default_coarsest_level_holds_at_most_2200_unknowns(cuda):
    """The default hierarchy stops at the first level with at most 2200 unknowns (13^3 nodes for 1x1,
    9^3 nodes for 3x3 blocks) and holds that level's exact inverse."""
    from warp_gb300 import multigrid, problems

    s = _system((24, 24, 24), sigma=1.5, seed=4)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    assert [lv.dims for lv in mg.levels] == [(25,) * 3, (13,) * 3]
    e = problems.elasticity((16, 16, 16), sigma=1.0, corr_length=0.3, seed=1)
    mge = multigrid.MultigridPreconditioner(e.A, e.geo, e.coef, faces=("x-",))
    assert [lv.dims for lv in mge.levels] == [(17,) * 3, (9,) * 3]
    for m in (mg, mge):
        last = m.levels[-1]
        dense = last.A.numpy_dense()
        inv = last.inv.cpu().numpy().astype(np.float64).reshape(dense.shape)
        assert np.abs(inv @ dense - np.eye(dense.shape[0])).max() < 1e-4


def test_refined_solve_from_zero_edge_cases(cuda):
    """Starting from x = 0 the refined solve reads the initial norms together with the first step's: a zero
    right-hand side returns x = 0 after no outer step, max_outer = 0 reports the initial residual, and a
    given starting iterate still goes through the synchronous first residual."""
    from warp_gb300 import multigrid
    from warp_gb300.optim import linear

    s = _system((16, 16, 16), sigma=1.0, seed=9)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    solver = linear.RefinedSolver(s.A, M=mg, method="fcg", inner_tol=1e-5)
    x, info = solver.solve(torch.zeros_like(s.b), tol=1e-8)
    assert info["outer"] == 0 and info["inner_iterations"] == 0 and info["converged"]
    assert float(x.abs().max()) == 0.0 and info["history"] == [0.0]
    x, info = solver.solve(s.b, tol=1e-8, max_outer=0)
    assert info["outer"] == 0 and info["rel_residual"] == 1.0 and not info["converged"]
    x, info = solver.solve(s.b, tol=1e-8)
    assert info["converged"] and info["history"][0] == 1.0 and info["rel_residual"] <= 1e-8
    x2, info2 = solver.solve(s.b, x64=x.clone(), tol=1e-8)
    assert info2["converged"] and info2["outer"] == 0
    # the x = 0 start hands b itself to the first correction solve; an explicit zero iterate goes through
    # the product, whose residual b - A 0 rounds to the same b, so both give the same bits
    for m in (solver, linear.RefinedSolver(s.A, method="cg", inner_tol=1e-5)):
        xa, ia = m.solve(s.b, tol=1e-8)
        xb, ib = m.solve(s.b, x64=torch.zeros(s.b.numel(), dtype=torch.float64, device=s.b.device), tol=1e-8)
        assert ia["converged"] and ia["inner_iterations"] == ib["inner_iterations"]
        # ||b|| by two reductions: fp32 products summed in fp64 here, exact products in the residual kernel
        np.testing.assert_allclose(ia["history"], ib["history"], rtol=1e-9)
        assert torch.equal(xa, xb)
    with pytest.raises(ValueError, match="b.shape"):
        solver.solve(s.b[:-1], tol=1e-8)


@pytest.mark.parametrize("m,n", [(37, 300), (700, 2197), (5, 4096)])
def test_dense_mv_matches_fp64(cuda, m, n):
    """gb_dense_mv (the coarsest level's inverse product): one warp per row for short rows, one CTA per row
    for long ones; z = alpha A x + beta y within fp32 summation error, and bitwise the same on a repeat."""
    import warp_gb300._native as N

    g = torch.Generator(device="cuda").manual_seed(m + n)
    Am = torch.randn(m, n, device="cuda", generator=g)
    x = torch.randn(n, device="cuda", generator=g)
    y = torch.randn(m, device="cuda", generator=g)
    z = torch.empty(m, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for alpha, beta in ((1.0, 0.0), (0.5, -2.0)):
        N.check(N.lib().gb_dense_mv(N.GB_F32, m, n, Am.data_ptr(), x.data_ptr(), y.data_ptr(), z.data_ptr(),
                                    alpha, beta, st))
        z1 = z.clone()
        N.check(N.lib().gb_dense_mv(N.GB_F32, m, n, Am.data_ptr(), x.data_ptr(), y.data_ptr(), z.data_ptr(),
                                    alpha, beta, st))
        ref = alpha * (Am.double() @ x.double()) + beta * y.double()
        bound = 1e-5 * (Am.double().abs() @ x.double().abs()) * abs(alpha) + 1e-6 * y.double().abs() * abs(beta)
        assert bool(((z.double() - ref).abs() <= bound + 1e-7).all())
        assert torch.equal(z, z1)
