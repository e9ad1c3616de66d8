"""GPU tests of the multigrid hierarchy on Q1 vec3 linear elasticity (3x3 blocks): component-wise
transfers equal the scalar transfers applied per component, the V-cycle is symmetric, and flexible CG
with it reaches the FP64 target in far fewer inner iterations than the Jacobi-CG drop-in (with fp32
and with bf16 inner matrix values)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FACES = ("x-",)  # the elasticity problems clamp the x = 0 face only


def _elasticity(res, seed=1, sigma=1.0):
    from warp_gb300 import problems

    return problems.elasticity((res,) * 3, sigma=sigma, seed=seed)


def test_vector_transfers_equal_scalar_transfers_per_component(cuda):
    import warp_gb300._native as N
    from warp_gb300 import multigrid

    s = _elasticity(8)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef, faces=FACES, coarsest_nodes=400)  # two levels
    f, c = mg.levels[0], mg.levels[1]
    L = N.lib()
    st = torch.cuda.current_stream().cuda_stream
    g = torch.Generator("cuda").manual_seed(3)
    t = torch.randn(f.n * 3, device="cuda", generator=g)
    zc = torch.randn(c.n * 3, device="cuda", generator=g)
    rc = torch.zeros(c.n * 3, device="cuda")
    pz = torch.randn(f.n * 3, device="cuda", generator=g)
    pz0 = pz.clone()
    N.check(L.gb_mg_restrict_c(3, *f.dims, *c.dims, t.data_ptr(), f.mask.data_ptr(), c.mask.data_ptr(), rc.data_ptr(),
                               st))
    N.check(L.gb_mg_prolong_add_c(3, *f.dims, *c.dims, zc.data_ptr(), f.mask.data_ptr(), 0.7, pz.data_ptr(), st))
    for comp in range(3):
        tk = t[comp::3].contiguous()
        rk = torch.zeros(c.n, device="cuda")
        N.check(L.gb_mg_restrict(*f.dims, *c.dims, tk.data_ptr(), f.mask.data_ptr(), c.mask.data_ptr(), rk.data_ptr(),
                                 st))
        assert torch.equal(rk, rc[comp::3])
        zk = zc[comp::3].contiguous()
        pk = pz0[comp::3].contiguous()
        N.check(L.gb_mg_prolong_add(*f.dims, *c.dims, zk.data_ptr(), f.mask.data_ptr(), 0.7, pk.data_ptr(), st))
        assert torch.equal(pk, pz[comp::3])


def test_elasticity_hierarchy_and_symmetric_vcycle(cuda):
    from warp_gb300 import multigrid

    s = _elasticity(16, seed=2)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef, faces=FACES, coarsest_nodes=400)  # three levels
    assert mg.bdim == 3 and mg.n == s.A.nrow * 3
    assert [lv.dims for lv in mg.levels] == [(17,) * 3, (9,) * 3, (5,) * 3]
    assert all(lv.A.block_shape == (3, 3) for lv in mg.levels)
    m = (1 - mg.levels[0].mask).repeat_interleave(3)
    g = torch.Generator("cuda").manual_seed(4)
    r1 = torch.randn(mg.n, device="cuda", generator=g) * m
    r2 = torch.randn(mg.n, device="cuda", generator=g) * m
    z1, z2 = mg.apply(r1), mg.apply(r2).clone()
    torch.cuda.synchronize()
    assert int(mg.status.item()) == 0
    a = float(torch.dot(r2.double(), z1.double()))
    b = float(torch.dot(r1.double(), z2.double()))
    assert abs(a - b) <= 1e-4 * (abs(a) + abs(b)), (a, b)
    assert float(torch.dot(r1.double(), z1.double())) > 0
    with pytest.raises(ValueError):
        from warp_gb300 import learned

        learned.LearnedSmoother(learned.ConvNet(seed=0), mg, s.coef)


@pytest.mark.parametrize("values", ["fp32", "bf16"])
def test_elasticity_mg_fcg_beats_jacobi_cg(cuda, values):
    from warp_gb300 import multigrid
    from warp_gb300.optim import linear

    s = _elasticity(16, seed=5, sigma=1.0)
    A = s.A
    nnz = A.nnz_sync()
    inner = A.values[:nnz].to(torch.bfloat16).contiguous() if values == "bf16" else None
    mg = multigrid.MultigridPreconditioner(A, s.geo, s.coef, faces=FACES)
    fsolver = linear.RefinedSolver(A, M=mg, method="fcg", inner_tol=1e-5, inner_values=inner)
    x, info = fsolver.solve(s.b, tol=1e-8)
    assert info["converged"] and info["rel_residual"] <= 1e-8
    # the FP64 residual, recomputed on the host (scipy BSR product of the same matrix)
    sp = pytest.importorskip("scipy.sparse")
    n = A.nrow * 3
    Ah = sp.bsr_matrix((A.values[:nnz].cpu().numpy().astype(np.float64).reshape(-1, 3, 3),
                        A.columns[:nnz].cpu().numpy(), A.offsets.cpu().numpy()), shape=(n, n))
    bd = s.b.cpu().numpy().astype(np.float64)
    res = np.linalg.norm(bd - Ah @ x.cpu().numpy()) / np.linalg.norm(bd)
    assert res <= 2e-8, res
    jsolver = linear.RefinedSolver(A, M=linear.preconditioner(A, "diag"), inner_tol=1e-5, inner_values=inner)
    _, jinfo = jsolver.solve(s.b, tol=1e-8)
    assert jinfo["converged"]
    assert info["inner_iterations"] * 5 < jinfo["inner_iterations"], (info, jinfo)


def test_refined_solver_stops_when_reduced_precision_corrections_diverge(cuda):
    """bf16 inner values on a rough lognormal field (sigma 1.5, correlation length 0.05) make the inner
    operator indefinite at its smallest eigenvalues: the outer residual grows, and the refined solve
    stops (the first correction makes the true residual over 100x worse) and reports non-convergence
    instead of running its outer steps out."""
    from warp_gb300 import multigrid
    from warp_gb300.optim import linear

    from warp_gb300 import problems

    s = problems.elasticity((64,) * 3, sigma=1.5, corr_length=0.05, seed=0)
    A = s.A
    nnz = A.nnz_sync()
    mg = multigrid.MultigridPreconditioner(A, s.geo, s.coef, faces=FACES)
    sol = linear.RefinedSolver(A, M=mg, method="fcg", inner_tol=1e-5, inner_maxiter=3000,
                               inner_values=A.values[:nnz].to(torch.bfloat16).contiguous())
    _, info = sol.solve(s.b, tol=1e-8)
    assert not info["converged"] and info["diverged"] and info["outer"] <= 2, info["history"]
    # the iterate returned is the last accepted one, not the one a diverging correction made
    assert info["rel_residual"] <= info["history"][0] * (1 + 1e-9), info["history"]
    # the same solve with FP32 inner values converges
    sol32 = linear.RefinedSolver(A, M=mg, method="fcg", inner_tol=1e-5, inner_maxiter=3000)
    x32, info32 = sol32.solve(s.b, tol=1e-8)
    assert info32["converged"] and info32["rel_residual"] <= 1e-8 and not info32["diverged"]
    # warm start from a good solution: the bf16 corrections cannot improve it; the solve must stop
    # without running its outer steps out and hand back an iterate no worse than the start
    x0 = x32.clone()
    xw, infow = sol.solve(s.b, x64=x0, tol=1e-12, max_outer=50)
    assert not infow["converged"] and infow["outer"] < 10, infow["history"]
    assert infow["rel_residual"] <= infow["history"][0] * (1 + 1e-6) or infow["rel_residual"] <= 1e-8, \
        infow["history"]


def test_bf16_values_inside_the_vcycle_converge_on_the_rough_field(cuda):
    """bf16 matrix values inside the V-cycle only (the flexible solver's product keeps fp32): on the
    rough field where bf16 inner operators make the refinement diverge, the solve still reaches the
    FP64 target, checked on the host, with close to the fp32 cycle's iteration count."""
    from warp_gb300 import multigrid, problems
    from warp_gb300.optim import linear

    s = problems.elasticity((32,) * 3, sigma=1.5, corr_length=0.05, seed=0)
    A = s.A
    nnz = A.nnz_sync()
    mg32 = multigrid.MultigridPreconditioner(A, s.geo, s.coef, faces=FACES)
    mg16 = multigrid.MultigridPreconditioner(A, s.geo, s.coef, faces=FACES, fine_values=torch.bfloat16)
    assert mg16.levels[0].vals.dtype == torch.bfloat16 and mg16.levels[1].vals.dtype == torch.float32
    x32, i32 = linear.RefinedSolver(A, M=mg32, method="fcg", inner_maxiter=3000).solve(s.b, tol=1e-8)
    x16, i16 = linear.RefinedSolver(A, M=mg16, method="fcg", inner_maxiter=3000).solve(s.b, tol=1e-8)
    assert i32["converged"] and i16["converged"], (i32, i16)
    assert i16["inner_iterations"] <= 1.5 * i32["inner_iterations"] + 5, (i16, i32)
    sp = pytest.importorskip("scipy.sparse")
    n = A.nrow * 3
    Ah = sp.bsr_matrix((A.values[:nnz].cpu().numpy().astype(np.float64).reshape(-1, 3, 3),
                        A.columns[:nnz].cpu().numpy(), A.offsets.cpu().numpy()), shape=(n, n))
    bd = s.b.cpu().numpy().astype(np.float64)
    res = np.linalg.norm(bd - Ah @ x16.cpu().numpy()) / np.linalg.norm(bd)
    assert res <= 2e-8, res
    assert int(mg16.status.item()) == 0


def test_trained_3_channel_smoother_solves_elasticity(cuda):
    """The committed 3-channel network (vec3 fields, tcgen05 layers) inside the vec3 V-cycle: flexible CG
    with FP64 refinement reaches 1e-8 on a rough elasticity field without falling back to Jacobi-CG."""
    from warp_gb300 import learned, multigrid, problems
    from warp_gb300.optim import linear

    net = learned.ConvNet.load(learned.ELASTICITY_WEIGHTS)
    assert net.ncomp == 3 and net.layers[-1][1] == 3
    s = problems.elasticity((32,) * 3, sigma=1.5, corr_length=0.05 * 128 / 32, seed=1)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef, faces=FACES, fine_values=torch.bfloat16)
    mg.smoother = learned.LearnedSmoother(net, mg, s.coef)
    solver = linear.RefinedSolver(s.A, M=mg, method="fcg", inner_maxiter=3000)
    x, info = solver.solve(s.b, tol=1e-8)
    assert info["converged"] and solver.fallbacks == 0, info
    nnz = s.A.nnz_sync()
    sp = pytest.importorskip("scipy.sparse")
    n = s.A.nrow * 3
    Ah = sp.bsr_matrix((s.A.values[:nnz].cpu().numpy().astype(np.float64).reshape(-1, 3, 3),
                        s.A.columns[:nnz].cpu().numpy(), s.A.offsets.cpu().numpy()), shape=(n, n))
    bd = s.b.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(bd - Ah @ x.cpu().numpy()) / np.linalg.norm(bd) <= 2e-8
    assert int(mg.status.item()) == 0


@pytest.mark.parametrize("values", ["fp32", "bf16"])
def test_block_jacobi_kernels_match_fp64(cuda, values):
    """Block-Jacobi pieces of the vec3 smoother against float64: the 3x3 diagonal-block inverses, the first
    step omega Dinv r and the fused step z + omega Dinv (r - A z) (fp32 or bf16 matrix values)."""
    import warp_gb300._native as N

    s = _elasticity(5, seed=4, sigma=1.0)
    A = s.A
    L = N.lib()
    st = torch.cuda.current_stream().cuda_stream
    n = A.nrow
    dense = A.numpy_dense()
    inv = torch.empty(n * 9, device="cuda")
    N.check(L.gb_bsr_block_inverse_diagonal3(n, A.offsets.data_ptr(), None, A.columns.data_ptr(),
                                             A.values.data_ptr(), inv.data_ptr(), st))
    blocks = np.stack([dense[3 * i:3 * i + 3, 3 * i:3 * i + 3] for i in range(n)])
    ref_inv = np.linalg.inv(blocks)
    got_inv = inv.cpu().numpy().astype(np.float64).reshape(n, 3, 3)
    assert np.abs(got_inv - ref_inv).max() <= 1e-5 * np.abs(ref_inv).max()
    g = torch.Generator(device="cuda").manual_seed(5)
    r = torch.randn(3 * n, device="cuda", generator=g)
    z = torch.randn(3 * n, device="cuda", generator=g)
    w = torch.empty_like(r)
    omega = 0.45
    N.check(L.gb_mg_block_jacobi0(n, omega, inv.data_ptr(), r.data_ptr(), w.data_ptr(), st))
    rr, zz = r.double().cpu().numpy(), z.double().cpu().numpy()
    ref_w = omega * np.einsum("nij,nj->ni", got_inv, rr.reshape(n, 3)).reshape(-1)
    assert np.abs(w.double().cpu().numpy() - ref_w).max() <= 1e-5 * np.abs(ref_w).max()
    vals = A.values if values == "fp32" else A.values.to(torch.bfloat16)
    dense_v = dense if values == "fp32" else _bf16_dense(A)
    out = torch.empty_like(r)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(L.gb_bsr_block_jacobi_smooth3(n, A.nnz_sync(), A.nnz_sync(), A.offsets.data_ptr(), A.columns.data_ptr(),
                                          vals.data_ptr(), N.GB_F32 if values == "fp32" else N.GB_BF16, r.data_ptr(),
                                          z.data_ptr(), inv.data_ptr(), omega, out.data_ptr(), status.data_ptr(), st))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    res = rr - dense_v @ zz
    ref = zz + omega * np.einsum("nij,nj->ni", got_inv, res.reshape(n, 3)).reshape(-1)
    scale = np.abs(zz).max() + omega * np.abs(got_inv).max() * (np.abs(dense_v) @ np.abs(zz) + np.abs(rr)).max()
    assert np.abs(out.double().cpu().numpy() - ref).max() <= 1e-5 * scale


def _bf16_dense(A):
    """The dense matrix of A's values rounded to bf16 (the values the bf16 kernels read)."""
    nnz = A.nnz_sync()
    off = A.offsets.cpu().numpy()
    cols = A.columns[:nnz].cpu().numpy()
    vals = A.values[:nnz].to(torch.bfloat16).double().cpu().numpy().reshape(-1, 3, 3)
    D = np.zeros((3 * A.nrow, 3 * A.ncol))
    for i in range(A.nrow):
        for k in range(off[i], off[i + 1]):
            D[3 * i:3 * i + 3, 3 * cols[k]:3 * cols[k] + 3] = vals[k]
    return D
