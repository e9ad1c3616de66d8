"""GPU parity of the solvers: fused BSR path and generic path, against the oracle and FP64 solves."""

import numpy as np
import pytest
import torch

import oracle
from oracle import fem_q1

pytestmark = pytest.mark.gpu


def _spd(n, seed):
    # warp/tests/test_linear_solvers.py:64-81
    rng = np.random.default_rng(seed)
    C = rng.uniform(-100, 100, (n, n))
    f = rng.uniform(-100, 100, n)
    return C @ C.T, C @ f


def _poisson(res, seed=0, coef=None, bs=1):
    """Q1 diffusion matrix + Dirichlet projection (oracle side) -> BSR on the device."""
    from warp_gb300 import sparse

    r, c, v = fem_q1.assemble_triplets(res, coef=coef)
    nn = int(np.prod([k + 1 for k in res]))
    o = oracle.bsr_from_triplets(nn, nn, r, c, v)
    mask = fem_q1.boundary_mask(res)
    off, cols, vals = o["offsets"], o["columns"], o["values"].astype(np.float64)
    rows = np.repeat(np.arange(nn), np.diff(off))
    keep = (1 - mask[rows]) * (1 - mask[cols])
    vals = vals * keep + np.where((rows == cols), mask[rows], 0.0)
    vals = vals.astype(np.float32)
    rng = np.random.default_rng(seed)
    b = fem_q1.assemble_rhs(res, f_nodal=rng.uniform(-1, 1, nn)).astype(np.float32) * (1 - mask)
    A = sparse.bsr_zeros(nn, nn, torch.float32)
    sparse.bsr_set_from_triplets(A, torch.from_numpy(rows.astype(np.int32)).cuda(),
                                 torch.from_numpy(cols.astype(np.int32)).cuda(), torch.from_numpy(vals).cuda(),
                                 prune_numerical_zeros=False)
    A.nnz_sync()
    return A, (off, cols, vals), b


def _true_rel_residual(host, x, b):
    off, cols, vals = host
    r = b.astype(np.float64) - oracle.bsr_mv_f64(off, cols, vals, x.astype(np.float64))
    return np.linalg.norm(r) / np.linalg.norm(b)


@pytest.mark.parametrize("check_every", [10, 0, 1])
@pytest.mark.parametrize("use_graph", [True, False])
def test_cg_fused_poisson(cuda, check_every, use_graph):
    from warp_gb300.optim import linear

    A, host, b = _poisson((24, 20, 16))
    M = linear.preconditioner(A, "diag")
    x = torch.zeros(A.nrow, dtype=torch.float32, device="cuda")
    bd = torch.from_numpy(b).cuda()
    state = linear.cg(A, bd, x, tol=1e-6, maxiter=2000, M=M, check_every=check_every, use_cuda_graph=use_graph,
                      run=False)
    assert state._fused
    out = state()
    if check_every == 0:
        it, rr, atol_sq = (int(out[0].item()), float(out[1].item()), float(out[2].item()))
        err, atol = np.sqrt(rr), np.sqrt(atol_sq)
    else:
        it, err, atol = out
    assert err <= atol
    rel = _true_rel_residual(host, x.cpu().numpy(), b)
    assert rel <= 32 * 1e-6, rel
    # oracle restatement of the same PCG (fp32 vectors): same iteration count within a few
    _, it_ref, err_ref, atol_ref = oracle.pcg_f32(host[0], host[1], host[2], b,
                                                  inv_diag=oracle.inverse_diagonal_f32(*host), tol=1e-6,
                                                  maxiter=2000)
    assert abs(it - it_ref) <= max(3, 0.05 * it_ref), (it, it_ref)


def test_cg_capture_whole_solve_in_user_graph(cuda):
    """check_every=0 inside the caller's own stream capture (reference test_linear_solvers.py:23-36)."""
    from warp_gb300.optim import linear

    A, host, b = _poisson((16, 16, 16), seed=3)
    M = linear.preconditioner(A, "diag")
    x = torch.zeros(A.nrow, dtype=torch.float32, device="cuda")
    bd = torch.from_numpy(b).cuda()
    state = linear.cg(A, bd, x, tol=1e-6, maxiter=1000, M=M, check_every=0, run=False)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            it, rr, atol_sq = state()
    g.replay()
    torch.cuda.synchronize()
    assert float(rr.item()) <= float(atol_sq.item())
    assert _true_rel_residual(host, x.cpu().numpy(), b) <= 32e-6
    # replay again from the converged state (warm start): converges immediately
    g.replay()
    torch.cuda.synchronize()
    assert int(it.item()) <= 2


@pytest.mark.parametrize("left", [False, True])
def test_bicgstab_fused_poisson(cuda, left):
    from warp_gb300.optim import linear

    A, host, b = _poisson((20, 18, 14), seed=5)
    M = linear.preconditioner(A, "diag")
    x = torch.zeros(A.nrow, dtype=torch.float32, device="cuda")
    st = linear.bicgstab(A, torch.from_numpy(b).cuda(), x, tol=1e-6, maxiter=2000, M=M,
                         is_left_preconditioner=left, run=False)
    assert st._fused
    it, err, atol = st()
    assert err <= atol
    assert _true_rel_residual(host, x.cpu().numpy(), b) <= 64e-6


def test_cg_elasticity_3x3(cuda):
    from warp_gb300 import fem, sparse
    from warp_gb300.optim import linear

    res = (8, 6, 5)
    geo = fem.Grid3D(res=res)
    space = fem.make_polynomial_space(geo, degree=1, dtype="vec3")
    lam, mu = fem.q1.lame_from_young(1e3, 0.3)
    K = fem.integrate(fem.linear_elasticity_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                      values={"lame": (float(lam), float(mu))})
    f = fem.integrate(fem.linear_form, fields={"v": fem.make_test(space)}, values={"f": (0.0, -9.81, 0.0)})
    P = fem.integrate(fem.boundary_projector_form, fields={"u": fem.make_trial(space, fem.BoundarySides(geo, ("x-",))),
                                                           "v": fem.make_test(space, fem.BoundarySides(geo, ("x-",)))},
                      assembly="nodal")
    fem.project_linear_system(K, f, P)
    M = linear.preconditioner(K, "diag")
    x = torch.zeros_like(f)
    st = linear.cg(K, f, x, tol=1e-6, maxiter=5000, M=M, run=False)
    assert st._fused
    it, err, atol = st()
    assert err <= atol
    nnz = K.nnz_sync()
    off, cols = K.offsets.cpu().numpy(), K.columns[:nnz].cpu().numpy()
    vals = K.values[:nnz].cpu().numpy()
    r = f.cpu().numpy().astype(np.float64) - oracle.bsr_mv_f64(off, cols, vals, x.cpu().numpy(), block_shape=(3, 3))
    assert np.linalg.norm(r) <= 32 * atol


@pytest.mark.parametrize("solver", ["cg", "bicgstab"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_generic_dense_path(cuda, solver, dtype):
    """Dense SPD systems through the generic LinearOperator path (test_linear_solvers.py:112-130)."""
    from warp_gb300.optim import linear

    n = 64 if dtype == torch.float64 else 16
    Ad, b = _spd(n, 123 if dtype == torch.float64 else 321)
    A = torch.from_numpy(Ad).to(dtype).cuda()
    bd = torch.from_numpy(b).to(dtype).cuda()
    f = linear.cg if solver == "cg" else linear.bicgstab
    for M in (None, linear.preconditioner(A, "diag")):
        x = torch.zeros_like(bd)
        it, err, atol = f(A, bd, x, maxiter=1000, M=M)
        assert err <= atol
        res = np.linalg.norm(Ad @ x.cpu().double().numpy() - b)
        assert res <= (2.0 if dtype == torch.float64 else 32.0) * atol


def test_generic_identity_system(cuda):
    from warp_gb300.optim import linear

    rng = np.random.default_rng(321)
    A = torch.eye(5, dtype=torch.float32, device="cuda")
    b = torch.from_numpy(rng.uniform(-1, 1, 5).astype(np.float32)).cuda()
    x = torch.zeros_like(b)
    it, err, atol = linear.cg(A, b, x, maxiter=30)
    assert err <= atol
    np.testing.assert_allclose(x.cpu().numpy(), b.cpu().numpy(), rtol=1e-6)


def test_refined_solve_reaches_fp64_tolerance(cuda):
    from warp_gb300.optim import linear

    rng = np.random.default_rng(4)
    res = (24, 24, 24)
    coef = np.exp(rng.standard_normal(int(np.prod(res))) * 1.0)
    A, host, b = _poisson(res, seed=9, coef=coef)
    M = linear.preconditioner(A, "diag")
    x64, info = linear.solve_refined(A, torch.from_numpy(b).cuda(), tol=1e-8, M=M, inner_tol=1e-4)
    assert info["converged"], info
    rel = _true_rel_residual(host, x64.cpu().numpy(), b)
    assert rel <= 1e-8, rel
    # the FP64 solution agrees with a direct FP64 solve of the same (fp32-valued) system
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    off, cols, vals = host
    S = sp.csr_matrix((vals.astype(np.float64), cols, off), shape=(A.nrow, A.nrow))
    xd = spla.spsolve(S.tocsc(), b.astype(np.float64))
    assert np.linalg.norm(x64.cpu().numpy() - xd) <= 1e-6 * np.linalg.norm(xd)


def test_nonfinite_rhs_reports_status(cuda):
    """Failure detection without a GPU fault: a NaN in b stops the loop and sets a status bit."""
    import warp_gb300._native as N
    from warp_gb300.optim import linear

    A, host, b = _poisson((8, 8, 8))
    b = b.copy()
    b[5] = np.nan
    x = torch.zeros(A.nrow, dtype=torch.float32, device="cuda")
    st = linear.cg(A, torch.from_numpy(b).cuda(), x, maxiter=100, M=linear.preconditioner(A, "diag"), run=False)
    it, err, atol = st()
    assert it == 0
    assert st.last_status & N.DEV_NONFINITE
