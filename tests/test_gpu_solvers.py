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
    """Fused graph CG vs the oracle's restatement of CG._run on the same system."""
    from warp_gb300.optim import linear

    A, host, b = _poisson((24, 20, 16))
    M = linear.preconditioner(A, "diag")
    x = torch.zeros(A.nrow, dtype=torch.float32, device="cuda")
    bd = torch.from_numpy(b).cuda()
    # atol=0: purely relative stopping rule (with atol=None the reference sets atol=tol, an absolute
    # floor that dominates for this small-norm right-hand side)
    state = linear.cg(A, bd, x, tol=1e-6, atol=0.0, maxiter=2000, M=M, check_every=check_every,
                      use_cuda_graph=use_graph, run=False)
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
                                                  inv_diag=oracle.inverse_diagonal_f32(*host), tol=1e-6, atol=0.0,
                                                  maxiter=2000)
    assert abs(it - it_ref) <= max(3, 0.05 * it_ref), (it, it_ref)


def test_cg_tolerance_rule_matches_reference(cuda):
    """tol only -> atol = tol (absolute floor), as _get_tolerances (linear.py:2018-2032); the fused
    solver stops exactly where the oracle restatement stops."""
    from warp_gb300.optim import linear

    A, host, b = _poisson((24, 20, 16))
    x = torch.zeros(A.nrow, dtype=torch.float32, device="cuda")
    it, err, atol = linear.cg(A, torch.from_numpy(b).cuda(), x, tol=1e-6, maxiter=2000,
                              M=linear.preconditioner(A, "diag"), check_every=1)
    xo, it_o, err_o, atol_o = oracle.pcg_f32(host[0], host[1], host[2], b, inv_diag=oracle.inverse_diagonal_f32(*host),
                                             tol=1e-6, maxiter=2000)
    assert atol == pytest.approx(1e-6) and atol_o == pytest.approx(1e-6)
    assert abs(it - it_o) <= 1
    np.testing.assert_allclose(x.cpu().numpy(), xo, rtol=1e-3, atol=1e-4 * np.abs(xo).max())


def test_cg_capture_whole_solve_in_user_graph(cuda):
    """check_every=0 inside the caller's own stream capture (reference test_linear_solvers.py:23-36)."""
    from warp_gb300.optim import linear

    A, host, b = _poisson((16, 16, 16), seed=3)
    M = linear.preconditioner(A, "diag")
    x = torch.zeros(A.nrow, dtype=torch.float32, device="cuda")
    bd = torch.from_numpy(b).cuda()
    state = linear.cg(A, bd, x, tol=1e-6, atol=0.0, maxiter=1000, M=M, check_every=0, run=False)
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
    st = linear.bicgstab(A, torch.from_numpy(b).cuda(), x, tol=1e-6, atol=0.0, maxiter=2000, M=M,
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


@pytest.mark.parametrize("bs", [1, 3])
def test_residual_double_float_vs_fp64_oracle(cuda, bs):
    """The refinement residual in double-float arithmetic matches the FP64 oracle to ~1e-12 of sum|A||x|."""
    import warp_gb300._native as N
    from warp_gb300 import sparse

    rng = np.random.default_rng(bs)
    nrow, n = 4000, 60000
    rows = rng.integers(0, nrow, n).astype(np.int32)
    cols = rng.integers(0, nrow, n).astype(np.int32)
    vals = rng.standard_normal((n, bs, bs)).astype(np.float32)
    A = sparse.bsr_zeros(nrow, nrow, torch.float32 if bs == 1 else ((3, 3), torch.float32))
    sparse.bsr_set_from_triplets(A, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(),
                                 torch.from_numpy(vals.reshape(n) if bs == 1 else vals).cuda())
    nnz = A.nnz_sync()
    x = rng.standard_normal(nrow * bs)
    b = rng.standard_normal(nrow * bs).astype(np.float32)
    x64 = torch.from_numpy(x).cuda()
    x2 = torch.zeros(2 * nrow * bs, dtype=torch.float32, device="cuda")
    N.check(N.lib().gb_update_solution(nrow * bs, x64.data_ptr(), x2.data_ptr(), None, 0.0,
                                       torch.cuda.current_stream().cuda_stream))
    ws = torch.zeros(int(N.lib().gb_residual_f64_workspace_bytes(bs, nrow, nnz, 0)), dtype=torch.uint8, device="cuda")
    norms = torch.zeros(2, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    off = A.offsets.cpu().numpy()
    cs = A.columns[:nnz].cpu().numpy()
    vs = A.values[:nnz].cpu().numpy()
    exp = b.astype(np.float64) - oracle.bsr_mv_f64(off, cs, vs, x, block_shape=(bs, bs))
    scale = oracle.bsr_abs_mv_f64(off, cs, vs, x, block_shape=(bs, bs)) + np.abs(b)
    for fn, xin in (("gb_residual_df", x2), ("gb_residual_f64", x64)):
        r64 = torch.zeros(nrow * bs, dtype=torch.float64, device="cuda")
        N.check(getattr(N.lib(), fn)(bs, nrow, nnz, A.capacity, A.offsets.data_ptr(), None, A.columns.data_ptr(),
                                     A.values.data_ptr(), N.GB_F32, xin.data_ptr(), torch.from_numpy(b).cuda().data_ptr(),
                                     r64.data_ptr(), None, norms.data_ptr(), ws.data_ptr(), ws.numel(),
                                     status.data_ptr(), torch.cuda.current_stream().cuda_stream))
        err = np.abs(r64.cpu().numpy() - exp)
        assert np.all(err <= 1e-12 * scale), (fn, float((err / scale).max()))
        np.testing.assert_allclose(norms[0].item(), np.dot(exp, exp), rtol=1e-5)
    assert int(status.item()) == 0
