"""The persistent CG (whole iteration loop in one cooperative launch) against the three-kernel
iteration and the oracle: iteration counts, solutions, chunked / eager / captured modes, status."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _host_csr(A):
    nnz = A.nnz_sync()
    off = A.offsets.cpu().numpy()
    cols = A.columns[:nnz].cpu().numpy()
    vals = A.values[:nnz].float().cpu().numpy().astype(np.float64)
    return off, cols, vals


def _rel_residual(A, x, b):
    off, cols, vals = _host_csr(A)
    bs = A.block_shape[0]
    if bs == 1:
        Ax = oracle.bsr_mv_f64(off, cols, vals, x.astype(np.float64))
    else:
        import scipy.sparse as sp

        S = sp.bsr_matrix((vals.reshape(-1, bs, bs), cols, off), shape=(A.nrow * bs, A.ncol * bs))
        Ax = S @ x.astype(np.float64)
    r = b.astype(np.float64) - Ax
    return np.linalg.norm(r) / np.linalg.norm(b)


def _solve(A, b, persistent, tol=1e-6, maxiter=4000, check_every=0, use_graph=True):
    from warp_gb300.optim import linear

    M = linear.preconditioner(A, "diag")
    x = torch.zeros_like(b)
    st = linear.CG(A, b, x, tol=tol, atol=0.0, maxiter=maxiter, M=M, check_every=check_every,
                   use_cuda_graph=use_graph, persistent=persistent)
    out = st()
    torch.cuda.synchronize()
    if check_every == 0:
        it = int(out[0].item())
        err, atol = float(out[1].item()) ** 0.5, float(out[2].item()) ** 0.5
        status = int(st._dev_status.item())
    else:
        it, err, atol = out
        status = st.last_status
    return st, x, it, err, atol, status


@pytest.mark.parametrize("case", ["diffusion32", "diffusion48_lognormal", "elasticity12", "elasticity12_bf16"])
def test_persistent_matches_three_kernel_iteration(cuda, case):
    from warp_gb300 import problems, sparse

    if case.startswith("diffusion"):
        res = 32 if case == "diffusion32" else 48
        sysm = problems.diffusion((res, res, res), sigma=0.0 if res == 32 else 1.5, corr_length=0.1, seed=2,
                                  lognormal=res != 32)
    else:
        sysm = problems.elasticity((12, 12, 12), sigma=1.0, seed=4)
    A = sysm.A
    if case.endswith("bf16"):
        A = sparse.bsr_copy(A, scalar_type=torch.bfloat16)
    b = sysm.b.reshape(-1).contiguous()
    st_p, x_p, it_p, err_p, atol_p, status_p = _solve(A, b, persistent=True)
    st_k, x_k, it_k, err_k, atol_k, status_k = _solve(A, b, persistent=False)
    assert st_p.persistent_active and not st_k.persistent_active
    assert status_p == 0 and status_k == 0
    assert err_p <= atol_p and err_k <= atol_k
    # same arithmetic per iteration; only the order of the partial sums differs
    assert abs(it_p - it_k) <= max(2, 0.01 * it_k), (it_p, it_k)
    bn = b.cpu().numpy()
    rp = _rel_residual(A, x_p.cpu().numpy(), bn)
    rk = _rel_residual(A, x_k.cpu().numpy(), bn)
    # the recurrence residual of fp32 CG drifts from the true one on the ill-conditioned elasticity
    # systems (both paths alike): the persistent path must do as well as the three-kernel one
    assert rp <= max(32e-6, 3.0 * rk), (rp, rk)
    if A.nrow * A.block_shape[0] > 40000:
        return
    # both against an FP64 direct solve of the same (fp32 / bf16-valued) system
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    off, cols, vals = _host_csr(A)
    bs = A.block_shape[0]
    S = sp.bsr_matrix((vals.reshape(-1, bs, bs), cols, off), shape=(A.nrow * bs, A.ncol * bs)).tocsc()
    xd = spla.spsolve(S, bn.astype(np.float64))
    ep = np.linalg.norm(x_p.cpu().numpy() - xd)
    ek = np.linalg.norm(x_k.cpu().numpy() - xd)
    assert ep <= max(2.0 * ek, 1e-5 * np.linalg.norm(xd)), (ep, ek)


def test_persistent_iterations_match_oracle_pcg(cuda):
    """Iteration count and solution of the persistent launch against the oracle's fp32 restatement of
    CG._run (warp/_src/optim/linear.py:934-1032) on the same system."""
    from warp_gb300 import problems

    sysm = problems.diffusion((24, 20, 16), sigma=1.5, corr_length=0.2, seed=9)
    A, b = sysm.A, sysm.b.reshape(-1).contiguous()
    st, x, it, err, atol, status = _solve(A, b, persistent=True, check_every=10)
    assert st.persistent_active and status == 0
    off, cols, vals = _host_csr(A)
    vals32 = vals.astype(np.float32)
    xo, it_o, err_o, atol_o = oracle.pcg_f32(off, cols, vals32, b.cpu().numpy(),
                                             inv_diag=oracle.inverse_diagonal_f32(off, cols, vals32), tol=1e-6,
                                             atol=0.0, maxiter=4000)
    assert abs(it - it_o) <= max(3, 0.05 * it_o), (it, it_o)
    np.testing.assert_allclose(x.cpu().numpy(), xo, rtol=0, atol=2e-3 * np.abs(xo).max())


@pytest.mark.parametrize("check_every,use_graph", [(7, True), (7, False), (0, False)])
def test_persistent_chunked_and_eager_modes(cuda, check_every, use_graph):
    """Chunks of `check_every` iterations (one cooperative launch each, cached in a graph or eager)
    and one launch per iteration reach the same iterate as the whole-solve launch."""
    from warp_gb300 import problems

    sysm = problems.diffusion((20, 20, 20), sigma=1.0, corr_length=0.2, seed=5)
    A, b = sysm.A, sysm.b.reshape(-1).contiguous()
    _, x0, it0, _, _, s0 = _solve(A, b, persistent=True)
    st, x1, it1, err1, atol1, s1 = _solve(A, b, persistent=True, check_every=check_every, use_graph=use_graph)
    assert st.persistent_active and s0 == 0 and s1 == 0
    assert err1 <= atol1
    assert it1 == it0
    torch.testing.assert_close(x1, x0, rtol=0, atol=0)


def test_persistent_capture_in_user_graph(cuda):
    """check_every=0 inside the caller's stream capture: the init kernel and the cooperative loop
    launch become nodes of the caller's graph; replays solve from scratch and from the converged state."""
    from warp_gb300 import problems
    from warp_gb300.optim import linear

    sysm = problems.diffusion((16, 16, 16), sigma=1.0, corr_length=0.2, seed=3)
    A, b = sysm.A, sysm.b.reshape(-1).contiguous()
    x = torch.zeros_like(b)
    st = linear.CG(A, b, x, tol=1e-6, atol=0.0, maxiter=1000, M=linear.preconditioner(A, "diag"), check_every=0)
    assert st.persistent_active
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            it, rr, atol_sq = st()
    g.replay()
    torch.cuda.synchronize()
    assert float(rr.item()) <= float(atol_sq.item())
    assert _rel_residual(A, x.cpu().numpy(), b.cpu().numpy()) <= 32e-6
    n_first = int(it.item())
    assert n_first > 5
    g.replay()  # warm start from the converged x
    torch.cuda.synchronize()
    assert int(it.item()) <= 2


def test_persistent_nonfinite_rhs_stops_with_status(cuda):
    """A NaN in b stops the persistent loop with GB_DEV_NONFINITE and no wait timeout."""
    import warp_gb300._native as N
    from warp_gb300 import problems

    sysm = problems.diffusion((10, 10, 10), sigma=0.0, seed=1, lognormal=False)
    b = sysm.b.reshape(-1).clone()
    b[17] = float("nan")
    st, x, it, err, atol, status = _solve(sysm.A, b, persistent=True, check_every=5)
    assert st.persistent_active
    assert it == 0
    assert status & N.DEV_NONFINITE
    assert not status & N.DEV_WAIT_TIMEOUT


@pytest.mark.parametrize("persistent", [True, False])
def test_breakdown_inside_the_loop_stops_it(cuda, persistent):
    """A NaN in the Jacobi preconditioner's inverse diagonal reaches the first p.Ap inside the loop:
    alpha is not finite, GB_DEV_BREAKDOWN is set and the loop ends after that iteration (every CTA of
    the persistent launch takes the same decision; no barrier waits run out)."""
    import warp_gb300._native as N
    from warp_gb300 import problems
    from warp_gb300.optim import linear

    sysm = problems.diffusion((10, 10, 10), sigma=0.0, seed=1, lognormal=False)
    A, b = sysm.A, sysm.b.reshape(-1).contiguous()
    M = linear.preconditioner(A, "diag")
    M._inv_diag[500] = float("nan")
    x = torch.zeros_like(b)
    st = linear.CG(A, b, x, tol=1e-6, atol=0.0, maxiter=200, M=M, check_every=0, persistent=persistent)
    assert st.persistent_active == persistent
    it, rr, atol_sq = st()
    torch.cuda.synchronize()
    status = int(st._dev_status.item())
    assert status & N.DEV_BREAKDOWN
    assert not status & N.DEV_WAIT_TIMEOUT
    assert int(it.item()) == 1


def test_persistent_solves_are_reproducible(cuda):
    """Several tiles per CTA, taken from the dynamic queues in a different order each run: repeated solves
    give the same iterate bit for bit (the schedule only reaches p.Ap at double-float rounding level)."""
    from warp_gb300 import problems

    sysm = problems.diffusion((48, 48, 48), sigma=1.5, corr_length=0.1, seed=4)
    A, b = sysm.A, sysm.b.reshape(-1).contiguous()
    _, x0, it0, _, _, s0 = _solve(A, b, persistent=True)
    for _ in range(2):
        st, x1, it1, _, _, s1 = _solve(A, b, persistent=True)
        assert st.persistent_active and s0 == 0 and s1 == 0
        assert it1 == it0
        assert torch.equal(x1, x0)
