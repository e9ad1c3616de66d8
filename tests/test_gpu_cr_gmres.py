"""GPU tests of the Conjugate Residual and restarted GMRES drop-ins against the float64 restatements
of the reference iterations (oracle.krylov) and the reference's test cases
(warp/tests/test_linear_solvers.py:350-415, restated)."""

import numpy as np
import pytest
import torch

from oracle import krylov

pytestmark = pytest.mark.gpu


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    Q = rng.standard_normal((n, n))
    return (Q @ Q.T + n * np.eye(n)).astype(np.float32), rng.standard_normal(n).astype(np.float32)


def _nonsym(n, seed):
    rng = np.random.default_rng(seed)
    return (4 * np.eye(n) + 0.3 * rng.standard_normal((n, n))).astype(np.float32), rng.standard_normal(n).astype(np.float32)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("precond", [False, True])
def test_cr_dense_spd_matches_restatement(cuda, precond):
    from warp_gb300.optim import linear

    Ad, bd = _spd(60, 1)
    A_, b = _dev(Ad), _dev(bd)
    M = _dev(1.0 / np.diag(Ad)) if precond else None
    x = torch.zeros_like(b)
    it, err, atol = linear.cr(A_, b, x, tol=1e-5, atol=0.0, maxiter=500, M=M, check_every=1)
    assert err <= atol
    res = np.linalg.norm(Ad.astype(np.float64) @ x.cpu().numpy() - bd)
    assert res <= 32 * 1e-5 * np.linalg.norm(bd)
    _, it_ref, _ = krylov.cr(Ad, bd, dinv=(1.0 / np.diag(Ad)) if precond else None, tol=1e-5, atol=0.0, maxiter=500)
    assert abs(it - it_ref) <= 3, (it, it_ref)


def test_cr_on_q1_bsr_with_jacobi(cuda):
    from warp_gb300 import problems
    from warp_gb300.optim import linear

    s = problems.diffusion((24, 24), sigma=1.0, corr_length=0.2, seed=2)
    x = torch.zeros_like(s.b)
    M = linear.preconditioner(s.A, "diag")
    it, err, atol = linear.cr(s.A, s.b, x, tol=1e-5, atol=0.0, maxiter=2000, M=M)
    assert err <= atol and it > 0
    Ad = s.A.numpy_dense()
    bd = s.b.cpu().numpy().astype(np.float64)
    _, it_ref, _ = krylov.cr(Ad, bd, dinv=1.0 / np.diag(Ad), tol=1e-5, atol=0.0, maxiter=2000)
    assert abs(it - it_ref) <= max(3, it_ref // 10), (it, it_ref)
    # check_every = 0: device arrays, no host synchronisation required
    x.zero_()
    it_d, rr_d, atol_sq_d = linear.cr(s.A, s.b, x, tol=1e-5, atol=0.0, maxiter=2000, M=M, check_every=0)
    assert float(rr_d[0]) <= float(atol_sq_d[0])


@pytest.mark.parametrize("mode", ["none", "right", "left"])
def test_gmres_nonsymmetric_matches_restatement(cuda, mode):
    from warp_gb300.optim import linear

    Ad, bd = _nonsym(80, 3)
    A_, b = _dev(Ad), _dev(bd)
    dinv = 1.0 / np.diag(Ad)
    M = None if mode == "none" else _dev(dinv)
    x = torch.zeros_like(b)
    it, err, atol = linear.gmres(A_, b, x, tol=1e-6, atol=0.0, restart=10, maxiter=400, M=M,
                                 is_left_preconditioner=(mode == "left"))
    assert err <= atol and it % 10 == 0
    xr, it_ref, _ = krylov.gmres(Ad, bd, dinv=None if mode == "none" else dinv, tol=1e-6, atol=0.0, restart=10,
                                 maxiter=400, left=(mode == "left"))
    assert abs(it - it_ref) <= 10, (it, it_ref)  # fp32 vectors may need one more cycle than float64
    np.testing.assert_allclose(x.cpu().numpy(), xr, rtol=1e-4, atol=1e-5 * np.abs(xr).max())


def test_gmres_identity_system_one_cycle(cuda):
    """Restates the reference's identity-system GMRES case: converges in the first cycle."""
    from warp_gb300.optim import linear

    rng = np.random.default_rng(123)
    b = _dev(rng.standard_normal(5).astype(np.float32))
    A_ = torch.eye(5, device="cuda")
    x = torch.zeros_like(b)
    it, err, atol = linear.gmres(A_, b, x, maxiter=120)
    assert err <= atol and it == 31  # one cycle of restart = min(31, maxiter); Arnoldi breaks down after 5 steps
    np.testing.assert_allclose(x.cpu().numpy(), b.cpu().numpy(), rtol=1e-6)


def test_gmres_on_bsr_matrix(cuda):
    """Nonsymmetric sparse operator (BSR from triplets) with Jacobi, right-preconditioned GMRES(20)."""
    from warp_gb300 import sparse
    from warp_gb300.optim import linear

    rng = np.random.default_rng(7)
    n = 300
    rows = np.concatenate([np.arange(n), rng.integers(0, n, 3000)]).astype(np.int32)
    cols = np.concatenate([np.arange(n), rng.integers(0, n, 3000)]).astype(np.int32)
    vals = np.concatenate([np.full(n, 8.0), rng.standard_normal(3000) * 0.5]).astype(np.float32)
    A_ = sparse.bsr_zeros(n, n, torch.float32)
    sparse.bsr_set_from_triplets(A_, _dev(rows), _dev(cols), _dev(vals))
    b = _dev(rng.standard_normal(n).astype(np.float32))
    x = torch.zeros_like(b)
    it, err, atol = linear.gmres(A_, b, x, tol=1e-6, atol=0.0, restart=20, maxiter=600,
                                 M=linear.preconditioner(A_, "diag"))
    assert err <= atol
    Ad = A_.numpy_dense()
    assert np.linalg.norm(Ad @ x.cpu().numpy() - b.cpu().numpy()) <= 32 * 1e-6 * float(b.norm())
