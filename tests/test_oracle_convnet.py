"""CPU checks of the conv-net oracle against an independent implementation (torch CPU conv3d +
autograd, float64), and of its V-cycle chain gradient against finite differences."""

import numpy as np
import pytest
import torch

from oracle import convnet as C


def _torch_w(W):  # [27, ci, co] -> [co, ci, 3, 3, 3] (tap t = 9 (dx+1) + 3 (dy+1) + (dz+1))
    return torch.from_numpy(W).permute(2, 1, 0).reshape(W.shape[2], W.shape[1], 3, 3, 3)


@pytest.mark.parametrize("dims,ci,co", [((5, 6, 7), 16, 16), ((4, 3, 9), 9, 1), ((3, 3, 3), 16, 8)])
def test_conv3_matches_torch(dims, ci, co):
    rng = np.random.default_rng(0)
    n = int(np.prod(dims))
    x = rng.standard_normal((n, ci))
    W = rng.standard_normal((27, ci, co))
    xt = torch.from_numpy(x.T.reshape(1, ci, *dims)).requires_grad_(True)
    Wt = _torch_w(W).clone().requires_grad_(True)
    yt = torch.nn.functional.conv3d(xt, Wt, padding=1)
    y = C.conv3_fwd(dims, x, W)
    np.testing.assert_allclose(y, yt.detach().numpy().reshape(co, n).T, rtol=1e-12, atol=1e-12)
    g = rng.standard_normal((n, co))
    yt.backward(torch.from_numpy(g.T.reshape(1, co, *dims)))
    np.testing.assert_allclose(C.conv3_bwd_data(dims, g, W), xt.grad.numpy().reshape(ci, n).T, rtol=1e-10, atol=1e-10)
    gW = C.conv3_bwd_weight(dims, x, g, ci, co)
    np.testing.assert_allclose(_torch_w(gW).numpy(), Wt.grad.numpy(), rtol=1e-10, atol=1e-10)


def test_adam_matches_torch():
    rng = np.random.default_rng(1)
    w0 = rng.standard_normal(50)
    p = torch.nn.Parameter(torch.from_numpy(w0.copy()))
    opt = torch.optim.Adam([p], lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    w, m, v = w0.copy(), np.zeros(50), np.zeros(50)
    for step in range(1, 6):
        g = rng.standard_normal(50)
        p.grad = torch.from_numpy(g.copy())
        opt.step()
        w, m, v = C.adam(w, g, m, v, 1e-2, 0.9, 0.999, 1e-8, step)
    np.testing.assert_allclose(w, p.detach().numpy(), rtol=1e-12, atol=1e-12)


def test_cell_features_layout():
    dims = (3, 4, 5)
    coef = np.exp(np.arange(2 * 3 * 4, dtype=np.float64) / 10.0)
    f = C.node_cell_features(dims, coef, 0.0, 1.0).reshape(3, 4, 5, 8)
    lc = np.log(coef).reshape(2, 3, 4)
    # node (1, 1, 1): cell (1-1+a, 1-1+b, 1-1+c)
    for k in range(8):
        a, b, c = k >> 2, (k >> 1) & 1, k & 1
        assert f[1, 1, 1, k] == pytest.approx(lc[a, b, c])
    assert f[0, 0, 0, 0] == 0.0 and f[0, 0, 0, 7] == pytest.approx(lc[0, 0, 0])


def _small_hierarchy():
    """Two-level hierarchy on a 5^3 node grid (constant coefficient, projected boundary)."""
    import scipy.sparse as sp

    from oracle import fem_q1

    def level(res):
        rows, cols, vals = fem_q1.assemble_triplets((res, res, res))
        m = res + 1
        A = sp.csr_matrix((vals.reshape(-1).astype(np.float64), (rows, cols)), shape=(m ** 3, m ** 3))
        mask = fem_q1.boundary_mask((res, res, res)).astype(np.float64)
        D = sp.diags(1 - mask)
        A = (D @ A @ D + sp.diags(mask)).tocsr()
        return A, mask

    A0, m0 = level(4)
    A1, m1 = level(2)
    P = C.prolongation((5, 5, 5), (3, 3, 3), m0, m1)
    return C.Hierarchy([A0, A1], [1 / A0.diagonal(), 1 / A1.diagonal()], [m0, m1], [P],
                       np.linalg.inv(A1.toarray()), 0.6)


def test_chain_gradient_finite_difference():
    H = _small_hierarchy()
    dims = (5, 5, 5)
    n = 125
    rng = np.random.default_rng(2)
    chat = rng.standard_normal((n, 8)) * 0.5
    shapes = [(16, 16), (16, 16), (16, 16), (16, 1)]
    Ws = [rng.standard_normal((27, ci, co)) * 0.1 for ci, co in shapes]
    relus = [True, True, True, False]
    keep = 1 - H.masks[0]
    pairs = []
    for _ in range(2):
        e = rng.standard_normal(n) * keep
        pairs.append((H.As[0] @ e, e))
    loss, grads = C.smoother_chain(H, dims, chat, Ws, relus, pairs)
    for li, idx in [(0, (13, 0, 3)), (2, (4, 5, 6)), (3, (13, 2, 0))]:
        h = 1e-6
        Wp = [W.copy() for W in Ws]
        Wm = [W.copy() for W in Ws]
        Wp[li][idx] += h
        Wm[li][idx] -= h
        fd = (C.smoother_chain(H, dims, chat, Wp, relus, pairs)[0] - C.smoother_chain(H, dims, chat, Wm, relus, pairs)[0]) / (2 * h)
        assert grads[li][idx] == pytest.approx(fd, rel=1e-4, abs=1e-9)
