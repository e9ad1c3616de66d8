"""CPU oracle (test infrastructure only) for the learned smoother's network and its training step.

NumPy float64 restatement of the product's conv-net kernels (no reference counterpart exists: Warp's
only preconditioner is Jacobi, warp/_src/optim/linear.py:236-329):

* ``conv3_fwd``: out[v][co] = sum_t sum_ci W[t][ci][co] in[v + off(t)][ci], taps
  t = 9 (dx+1) + 3 (dy+1) + (dz+1), zero outside the node grid (3x3x3 cross-correlation, "same" size);
* ``conv3_bwd_data`` / ``conv3_bwd_weight``: its exact adjoints;
* ``adam``: Kingma & Ba (2015) with bias correction;
* ``node_cell_features`` / ``features`` / ``combine``: the smoother's input and output maps;
* ``smoother_chain``: loss ||e - V(r)||_A^2 / ||e||_A^2 of the V-cycle whose fine pre-smoother is
  the network, and its gradient with respect to every weight, for a hierarchy given as SciPy
  matrices (levels' operators, masks, transfers, coarsest inverse).

This module is pinned against an independent implementation (torch's CPU conv3d and autograd) in
``tests/test_oracle_convnet.py``; only tests may import it.
"""

from __future__ import annotations

import numpy as np

TAPS = [(dx, dy, dz) for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)]


def _shift(a: np.ndarray, d) -> np.ndarray:
    """s[x, y, z] = a[x + dx, y + dy, z + dz] (zero outside); a is [nx, ny, nz, C]."""
    out = np.zeros_like(a)
    nx, ny, nz = a.shape[:3]
    dx, dy, dz = d
    xs = slice(max(0, -dx), nx - max(0, dx))
    ys = slice(max(0, -dy), ny - max(0, dy))
    zs = slice(max(0, -dz), nz - max(0, dz))
    xsrc = slice(max(0, dx), nx + min(0, dx))
    ysrc = slice(max(0, dy), ny + min(0, dy))
    zsrc = slice(max(0, dz), nz + min(0, dz))
    out[xs, ys, zs] = a[xsrc, ysrc, zsrc]
    return out


def conv3_fwd(dims, inp: np.ndarray, W: np.ndarray, relu: bool = False) -> np.ndarray:
    """inp [n, ci], W [27, ci, co] -> [n, co]."""
    nx, ny, nz = dims
    ci, co = W.shape[1], W.shape[2]
    a = np.asarray(inp, np.float64).reshape(nx, ny, nz, ci)
    out = np.zeros((nx, ny, nz, co))
    for t, d in enumerate(TAPS):
        out += _shift(a, d) @ W[t]
    if relu:
        out = np.maximum(out, 0.0)
    return out.reshape(-1, co)


def conv3_bwd_data(dims, gout: np.ndarray, W: np.ndarray) -> np.ndarray:
    """gin[v][ci] = sum_t sum_co W[t][ci][co] gout[v - off(t)][co]."""
    nx, ny, nz = dims
    ci, co = W.shape[1], W.shape[2]
    g = np.asarray(gout, np.float64).reshape(nx, ny, nz, co)
    out = np.zeros((nx, ny, nz, ci))
    for t, d in enumerate(TAPS):
        out += _shift(g, tuple(-c for c in d)) @ W[t].T
    return out.reshape(-1, ci)


def conv3_bwd_weight(dims, inp: np.ndarray, gout: np.ndarray, ci: int, co: int) -> np.ndarray:
    """gW[t][ci][co] = sum_v in[v + off(t)][ci] gout[v][co]."""
    nx, ny, nz = dims
    a = np.asarray(inp, np.float64).reshape(nx, ny, nz, ci)
    g = np.asarray(gout, np.float64).reshape(-1, co)
    gW = np.zeros((27, ci, co))
    for t, d in enumerate(TAPS):
        gW[t] = _shift(a, d).reshape(-1, ci).T @ g
    return gW


def adam(w, g, m, v, lr, b1, b2, eps, step):
    """One Adam update; returns (w, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def node_cell_features(dims, cell_coef: np.ndarray, mean_log: float, inv_std: float) -> np.ndarray:
    """[n, 8]: normalised log-coefficient of cell (x-1+a, y-1+b, z-1+c), k = 4a + 2b + c."""
    nx, ny, nz = dims
    cx, cy, cz = nx - 1, ny - 1, nz - 1
    lc = (np.log(np.asarray(cell_coef, np.float64).reshape(cx, cy, cz)) - mean_log) * inv_std
    out = np.zeros((nx, ny, nz, 8))
    for k in range(8):
        a, b, c = k >> 2, (k >> 1) & 1, k & 1
        out[1 - a:1 - a + cx, 1 - b:1 - b + cy, 1 - c:1 - c + cz, k] = lc
    return out.reshape(-1, 8)


def features(r, dinv, chat, mask) -> np.ndarray:
    """[n, 16]: x = dinv r (0 at masked nodes), x * chat[:, k], zeros."""
    x = np.where(mask != 0, 0.0, np.asarray(dinv, np.float64) * r)
    f = np.zeros((len(r), 16))
    f[:, 0] = x
    f[:, 1:9] = x[:, None] * chat
    return f


def combine(out0, mask, omega, dinv, r) -> np.ndarray:
    return np.where(mask != 0, 0.0, out0) + omega * dinv * r


def features_vec3(r, dinv, chat, mask) -> np.ndarray:
    """Vec3 fields (3 interleaved components per node): [n, 16] with x_c = dinv_c r_c (0 at masked
    nodes) in channels 0..2 and x_c * s_j in channel 3 + 4c + j, where s_0 is the mean of the node's 8
    cell values chat[:, k] and s_1..3 their x / y / z contrasts (mean over the cells with bit 2 / 1 / 0 of
    k set minus the others)."""
    n = len(mask)
    x = np.where((mask != 0)[:, None], 0.0, (np.asarray(dinv, np.float64) * r).reshape(n, 3))
    k = np.arange(8)
    sign = np.stack([np.ones(8), np.where(k >> 2, 1.0, -1.0), np.where((k >> 1) & 1, 1.0, -1.0),
                     np.where(k & 1, 1.0, -1.0)])  # [4, 8]
    s = np.asarray(chat, np.float64) @ sign.T / 8.0  # [n, 4]
    f = np.zeros((n, 16))
    f[:, 0:3] = x
    for c in range(3):
        f[:, 3 + 4 * c:7 + 4 * c] = x[:, c:c + 1] * s
    return f


def combine_vec3(out, mask, omega, dinv, r) -> np.ndarray:
    """[3n]: omega dinv r + (mask[node] ? 0 : out[node][c])."""
    n = len(mask)
    return (np.where((mask != 0)[:, None], 0.0, np.asarray(out).reshape(n, 3)).reshape(-1)
            + omega * np.asarray(dinv, np.float64) * r)


def net_forward(dims, feats, Ws, relus):
    acts = []
    x = feats
    for W, relu in zip(Ws, relus):
        x = conv3_fwd(dims, x, W, relu)
        acts.append(x)
    return acts


def net_backward(dims, feats, acts, Ws, relus, g_out):
    """Returns dL/dW for every layer given dL/d(last output)."""
    grads = [None] * len(Ws)
    g = np.asarray(g_out, np.float64).reshape(len(feats), -1)
    for li in range(len(Ws) - 1, -1, -1):
        inp = feats if li == 0 else acts[li - 1]
        grads[li] = conv3_bwd_weight(dims, inp, g, Ws[li].shape[1], Ws[li].shape[2])
        if li == 0:
            break
        g = conv3_bwd_data(dims, g, Ws[li])
        if relus[li - 1]:
            g = g * (acts[li - 1] > 0)
    return grads


class Hierarchy:
    """CPU copy of a V-cycle: levels' (A csr, dinv, mask), transfers P_l (fine <- coarse, masked as the
    product's kernels are), the coarsest inverse, and omega."""

    def __init__(self, As, dinvs, masks, Ps, coarse_inv, omega):
        self.As, self.dinvs, self.masks, self.Ps = As, dinvs, masks, Ps
        self.coarse_inv, self.omega = coarse_inv, omega

    def vcycle(self, r, li=0, w0=None):
        if li == len(self.As) - 1:
            return self.coarse_inv @ r
        A, d = self.As[li], self.dinvs[li]
        w = self.omega * d * r if w0 is None else w0
        t = r - A @ w
        P = self.Ps[li]
        zc = self.vcycle(P.T @ t, li + 1)
        w = w + P @ zc
        return w + self.omega * d * (r - A @ w)


def prolongation(fdims, cdims, fmask, cmask):
    """Trilinear P (vertex-centred 2:1), rows of masked fine nodes and columns of masked coarse
    nodes removed (the product restricts with both masks and prolongs into unmasked nodes only)."""
    import scipy.sparse as sp

    def p1(mf, mc):
        rows, cols, vals = [], [], []
        for i in range(mf):
            if i % 2 == 0:
                rows.append(i); cols.append(i // 2); vals.append(1.0)
            else:
                rows += [i, i]; cols += [i // 2, i // 2 + 1]; vals += [0.5, 0.5]
        return sp.csr_matrix((vals, (rows, cols)), shape=(mf, mc))

    P = sp.kron(sp.kron(p1(fdims[0], cdims[0]), p1(fdims[1], cdims[1])), p1(fdims[2], cdims[2])).tocsr()
    return (sp.diags(1.0 - fmask) @ P @ sp.diags(1.0 - cmask)).tocsr()


def smoother_chain(H: Hierarchy, dims, chat, Ws, relus, pairs):
    """Mean loss over pairs and its gradient with respect to every layer's W (float64)."""
    A0, d0, m0 = H.As[0], H.dinvs[0], H.masks[0]
    grads = [np.zeros_like(W) for W in Ws]
    losses = []
    for r, e in pairs:
        r = np.asarray(r, np.float64)
        e = np.asarray(e, np.float64)
        f = features(r, d0, chat, m0)
        acts = net_forward(dims, f, Ws, relus)
        w = combine(acts[-1][:, 0], m0, H.omega, d0, r)
        z = H.vcycle(r, 0, w)
        rz = r - A0 @ z
        den = e @ r
        losses.append((e - z) @ rz / den)
        gz = -2.0 * rz / den / len(pairs)
        gw2 = gz - H.omega * (A0 @ (d0 * gz))
        P = H.Ps[0]
        gw = gw2 - A0 @ (P @ H.vcycle(P.T @ gw2, 1))
        gout = np.where(m0 != 0, 0.0, gw)
        for i, g in enumerate(net_backward(dims, f, acts, Ws, relus, gout[:, None])):
            grads[i] += g
    return float(np.mean(losses)), grads
