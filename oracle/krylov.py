"""CPU oracle (test infrastructure only): NumPy float64 restatements of the reference's Conjugate
Residual and restarted GMRES iterations, for small dense systems.

* ``cr``: warp/_src/optim/linear.py:1124-1286 with the update kernels :2377-2423 (alpha and beta
  frozen at 0 once the residual meets the tolerance; y = M Ap; z updated recursively).
* ``gmres``: warp/_src/optim/linear.py:1653-1916 (k Arnoldi steps per cycle, one-pass classical
  Gram-Schmidt, Givens least squares with pivot tolerance eps^2 :2497-2560, true residual after
  every cycle, iteration count advancing by k).
Tolerances follow _get_tolerances (linear.py:2010-2032): atol_eff = max(tol ||b||, atol).
"""

from __future__ import annotations

import math

import numpy as np


def cr(A, b, x0=None, dinv=None, tol=1e-6, atol=0.0, maxiter=1000):
    A = np.asarray(A, np.float64)
    b = np.asarray(b, np.float64)
    x = np.zeros_like(b) if x0 is None else np.array(x0, np.float64)
    Mv = (lambda v: v) if dinv is None else (lambda v: np.asarray(dinv, np.float64) * v)
    atol_sq = max(tol * math.sqrt(b @ b), atol) ** 2
    r = b - A @ x
    z = Mv(r)
    Az = A @ z
    rr, zAz = r @ r, z @ Az
    p, Ap = z.copy(), Az.copy()
    it = 0
    while rr > atol_sq and it < maxiter:
        zAz_old = zAz
        y = Mv(Ap)
        yAp = Ap @ y
        alpha = zAz_old / yAp if yAp > 0 else 0.0
        x += alpha * p
        r -= alpha * Ap
        z = z - alpha * y if dinv is not None else r.copy()
        Az = A @ z
        rr, zAz = r @ r, z @ Az
        beta = zAz / zAz_old if (rr > atol_sq and zAz_old > 0) else 0.0
        p = z + beta * p
        Ap = Az + beta * Ap
        it += 1
    return x, it, math.sqrt(rr)


def gmres(A, b, x0=None, dinv=None, tol=1e-6, atol=0.0, restart=31, maxiter=1000, left=False, eps=1e-8):
    A = np.asarray(A, np.float64)
    b = np.asarray(b, np.float64)
    n = b.size
    x = np.zeros_like(b) if x0 is None else np.array(x0, np.float64)
    Mv = None if dinv is None else (lambda v: np.asarray(dinv, np.float64) * v)
    k = max(1, min(restart, maxiter))
    atol_sq = max(tol * math.sqrt(b @ b), atol) ** 2
    r = b - A @ x
    rr = r @ r
    it = 0
    while rr > atol_sq and it < maxiter:
        rh = Mv(r) if (Mv and left) else r
        beta = math.sqrt(rh @ rh)
        V = np.zeros((k + 1, n))
        V[0] = rh / beta if beta else rh
        H = np.zeros((k + 1, k))
        for j in range(k):
            if Mv is None:
                w = A @ V[j]
            elif left:
                w = Mv(A @ V[j])
            else:
                w = A @ Mv(V[j])
            h = V[: j + 1] @ w
            w = w - h @ V[: j + 1]
            H[: j + 1, j] = h
            hn = math.sqrt(w @ w)
            H[j + 1, j] = hn
            V[j + 1] = w / hn if hn else w
        # Givens least squares with the pivot tolerance eps^2
        Hc = H.copy()
        g = np.zeros(k + 1)
        rhs = beta
        kk = k
        for i in range(k):
            a, c2 = Hc[i, i], Hc[i + 1, i]
            n2 = a * a + c2 * c2
            if n2 < eps * eps:
                kk = i
                break
            nrm = math.sqrt(n2)
            c, s = a / nrm, c2 / nrm
            Hi, Hj = Hc[i, i:].copy(), Hc[i + 1, i:].copy()
            Hc[i, i:] = c * Hi + s * Hj
            Hc[i + 1, i:] = c * Hj - s * Hi
            g[i] = c * rhs
            rhs = -s * rhs
        y = np.zeros(kk)
        for i in range(kk - 1, -1, -1):
            y[i] = (g[i] - Hc[i, i + 1:kk] @ y[i + 1:kk]) / Hc[i, i]
        dx = y @ V[:kk]
        x += Mv(dx) if (Mv is not None and not left) else dx
        r = b - A @ x
        rr = r @ r
        it += k
    return x, it, math.sqrt(rr)
