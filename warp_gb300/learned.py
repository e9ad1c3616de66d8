"""Learned fine-level smoother: a 4-layer 3x3x3 convolutional network inside the multigrid V-cycle.

No reference counterpart (Warp's only preconditioner is Jacobi, ``warp/_src/optim/linear.py:236-329``).
The network N maps the residual r on the Q1 node grid to a correction and replaces the first
(pre-smoothing) Jacobi step of the V-cycle on the fine level:

    w = omega D^-1 r + mask * N(features(r)),   features: x = D^-1 r, x * c_k (k = 1..8)

where c_k is the normalised log-coefficient of the k-th cell adjacent to the node.  Layers:
16 -> 16 -> 16 -> 16 -> 1 channels, 3x3x3 kernels, ReLU between layers, no biases (so N is
positively homogeneous: N(s r) = s N(r) for s > 0, and no residual normalisation is needed).  The
last layer starts at zero, so an untrained network is exactly the Jacobi-smoothed V-cycle.

Inference: bf16 weights and activations, fp32 accumulation on the tcgen05 tensor cores
(``gb_conv3_fwd_tc``).  Training: fp32 forward / backward / Adam kernels (``gb_conv3_*_f32``,
``gb_adam_step``), loss = ||e - V(r)||_A^2 / ||e||_A^2 over (residual, error) pairs with r = A e,
back-propagated through the rest of the V-cycle with the cycle's own transposed pieces:
    z = (I - w D^-1 A)(I - P Vc R A) w + ...   =>   g_w = (I - A P Vc R)(I - w A D^-1) g_z
(R = P^T and the coarse cycle Vc is symmetric, so the same restrict / coarse-cycle / prolong
kernels serve the backward pass).

Pairs come from the plain solvers run on seeded coefficient fields: iterates of Jacobi-CG on random
right-hand sides (error = converged solution - iterate), and the errors left by stationary
V-cycle iterations (e <- e - V(A e)) from random starts, refreshed with the current network so that
training keeps attacking the modes the learned cycle reduces worst.
"""

from __future__ import annotations

import ctypes
import math
import os

import numpy as np
import torch

from . import _arrays as A
from . import _native as N
from . import multigrid, sparse

# (cin, cout, relu) per layer: scalar fields, and vec3 fields (3 outputs per node)
LAYERS = ((16, 16, True), (16, 16, True), (16, 16, True), (16, 1, False))
LAYERS_VEC3 = ((16, 16, True), (16, 16, True), (16, 16, True), (16, 3, False))
CH = 16
ELASTICITY_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "smoother_q1_elasticity.npz")
SIGMA_DEFAULT = 1.5
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "smoother_q1_diffusion.npz")


def _stream():
    return A.stream()


class ConvNet:
    """Weights (fp32 masters W[t][ci][co], t = 9 (dx+1) + 3 (dy+1) + (dz+1)), Adam state, gradients."""

    def __init__(self, seed: int = 0, device="cuda", ncomp: int = 1):
        if ncomp not in (1, 3):
            raise ValueError("ncomp: 1 (scalar fields) or 3 (vec3 fields)")
        self.ncomp = int(ncomp)
        self.layers = LAYERS if ncomp == 1 else LAYERS_VEC3
        g = torch.Generator().manual_seed(seed)
        self.W, self.gW, self.m, self.v = [], [], [], []
        for li, (ci, co, _) in enumerate(self.layers):
            std = math.sqrt(2.0 / (27 * ci))
            w = torch.randn(27 * ci * co, generator=g, dtype=torch.float32) * std
            if li == len(self.layers) - 1:
                w.zero_()
            self.W.append(w.to(device))
            self.gW.append(torch.zeros(27 * ci * co, device=device))
            self.m.append(torch.zeros(27 * ci * co, device=device))
            self.v.append(torch.zeros(27 * ci * co, device=device))
        self.step_count = 0
        self.mean_log = 0.0
        self.inv_std = 1.0 / SIGMA_DEFAULT
        self.omega = 0.6
        # Jacobi damping of the V-cycle the network is trained in and then serves: a number for every
        # level, or None for the hierarchy's own per-level estimate ("auto")
        self.cycle_omega = 0.6 if ncomp == 1 else None

    # --- persistence -------------------------------------------------------------------------
    def save(self, path: str, **meta) -> None:
        arrs = {f"W{i}": w.detach().cpu().numpy() for i, w in enumerate(self.W)}
        np.savez(path, mean_log=self.mean_log, inv_std=self.inv_std, omega=self.omega, steps=self.step_count,
                 ncomp=self.ncomp, cycle_omega=np.nan if self.cycle_omega is None else self.cycle_omega, **arrs,
                 **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path: str = DEFAULT_WEIGHTS, device="cuda") -> "ConvNet":
        d = np.load(path)
        net = cls(device=device, ncomp=int(d["ncomp"]) if "ncomp" in d else 1)
        for i in range(len(net.layers)):
            net.W[i] = torch.from_numpy(np.asarray(d[f"W{i}"], np.float32)).to(device)
        net.mean_log, net.inv_std, net.omega = float(d["mean_log"]), float(d["inv_std"]), float(d["omega"])
        if "cycle_omega" in d:  # (files written before the field: the constructor's default for ncomp)
            v = float(d["cycle_omega"])
            net.cycle_omega = None if math.isnan(v) else v
        net.step_count = int(d["steps"])
        return net

    def bf16_weights(self, last_cout: int = 16) -> list[torch.Tensor]:
        """Inference layout Wt[t][co_pad][ci] bf16 (co padded to ``last_cout`` for the last layer)."""
        out = []
        for (ci, co, _), w in zip(self.layers, self.W):
            wt = w.reshape(27, ci, co).permute(0, 2, 1)  # [t][co][ci]
            cop = 16 if co == 16 else last_cout
            full = torch.zeros(27, cop, CH, device=w.device, dtype=torch.float32)
            full[:, :co, :ci] = wt
            out.append(full.to(torch.bfloat16).contiguous())
        return out

    # --- fp32 training passes ----------------------------------------------------------------
    def forward_f32(self, dims, feats: torch.Tensor, acts: list[torch.Tensor], stream) -> None:
        """acts[i] <- layer i output (acts[-1] is the [n][ncomp] network output)."""
        L = N.lib()
        nx, ny, nz = dims
        x = feats
        for (ci, co, relu), w, a in zip(self.layers, self.W, acts):
            N.check(L.gb_conv3_fwd_f32(nx, ny, nz, ci, co, A.ptr(x), A.ptr(w), int(relu), A.ptr(a), stream), "conv fwd")
            x = a

    def backward_f32(self, dims, feats, acts, g_out: torch.Tensor, gbuf: list[torch.Tensor], ws: torch.Tensor,
                     stream, need_input_grad: bool = False) -> None:
        """Accumulates dL/dW into self.gW given g_out = dL/d(network output) ([n][ncomp]); gbuf holds
        two [n][16] fp32 scratch buffers (and a third one for the input gradient if requested)."""
        L = N.lib()
        nx, ny, nz = dims
        n = nx * ny * nz
        g = g_out
        for li in range(len(self.layers) - 1, -1, -1):
            ci, co, relu = self.layers[li]
            inp = feats if li == 0 else acts[li - 1]
            N.check(L.gb_conv3_bwd_weight_f32(nx, ny, nz, ci, co, A.ptr(inp), A.ptr(g), A.ptr(self.gW[li]), A.ptr(ws),
                                              ws.numel(), stream), "conv bwd weight")
            if li == 0 and not need_input_grad:
                break
            gin = gbuf[li % 2] if li > 0 else gbuf[2]
            N.check(L.gb_conv3_bwd_data_f32(nx, ny, nz, ci, co, A.ptr(g), A.ptr(self.W[li]), A.ptr(gin), stream),
                    "conv bwd data")
            if li > 0 and self.layers[li - 1][2]:
                N.check(L.gb_relu_bwd(n * ci, A.ptr(acts[li - 1]), A.ptr(gin), stream), "relu bwd")
            g = gin

    def zero_grad(self) -> None:
        for g in self.gW:
            g.zero_()

    def adam(self, lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8, stream=None) -> None:
        stream = _stream() if stream is None else stream
        L = N.lib()
        self.step_count += 1
        for w, g, m, v in zip(self.W, self.gW, self.m, self.v):
            N.check(L.gb_adam_step(w.numel(), A.ptr(w), A.ptr(g), A.ptr(m), A.ptr(v), lr, b1, b2, eps, self.step_count,
                                   None, stream), "adam")

    def bwd_weight_workspace(self, dims) -> torch.Tensor:
        L = N.lib()
        nb = max(L.gb_conv3_bwd_weight_workspace_bytes(*dims, ci, co) for ci, co, _ in self.layers)
        return A.workspace(nb)


def cell_features(dims, coef: torch.Tensor, mean_log: float, inv_std: float) -> torch.Tensor:
    """[n][8] normalised log-coefficients of the cells around each node (0 outside the grid)."""
    n = dims[0] * dims[1] * dims[2]
    chat = A.empty(n * 8, torch.float32)
    N.check(N.lib().gb_net_cell_features(*dims, A.ptr(coef), mean_log, inv_std, A.ptr(chat), _stream()), "cell feats")
    return chat


def planar_rows(dims) -> int:
    return int(N.lib().gb_conv3_planar_rows(*dims))


def to_planar(act: torch.Tensor, dims) -> torch.Tensor:
    """[n, 16] activations -> planar padded bf16 buffer [2, rows, 8] (border rows zero)."""
    nx, ny, nz = dims
    rows = planar_rows(dims)
    buf = torch.zeros(2, rows, 8, dtype=torch.bfloat16, device=act.device)
    p = padded_rows(dims, act.device)
    a = act.reshape(-1, 16).to(torch.bfloat16)
    buf[0, p] = a[:, :8]
    buf[1, p] = a[:, 8:]
    return buf


def from_planar(buf: torch.Tensor, dims) -> torch.Tensor:
    p = padded_rows(dims, buf.device)
    return torch.cat([buf[0, p], buf[1, p]], dim=1)


def padded_rows(dims, device) -> torch.Tensor:
    nx, ny, nz = dims
    v = torch.arange(nx * ny * nz, device=device)
    x, y, z = v // (ny * nz), (v // nz) % ny, v % nz
    return ((x + 1) * (ny + 2) + (y + 1)) * (nz + 2) + (z + 1)


class LearnedSmoother:
    """The inference smoother plugged into ``MultigridPreconditioner.smoother``.

    tcgen05 implicit-GEMM layers on the planar padded layout (features + 4 layers, the last one fused
    with the Jacobi step).  ``launches``: 5 -- the features kernel and one launch per layer; 2 -- the
    features kernel, then the four layers in one cooperative launch whose CTAs wait on per-item
    completion counters instead of kernel boundaries; 1 -- the features computed inside that launch
    too.  All three write the same values, bit for bit."""

    def __init__(self, net: ConvNet, mg: multigrid.MultigridPreconditioner, coef, backend: str = "tc",
                 launches: int = 2):
        bdim = getattr(mg, "bdim", 1)
        if bdim != net.ncomp:
            raise ValueError(f"learned smoother: a network for {net.ncomp}-component fields on a {bdim}x{bdim} "
                             "hierarchy")
        lv = mg.levels[0]
        if len(lv.dims) != 3:
            raise ValueError("learned smoother: 3-D grids only")
        if backend != "tc":
            raise ValueError(f"unknown backend {backend!r} (the tcgen05 layers are the only inference path)")
        self.backend = backend
        self.ncomp = bdim
        self.mg = mg
        self.dims = lv.dims
        self.n = lv.n
        if net.cycle_omega is not None:
            # the network serves the cycle it was trained in: its Jacobi damping on every level
            for level in mg.levels:
                level.omega = float(net.cycle_omega)
        self.omega = float(lv.omega)
        self.mask, self.dinv = lv.mask, lv.dinv
        self.status = mg.status
        coef_t = coef if isinstance(coef, torch.Tensor) else A.from_numpy(np.asarray(coef, np.float32).reshape(-1))
        self.chat = cell_features(self.dims, coef_t.reshape(-1).float().contiguous(), net.mean_log, net.inv_std)
        self.Wt = net.bf16_weights(last_cout=16)
        rows = planar_rows(self.dims)
        self.buf = [A.zeros(2 * rows * 8, torch.bfloat16), A.zeros(2 * rows * 8, torch.bfloat16)]
        if launches not in (1, 2, 5):
            raise ValueError("launches must be 1, 2 or 5")
        self.kernels_per_apply = 5
        self.whole_network = launches < 5 and 2 <= len(self.Wt) <= 4
        self._features_in_network = launches == 1
        if self.whole_network:
            L = N.lib()
            nl = len(self.Wt)
            # one planar buffer per layer input: no layer overwrites what another CTA may still stage
            self.buf += [A.zeros(2 * rows * 8, torch.bfloat16) for _ in range(nl - 2)]
            self.flags = A.zeros(int(L.gb_convnet_tc_items(*self.dims)), torch.int32)
            self.epoch = A.zeros(2, torch.int32)
            self._act = (ctypes.c_void_p * nl)(*[A.ptr(b) for b in self.buf[:nl]])
            self._wt = (ctypes.c_void_p * nl)(*[A.ptr(t) for t in self.Wt])
            self.kernels_per_apply = 1 if self._features_in_network else 2

    def launch(self, stream, r: int, w: int) -> None:
        L = N.lib()
        if self.whole_network:
            if not self._features_in_network:
                N.check(L.gb_net_features_planar(self.ncomp, *self.dims, r, A.ptr(self.dinv), A.ptr(self.chat),
                                                 A.ptr(self.mask), A.ptr(self.buf[0]), stream), "features")
            chat = None if not self._features_in_network else A.ptr(self.chat)
            N.check(L.gb_convnet_fwd_tc(*self.dims, self.ncomp, len(self.Wt), self._act, self._wt, w, r,
                                        A.ptr(self.dinv), chat, A.ptr(self.mask), self.omega,
                                        A.ptr(self.flags), A.ptr(self.epoch), A.ptr(self.status), stream),
                    "convnet tc")
            return
        N.check(L.gb_net_features_planar(self.ncomp, *self.dims, r, A.ptr(self.dinv), A.ptr(self.chat),
                                         A.ptr(self.mask), A.ptr(self.buf[0]), stream), "features")
        src, dst = self.buf[0], self.buf[1]
        for li, wt in enumerate(self.Wt):
            last = li == len(self.Wt) - 1
            mode = (1 if self.ncomp == 1 else 3) if last else 0
            N.check(L.gb_conv3_fwd_tc(*self.dims, mode, A.ptr(src), A.ptr(wt), None if last else A.ptr(dst),
                                      w if last else None, r if last else None, A.ptr(self.dinv) if last else None,
                                      A.ptr(self.mask) if last else None, self.omega, A.ptr(self.status), stream),
                    "conv tc")
            src, dst = dst, src


class TrainingSmoother:
    """fp32 forward that keeps every activation, used while training."""

    kernels_per_apply = 6

    def __init__(self, net: ConvNet, mg: multigrid.MultigridPreconditioner, coef):
        lv = mg.levels[0]
        self.net, self.mg = net, mg
        self.ncomp = getattr(mg, "bdim", 1)
        self.dims, self.n, self.omega = lv.dims, lv.n, float(lv.omega)
        self.mask, self.dinv = lv.mask, lv.dinv
        coef_t = coef if isinstance(coef, torch.Tensor) else A.from_numpy(np.asarray(coef, np.float32).reshape(-1))
        self.chat = cell_features(self.dims, coef_t.reshape(-1).float().contiguous(), net.mean_log, net.inv_std)
        self.feats = A.empty(self.n * CH, torch.float32)
        self.acts = [A.empty(self.n * co, torch.float32) for _, co, _ in net.layers]

    def launch(self, stream, r: int, w: int) -> None:
        L = N.lib()
        N.check(L.gb_net_features(N.GB_F32, self.ncomp, self.n, r, A.ptr(self.dinv), A.ptr(self.chat),
                                  A.ptr(self.mask), A.ptr(self.feats), stream), "features")
        self.net.forward_f32(self.dims, self.feats, self.acts, stream)
        N.check(L.gb_net_combine(N.GB_F32, self.ncomp, self.n, self.ncomp, A.ptr(self.acts[-1]), A.ptr(self.mask),
                                 self.omega, A.ptr(self.dinv), r, w, stream), "combine")


class _Field:
    """One training problem: system, hierarchy, fp32 training smoother and scratch vectors."""

    def __init__(self, system, net: ConvNet, coarsest_nodes: int = 400):
        self.sys = system
        faces = ("x-",) if system.A.block_shape == (3, 3) else ("x-", "x+", "y-", "y+", "z-", "z+")
        # the training hierarchy (the shipped weights: coarsest grid <= 400 nodes) in the network's damping
        self.mg = multigrid.MultigridPreconditioner(system.A, system.geo, system.coef, faces=faces,
                                                    coarsest_nodes=coarsest_nodes,
                                                    omega="auto" if net.cycle_omega is None else net.cycle_omega)
        self.bdim = self.mg.bdim
        self.sm = TrainingSmoother(net, self.mg, system.coef)
        n = self.mg.n
        self.n = n
        self.z, self.gz, self.u, self.g, self.p = (A.zeros(n, torch.float32) for _ in range(5))
        # per-dof Dirichlet mask of the fine level (the hierarchy keeps one per node)
        self.mask_dof = self.mg.levels[0].mask.repeat_interleave(self.bdim).contiguous()
        nc = self.mg.levels[1].n * self.bdim if len(self.mg.levels) > 1 else 0
        self.coarse_rhs = A.zeros(nc, torch.float32) if nc else None
        self.coarse_sol = A.zeros(nc, torch.float32) if nc else None


def _spmv(Am: sparse.BsrMatrix, x: torch.Tensor, y: torch.Tensor, alpha: float, beta: float, stream, status) -> None:
    br, bc = Am.block_shape
    N.check(N.lib().gb_bsr_mv(br, bc, Am.nrow, Am.ncol, Am.nnz_sync(), Am.capacity, A.ptr(Am.offsets), None,
                              A.ptr(Am.columns), A.ptr(Am.values), N.GB_F32, A.ptr(x), A.ptr(y), A.ptr(y), N.GB_F32,
                              alpha, beta, 0, 0, 0, -1, A.ptr(status), stream), "spmv")


class SmootherTrainer:
    """GPU training of the learned smoother with the package's own kernels."""

    def __init__(self, net: ConvNet, lr: float = 1e-3, coarsest_nodes: int = 400):
        self.net = net
        self.lr = lr
        self.coarsest_nodes = coarsest_nodes
        self._ws = None
        self._ws_dims = None
        self._gbuf = None
        self._dots_ws = A.zeros(int(N.lib().gb_dots_workspace_bytes()), torch.uint8)  # arrival counter starts at 0
        self._dots_out = A.zeros(4, torch.float64)

    def field(self, system) -> _Field:
        f = _Field(system, self.net, self.coarsest_nodes)
        f.mg.smoother = f.sm
        return f

    def _scratch(self, dims):
        if self._ws_dims != dims:
            n = dims[0] * dims[1] * dims[2]
            self._ws = self.net.bwd_weight_workspace(dims)
            self._gbuf = [A.empty(n * CH, torch.float32) for _ in range(3)]
            self._ws_dims = dims
        return self._ws, self._gbuf

    def _dots(self, pairs, n) -> torch.Tensor:
        xs = (ctypes.c_void_p * 4)(*[A.ptr(a) for a, _ in pairs])
        ys = (ctypes.c_void_p * 4)(*[A.ptr(b) for _, b in pairs])
        N.check(N.lib().gb_dots(N.GB_F32, n, len(pairs), xs, ys, A.ptr(self._dots_out), A.ptr(self._dots_ws),
                                _stream()), "dots")
        return self._dots_out[: len(pairs)]

    def loss_and_grad(self, f: _Field, r: torch.Tensor, e: torch.Tensor, weight: float = 1.0) -> torch.Tensor:
        """Forward V-cycle with the fp32 network, loss ||e - z||_A^2 / ||e||_A^2 (device scalar), and
        accumulation of weight * dLoss/dW into net.gW."""
        stream = _stream()
        L = N.lib()
        mg, n = f.mg, f.n
        lv0 = mg.levels[0]
        st = mg.status
        mg.launch(stream, A.ptr(r), A.ptr(f.z))  # z = V(r), activations kept in f.sm
        # gz = r - A z ; loss = (e - z).gz / e.r
        f.gz.copy_(r)
        _spmv(lv0.A, f.z, f.gz, -1.0, 1.0, stream, st)
        f.u.copy_(e).sub_(f.z)
        d = self._dots([(f.u, f.gz), (e, r)], n)
        den = d[1].clamp_min(1e-300)
        loss = (d[0] / den).clone()
        # dL/dz = -2 (r - A z) / den
        scale = (-2.0 * weight / den).to(torch.float32)
        f.gz.mul_(scale)
        # g_w2 = gz - omega A D^-1 gz (D the fine level's smoothing diagonal: the 3x3 node blocks under
        # block Jacobi)
        if getattr(lv0, "dinvb", None) is not None:
            N.check(L.gb_mg_block_jacobi0(lv0.n, 1.0, A.ptr(lv0.dinvb), A.ptr(f.gz), A.ptr(f.u), stream), "dinvb")
        else:
            torch.mul(lv0.dinv, f.gz, out=f.u)
        f.g.copy_(f.gz)
        _spmv(lv0.A, f.u, f.g, -float(lv0.omega), 1.0, stream, st)
        # g_w = g_w2 - A P Vc R g_w2
        if len(mg.levels) > 1:
            lv1 = mg.levels[1]
            N.check(L.gb_mg_restrict_c(f.bdim, *lv0.dims, *lv1.dims, A.ptr(f.g), A.ptr(lv0.mask), A.ptr(lv1.mask),
                                       A.ptr(f.coarse_rhs), stream), "restrict")
            mg._vcycle(1, A.ptr(f.coarse_rhs), A.ptr(f.coarse_sol), stream)
            f.p.zero_()
            N.check(L.gb_mg_prolong_add_c(f.bdim, *lv0.dims, *lv1.dims, A.ptr(f.coarse_sol), A.ptr(lv0.mask), 1.0,
                                          A.ptr(f.p), stream), "prolong")
            _spmv(lv0.A, f.p, f.g, -1.0, 1.0, stream, st)
        # network output gradient (masked nodes do not take the network's value); [n][ncomp] is the
        # interleaved dof layout
        f.g.mul_(1.0 - f.mask_dof)
        ws, gbuf = self._scratch(f.sm.dims)
        self.net.backward_f32(f.sm.dims, f.sm.feats, f.sm.acts, f.g, gbuf, ws, stream)
        return loss

    def eval_loss(self, f: _Field, r: torch.Tensor, e: torch.Tensor, smoother=None) -> float:
        """Loss of the V-cycle with the given smoother (None: Jacobi) without touching gradients."""
        saved = f.mg.smoother
        f.mg.smoother = smoother
        stream = _stream()
        f.mg.launch(stream, A.ptr(r), A.ptr(f.z))
        f.gz.copy_(r)
        _spmv(f.mg.levels[0].A, f.z, f.gz, -1.0, 1.0, stream, f.mg.status)
        f.u.copy_(e).sub_(f.z)
        d = self._dots([(f.u, f.gz), (e, r)], f.n)
        f.mg.smoother = saved
        return float(d[0] / d[1])

    # a batch whose loss exceeds this in magnitude is degenerate (a pair whose error is nearly A-orthogonal
    # to its residual gives a vanishing denominator, a diverging network a runaway output); its gradient
    # is dropped instead of applied
    MAX_BATCH_LOSS = 1e3

    def step(self, f: _Field, pairs) -> float:
        self.net.zero_grad()
        losses = []
        for r, e in pairs:
            losses.append(self.loss_and_grad(f, r, e, 1.0 / len(pairs)))
        tot = float(torch.stack(losses).mean())
        if math.isfinite(tot) and abs(tot) <= self.MAX_BATCH_LOSS:
            self.net.adam(self.lr)
        else:
            self.skipped_steps = getattr(self, "skipped_steps", 0) + 1
            self.net.zero_grad()
        return tot


def training_problem(res: int = 48, seed: int = 0, sigma: float = SIGMA_DEFAULT, corr_length: float = 0.1,
                     cell_size: float = 1.0 / 96):
    """A training field: Q1 diffusion on res^3 cells whose lognormal coefficient has the statistics of
    the 96^3 unit-cube problem (correlation length in cells = corr_length / cell_size)."""
    from . import problems

    return problems.diffusion((res, res, res), sigma=sigma, corr_length=corr_length, seed=seed,
                              field_cell_size=cell_size)


# --- training pairs from the plain solvers -----------------------------------------------------
def cg_pairs(f: _Field, nrhs: int, rng: np.random.Generator, iters=(0, 1, 2, 4, 8, 16, 32, 64)):
    """(r_k, e_k) along Jacobi-CG runs on random right-hand sides (e_k = x* - x_k, x* from a tight
    multigrid-FCG solve)."""
    from .optim import linear

    A_ = f.sys.A
    n = f.n
    keep = 1.0 - f.mask_dof
    out = []
    M = linear.preconditioner(A_, "diag")
    for _ in range(nrhs):
        b = A.from_numpy(rng.uniform(-1.0, 1.0, n).astype(np.float32)) * keep
        xs = torch.zeros(n, device=b.device)
        saved = f.mg.smoother
        f.mg.smoother = None
        linear.fcg(A_, b, xs, tol=1e-7, atol=0.0, maxiter=200, M=f.mg, check_every=0)
        f.mg.smoother = saved
        x = torch.zeros(n, device=b.device)
        snaps = {}

        def grab(it, err, atol_v, x=x, snaps=snaps):
            if it in iters:
                snaps[it] = x.clone()

        linear.cg(A_, b, x, tol=0.0, atol=0.0, maxiter=max(iters), M=M, callback=grab, check_every=1,
                  use_cuda_graph=False)
        for k in iters:
            if k not in snaps:  # the run stopped early (exact convergence)
                continue
            xk = snaps[k]
            r = b.clone()
            _spmv(A_, xk, r, -1.0, 1.0, _stream(), f.mg.status)
            e = xs - xk
            s = 1.0 / float(e.norm().clamp_min(1e-30))
            out.append((r * s, e * s))
    return out


def fcg_pairs(f: _Field, nrhs: int, rng: np.random.Generator, iters=(1, 2, 4, 6, 8, 12)):
    """(r_k, e_k) along the flexible-CG runs the network will serve in: FCG preconditioned by the V-cycle
    with the current (training) network, on random right-hand sides (e_k = x* - x_k, x* from a tight
    solve with the Jacobi-smoothed cycle; normalised)."""
    from .optim import linear

    A_ = f.sys.A
    n = f.n
    keep = 1.0 - f.mask_dof
    out = []
    for _ in range(nrhs):
        b = A.from_numpy(rng.uniform(-1.0, 1.0, n).astype(np.float32)) * keep
        xs = torch.zeros(n, device=b.device)
        saved = f.mg.smoother
        f.mg.smoother = None
        linear.fcg(A_, b, xs, tol=1e-7, atol=0.0, maxiter=400, M=f.mg, check_every=0)
        f.mg.smoother = saved
        x = torch.zeros(n, device=b.device)
        snaps = {}

        def grab(it, err, atol_v, x=x, snaps=snaps):
            if it in iters:
                snaps[it] = x.clone()

        linear.fcg(A_, b, x, tol=0.0, atol=0.0, maxiter=max(iters), M=f.mg, callback=grab, check_every=1,
                   use_cuda_graph=False)
        for k in iters:
            if k not in snaps:
                continue
            xk = snaps[k]
            r = b.clone()
            _spmv(A_, xk, r, -1.0, 1.0, _stream(), f.mg.status)
            e = xs - xk
            s = 1.0 / float(e.norm().clamp_min(1e-30))
            out.append((r * s, e * s))
    return out


def slow_pairs(f: _Field, nrhs: int, rng: np.random.Generator, sweeps=(1, 2, 3, 5), smoother="current"):
    """Errors left by stationary V-cycle sweeps e <- e - V(A e) from random starts (normalised)."""
    n = f.n
    keep = 1.0 - f.mask_dof
    A_ = f.sys.A
    out = []
    saved = f.mg.smoother
    if smoother is None:
        f.mg.smoother = None
    stream = _stream()
    r = A.zeros(n, torch.float32)
    z = A.zeros(n, torch.float32)
    for _ in range(nrhs):
        e = A.from_numpy(rng.standard_normal(n).astype(np.float32)) * keep
        for k in range(max(sweeps) + 1):
            r.zero_()
            _spmv(A_, e, r, 1.0, 0.0, stream, f.mg.status)
            if k in sweeps:
                s = 1.0 / float(e.norm().clamp_min(1e-30))
                out.append((r * s, e * s))
            f.mg.launch(stream, A.ptr(r), A.ptr(z))
            e = e - z
    f.mg.smoother = saved
    return out
