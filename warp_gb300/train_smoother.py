"""Train the learned smoother on the GPU with the package's own kernels.

    python -m warp_gb300.train_smoother --fields 2000 --res 48 --out warp_gb300/data/smoother_q1_diffusion.npz
    python -m warp_gb300.train_smoother --problem elasticity --fields 400 --res 32 \
        --out warp_gb300/data/smoother_q1_elasticity.npz

Each seeded coefficient field (lognormal, squared-exponential GRF, sigma 1.5, correlation length 0.1
on cells of size 1/96: a 48^3 sub-block of the 96^3 unit-cube problem) contributes (residual, error)
pairs from the plain solvers -- Jacobi-CG iterates on a random right-hand side and the errors left
by stationary V-cycle sweeps (with the current network and with Jacobi smoothing) -- and
``steps_per_field`` Adam steps on random batches of them (cosine learning-rate decay).
"""

from __future__ import annotations

import argparse
import math
import time

import numpy as np
import torch

from . import learned, problems


def grf_device(shape, corr_length: float, sigma: float, seed: int, cell_size: float) -> np.ndarray:
    """Squared-exponential Gaussian random field by spectral synthesis on a periodic grid twice the
    size (the method of ``fem.gaussian_random_field``), drawn and transformed on the GPU."""
    gen = torch.Generator(device="cuda").manual_seed(int(seed))
    ext = [2 * s for s in shape]
    freqs = torch.meshgrid(*[torch.fft.fftfreq(n, d=cell_size, device="cuda", dtype=torch.float64) for n in ext],
                           indexing="ij")
    k2 = sum(f * f for f in freqs)
    amp = torch.exp(-math.pi ** 2 * corr_length ** 2 * k2)  # sqrt of exp(-2 pi^2 l^2 k^2)
    noise = torch.randn(ext, generator=gen, device="cuda", dtype=torch.float64)
    field = torch.fft.ifftn(torch.fft.fftn(noise) * amp).real[tuple(slice(0, s) for s in shape)]
    field = (field - field.mean()) / (field.std() + 1e-300) * sigma
    return field.reshape(-1).cpu().numpy()


def make_field(res: int, seed: int, sigma: float = learned.SIGMA_DEFAULT, corr_length: float = 0.1,
               cell_size: float = 1.0 / 96):
    g = grf_device((res, res, res), corr_length, sigma, seed, cell_size)
    return problems.diffusion((res, res, res), seed=seed, coef=np.exp(g))


def make_elasticity_field(res: int, seed: int, sigma: float = learned.SIGMA_DEFAULT, corr_length: float = 0.05,
                          cell_size: float = 1.0 / 128):
    """Q1 vec3 elasticity on res^3 cells whose lognormal Young's modulus has the statistics of the 128^3
    unit-cube configuration (correlation length corr_length on cells of size 1/128), x = 0 clamped."""
    return problems.elasticity((res, res, res), sigma=sigma, corr_length=corr_length / (cell_size * res), seed=seed)


def train(fields: int = 2000, res: int = 48, steps_per_field: int = 2, batch: int = 6, lr: float = 2e-3,
          lr_min: float = 1e-4, seed0: int = 10_000, eval_every: int = 250, out: str | None = None, log=print,
          net: learned.ConvNet | None = None, max_minutes: float | None = None,
          problem: str = "diffusion", fcg_rhs: int = 0, coarsest_nodes: int = 400) -> learned.ConvNet:
    if problem not in ("diffusion", "elasticity"):
        raise ValueError("problem: diffusion or elasticity")
    field_of = make_field if problem == "diffusion" else make_elasticity_field
    if net is None:
        net = learned.ConvNet(seed=0, ncomp=1 if problem == "diffusion" else 3)
        if problem == "elasticity":  # E = 1e3 exp(g), g ~ N(0, sigma^2)
            net.mean_log, net.inv_std = math.log(1e3), 1.0 / learned.SIGMA_DEFAULT
    tr = learned.SmootherTrainer(net, lr=lr, coarsest_nodes=coarsest_nodes)
    rng = np.random.default_rng(seed0)
    held = tr.field(field_of(res, seed=seed0 - 1))
    held_pairs = learned.slow_pairs(held, 2, np.random.default_rng(1), smoother=None)
    base = np.mean([tr.eval_loss(held, r, e, None) for r, e in held_pairs])
    log(f"held-out field: Jacobi-smoothed V-cycle loss {base:.5f}")
    total = fields * steps_per_field
    step = 0
    t0 = time.time()
    hist = []
    for k in range(fields):
        f = tr.field(field_of(res, seed=seed0 + k))
        pairs = (learned.cg_pairs(f, 1, rng, iters=(0, 2, 8, 32))
                 + learned.slow_pairs(f, 1, rng, sweeps=(1, 2, 4))
                 + learned.slow_pairs(f, 1, rng, sweeps=(2,), smoother=None))
        if fcg_rhs:  # residuals of the flexible solver the network serves, with the current network
            pairs += learned.fcg_pairs(f, fcg_rhs, rng)
        for _ in range(steps_per_field):
            tr.lr = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * step / max(total - 1, 1)))
            idx = rng.choice(len(pairs), size=min(batch, len(pairs)), replace=False)
            hist.append(tr.step(f, [pairs[i] for i in idx]))
            step += 1
        out_of_time = max_minutes is not None and time.time() - t0 > 60.0 * max_minutes
        if (k + 1) % eval_every == 0 or k + 1 == fields or out_of_time:
            got = np.mean([tr.eval_loss(held, r, e, held.sm) for r, e in held_pairs])
            kept = [h for h in hist[-eval_every:] if abs(h) <= tr.MAX_BATCH_LOSS]
            skipped = getattr(tr, "skipped_steps", 0)
            log(f"fields {k + 1}/{fields}  train loss {np.mean(kept) if kept else float('nan'):.5f}  held-out {got:.5f} "
                f"(Jacobi {base:.5f})  {time.time() - t0:.0f}s" + (f"  ({skipped} degenerate batches skipped)" if skipped else ""))
            if out:
                net.save(out, fields=k + 1, res=res, held_out_loss=got, jacobi_loss=base)
        if out_of_time:
            log(f"stopped after {k + 1} fields (time limit)")
            break
    return net


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--fields", type=int, default=2000)
    ap.add_argument("--res", type=int, default=48)
    ap.add_argument("--steps-per-field", type=int, default=2)
    ap.add_argument("--batch", type=int, default=6)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--eval-every", type=int, default=250)
    ap.add_argument("--out", default=learned.DEFAULT_WEIGHTS)
    ap.add_argument("--max-minutes", type=float, default=None)
    ap.add_argument("--problem", choices=["diffusion", "elasticity"], default="diffusion")
    ap.add_argument("--fcg-rhs", type=int, default=0,
                    help="right-hand sides per field whose flexible-CG residuals (current network) join the pairs")
    ap.add_argument("--init", default=None, help="start from these weights instead of a fresh network")
    ap.add_argument("--cycle-omega", default=None,
                    help="Jacobi damping of the training (and serving) cycle: a number, or 'auto' for the "
                         "hierarchy's per-level estimate (default: the network's own, 0.6 for scalar fields)")
    ap.add_argument("--coarsest-nodes", type=int, default=400, help="coarsest level of the training hierarchy")
    a = ap.parse_args()
    import os

    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    net = learned.ConvNet.load(a.init) if a.init else None
    if a.cycle_omega is not None:
        if net is None:
            net = learned.ConvNet(seed=0, ncomp=1 if a.problem == "diffusion" else 3)
            if a.problem == "elasticity":  # E = 1e3 exp(g), g ~ N(0, sigma^2)
                net.mean_log, net.inv_std = math.log(1e3), 1.0 / learned.SIGMA_DEFAULT
        net.cycle_omega = None if a.cycle_omega == "auto" else float(a.cycle_omega)
    train(a.fields, a.res, a.steps_per_field, a.batch, a.lr, eval_every=a.eval_every, out=a.out,
          log=lambda m: print(m, flush=True), max_minutes=a.max_minutes, problem=a.problem, fcg_rhs=a.fcg_rhs,
          net=net, coarsest_nodes=a.coarsest_nodes)


if __name__ == "__main__":
    main()
