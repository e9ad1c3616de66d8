"""GPU tests of the learned smoother: conv-net kernels against the CPU oracle, the training
gradient through the V-cycle against the oracle's chain gradient, and the trained network's gain."""

import numpy as np
import pytest
import torch

from oracle import convnet as C

pytestmark = pytest.mark.gpu

STREAM = lambda: torch.cuda.current_stream().cuda_stream  # noqa: E731


def _dev(a, dtype=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dtype).cuda()


@pytest.mark.parametrize("dims,ci,co,relu", [((7, 9, 11), 16, 16, True), ((5, 4, 33), 16, 1, False),
                                             ((3, 3, 3), 9, 16, False)])
def test_conv3_f32_kernels_match_oracle(cuda, dims, ci, co, relu):
    import warp_gb300._native as N

    L = N.lib()
    rng = np.random.default_rng(0)
    n = int(np.prod(dims))
    x = rng.standard_normal((n, ci)).astype(np.float32)
    W = (rng.standard_normal((27, ci, co)) * 0.3).astype(np.float32)
    g = rng.standard_normal((n, co)).astype(np.float32)
    xd, Wd, gd = _dev(x), _dev(W), _dev(g)
    y = torch.empty(n * co, device="cuda")
    N.check(L.gb_conv3_fwd_f32(*dims, ci, co, xd.data_ptr(), Wd.data_ptr(), int(relu), y.data_ptr(), STREAM()))
    ref = C.conv3_fwd(dims, x, W, relu)
    np.testing.assert_allclose(y.cpu().numpy().reshape(n, co), ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    gin = torch.empty(n * ci, device="cuda")
    N.check(L.gb_conv3_bwd_data_f32(*dims, ci, co, gd.data_ptr(), Wd.data_ptr(), gin.data_ptr(), STREAM()))
    ref = C.conv3_bwd_data(dims, g, W)
    np.testing.assert_allclose(gin.cpu().numpy().reshape(n, ci), ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    ws = torch.empty(L.gb_conv3_bwd_weight_workspace_bytes(*dims, ci, co), dtype=torch.uint8, device="cuda")
    gW = torch.full((27 * ci * co,), 0.5, device="cuda")  # accumulates
    N.check(L.gb_conv3_bwd_weight_f32(*dims, ci, co, xd.data_ptr(), gd.data_ptr(), gW.data_ptr(), ws.data_ptr(),
                                      ws.numel(), STREAM()))
    ref = C.conv3_bwd_weight(dims, x, g, ci, co) + 0.5
    np.testing.assert_allclose(gW.cpu().numpy().reshape(27, ci, co), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())


def test_conv3_bwd_weight_is_deterministic(cuda):
    import warp_gb300._native as N

    L = N.lib()
    dims = (40, 40, 40)
    n = 40 ** 3
    rng = np.random.default_rng(1)
    x, g = _dev(rng.standard_normal((n, 16))), _dev(rng.standard_normal((n, 16)))
    ws = torch.empty(L.gb_conv3_bwd_weight_workspace_bytes(*dims, 16, 16), dtype=torch.uint8, device="cuda")
    outs = []
    for _ in range(2):
        gW = torch.zeros(27 * 256, device="cuda")
        N.check(L.gb_conv3_bwd_weight_f32(*dims, 16, 16, x.data_ptr(), g.data_ptr(), gW.data_ptr(), ws.data_ptr(),
                                          ws.numel(), STREAM()))
        outs.append(gW.cpu())
    assert torch.equal(outs[0], outs[1])


def test_adam_kernel_matches_oracle(cuda):
    import warp_gb300._native as N

    rng = np.random.default_rng(2)
    w0 = rng.standard_normal(1000).astype(np.float32)
    w, m, v = _dev(w0), torch.zeros(1000, device="cuda"), torch.zeros(1000, device="cuda")
    wr, mr, vr = w0.astype(np.float64), np.zeros(1000), np.zeros(1000)
    for step in range(1, 8):
        g = rng.standard_normal(1000).astype(np.float32)
        gd = _dev(g)
        N.check(N.lib().gb_adam_step(1000, w.data_ptr(), gd.data_ptr(), m.data_ptr(), v.data_ptr(), 1e-2, 0.9, 0.999,
                                     1e-8, step, None, STREAM()))
        wr, mr, vr = C.adam(wr, g.astype(np.float64), mr, vr, 1e-2, 0.9, 0.999, 1e-8, step)
    np.testing.assert_allclose(w.cpu().numpy(), wr, rtol=1e-5, atol=1e-6)


def _bf16_round(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16).float().numpy()


# (1, 1, 1) and (2, 4, 16): one x-plane, runs of one plane (the MMAs of the first and last input planes
# feed one output plane only); (64, 40, 40) and (300, 10, 10): more work items (columns x planes) than
# CTAs, so CTAs walk runs of x-planes, cross column boundaries and wrap their TMEM chunk ring many
# times; (160, 4, 300) and (160, 3, 450): long z rows shrink the shared-memory ring of x-plane blocks
@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 4, 16), (7, 9, 11), (9, 7, 35), (33, 17, 20), (20, 12, 97),
                                  (64, 40, 40), (300, 10, 10), (160, 4, 300), (160, 3, 450)])
def test_conv3_tcgen05_layer_matches_oracle(cuda, dims):
    """tcgen05 implicit-GEMM layer on the planar padded layout: equal to the oracle on bf16-rounded
    operands up to output rounding; border rows stay zero; no device status raised."""
    import warp_gb300._native as N
    from warp_gb300 import learned

    rng = np.random.default_rng(9)
    n = int(np.prod(dims))
    x = _bf16_round(rng.standard_normal((n, 16)))
    W = _bf16_round(rng.standard_normal((27, 16, 16)) * 0.2)
    src = learned.to_planar(_dev(x), dims)
    dst = torch.zeros_like(src)
    Wt = _dev(W.transpose(0, 2, 1), torch.bfloat16)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(N.lib().gb_conv3_fwd_tc(*dims, 0, src.data_ptr(), Wt.data_ptr(), dst.data_ptr(), None, None, None, None,
                                    0.0, status.data_ptr(), STREAM()))
    got = learned.from_planar(dst, dims).float().cpu().numpy()
    ref = C.conv3_fwd(dims, x, W, True)
    np.testing.assert_allclose(got, ref, rtol=8e-3, atol=1e-3 * max(np.abs(ref).max(), 1e-30))
    border = torch.ones(dst.shape[1], dtype=torch.bool, device="cuda")
    border[learned.padded_rows(dims, "cuda")] = False
    assert not dst[:, border].any()
    assert int(status.item()) == 0


@pytest.mark.parametrize("dims", [(5, 6, 7), (24, 25, 25), (64, 40, 40)])
def test_conv3_tcgen05_last_layer_fuses_jacobi_step(cuda, dims):
    import warp_gb300._native as N
    from warp_gb300 import learned

    rng = np.random.default_rng(10)
    n = int(np.prod(dims))
    x = _bf16_round(rng.standard_normal((n, 16)))
    W = np.zeros((27, 16, 16), np.float32)
    W[:, :, 0] = _bf16_round(rng.standard_normal((27, 16)) * 0.2)
    r = rng.standard_normal(n).astype(np.float32)
    dinv = rng.uniform(0.5, 2, n).astype(np.float32)
    mask = (rng.uniform(size=n) < 0.2).astype(np.float32)
    src = learned.to_planar(_dev(x), dims)
    Wt = _dev(W.transpose(0, 2, 1), torch.bfloat16)
    w = torch.full((n,), float("nan"), device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rd, dd, md = _dev(r), _dev(dinv), _dev(mask)  # keep the device copies alive across the launch
    N.check(N.lib().gb_conv3_fwd_tc(*dims, 1, src.data_ptr(), Wt.data_ptr(), None, w.data_ptr(), rd.data_ptr(),
                                    dd.data_ptr(), md.data_ptr(), 0.6, status.data_ptr(), STREAM()))
    out0 = C.conv3_fwd(dims, x, W)[:, 0]
    ref = C.combine(out0, mask, 0.6, dinv, r)
    np.testing.assert_allclose(w.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
    assert int(status.item()) == 0


def test_features_and_combine_match_oracle(cuda):
    import warp_gb300._native as N

    L = N.lib()
    dims = (6, 7, 8)
    n = int(np.prod(dims))
    rng = np.random.default_rng(4)
    coef = np.exp(rng.standard_normal(5 * 6 * 7)).astype(np.float32)
    chat = torch.empty(n * 8, device="cuda")
    N.check(L.gb_net_cell_features(*dims, _dev(coef).data_ptr(), 0.1, 0.5, chat.data_ptr(), STREAM()))
    ref_chat = C.node_cell_features(dims, coef, 0.1, 0.5)
    np.testing.assert_allclose(chat.cpu().numpy().reshape(n, 8), ref_chat, rtol=1e-5, atol=1e-6)
    r = rng.standard_normal(n).astype(np.float32)
    dinv = rng.uniform(0.5, 2, n).astype(np.float32)
    mask = (rng.uniform(size=n) < 0.2).astype(np.float32)
    rd, dd, md = _dev(r), _dev(dinv), _dev(mask)
    f = torch.empty(n * 16, device="cuda")
    N.check(L.gb_net_features(N.GB_F32, 1, n, rd.data_ptr(), dd.data_ptr(), chat.data_ptr(), md.data_ptr(), f.data_ptr(),
                              STREAM()))
    ref_f = C.features(r, dinv, ref_chat, mask)
    np.testing.assert_allclose(f.cpu().numpy().reshape(n, 16), ref_f, rtol=1e-5, atol=1e-6)
    fb = torch.empty(n * 16, dtype=torch.bfloat16, device="cuda")
    N.check(L.gb_net_features(N.GB_BF16, 1, n, rd.data_ptr(), dd.data_ptr(), chat.data_ptr(), md.data_ptr(),
                              fb.data_ptr(), STREAM()))
    np.testing.assert_allclose(fb.float().cpu().numpy().reshape(n, 16), ref_f, rtol=8e-3, atol=1e-6)
    act = rng.standard_normal(n).astype(np.float32)
    out = torch.empty(n, device="cuda")
    N.check(L.gb_net_combine(N.GB_F32, 1, n, 1, _dev(act).data_ptr(), md.data_ptr(), 0.6, dd.data_ptr(), rd.data_ptr(),
                             out.data_ptr(), STREAM()))
    np.testing.assert_allclose(out.cpu().numpy(), C.combine(act, mask, 0.6, dinv, r), rtol=1e-5, atol=1e-6)


def _hierarchy_on_host(mg):
    import scipy.sparse as sp

    As, dinvs, masks, Ps = [], [], [], []
    for lv in mg.levels:
        nnz = lv.A.nnz_sync()
        off = lv.A.offsets.cpu().numpy()
        col = lv.A.columns[:nnz].cpu().numpy()
        val = lv.A.values[:nnz].reshape(-1).double().cpu().numpy()
        As.append(sp.csr_matrix((val, col, off), shape=(lv.n, lv.n)))
        dinvs.append(lv.dinv.double().cpu().numpy())
        masks.append(lv.mask.double().cpu().numpy())
    for i in range(len(mg.levels) - 1):
        Ps.append(C.prolongation(mg.levels[i].dims, mg.levels[i + 1].dims, masks[i], masks[i + 1]))
    inv = mg.levels[-1].inv.double().cpu().numpy()
    return C.Hierarchy(As, dinvs, masks, Ps, inv, mg.omega)


def test_training_gradient_matches_oracle_chain(cuda):
    """The GPU loss and dLoss/dW through the whole V-cycle equal the float64 oracle's."""
    from warp_gb300 import learned, problems

    s = problems.diffusion((16, 16, 16), sigma=1.5, corr_length=0.3, seed=5)
    net = learned.ConvNet(seed=1)
    gen = torch.Generator().manual_seed(7)
    net.W[3] = (torch.randn(net.W[3].numel(), generator=gen) * 0.05).cuda()
    tr = learned.SmootherTrainer(net)
    f = tr.field(s)
    assert len(f.mg.levels) == 3
    rng = np.random.default_rng(6)
    keep = (1 - f.mg.levels[0].mask).cpu().numpy()
    H = _hierarchy_on_host(f.mg)
    pairs_h, pairs_d = [], []
    for _ in range(2):
        e = rng.standard_normal(f.n) * keep
        r = H.As[0] @ e
        pairs_h.append((r, e))
        pairs_d.append((_dev(r), _dev(e)))
    net.zero_grad()
    losses = [tr.loss_and_grad(f, r, e, 0.5) for r, e in pairs_d]
    loss = float(torch.stack(losses).mean())
    chat = f.sm.chat.double().cpu().numpy().reshape(-1, 8)
    Ws = [w.double().cpu().numpy().reshape(27, ci, co) for w, (ci, co, _) in zip(net.W, learned.LAYERS)]
    ref_loss, ref_g = C.smoother_chain(H, f.mg.levels[0].dims, chat, Ws, [True, True, True, False], pairs_h)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    for li, (g, (ci, co, _)) in enumerate(zip(net.gW, learned.LAYERS)):
        got = g.double().cpu().numpy().reshape(27, ci, co)
        scale = np.abs(ref_g[li]).max()
        assert scale > 0
        assert np.abs(got - ref_g[li]).max() <= 5e-3 * scale, f"layer {li}"


def test_learned_smoother_inference_matches_training_forward(cuda):
    """The bf16 tensor-core smoother equals the fp32 training forward up to bf16 rounding."""
    from warp_gb300 import learned, problems

    s = problems.diffusion((24, 24, 24), sigma=1.5, corr_length=0.2, seed=8)
    net = learned.ConvNet(seed=2)
    net.W[3] = (torch.randn(net.W[3].numel(), generator=torch.Generator().manual_seed(3)) * 0.05).cuda()
    tr = learned.SmootherTrainer(net)
    f = tr.field(s)
    r = torch.randn(f.n, device="cuda") * (1 - f.mg.levels[0].mask)
    w32 = torch.empty_like(r)
    f.sm.launch(STREAM(), r.data_ptr(), w32.data_ptr())
    inf = learned.LearnedSmoother(net, f.mg, s.coef)
    w16 = torch.empty_like(r)
    inf.launch(STREAM(), r.data_ptr(), w16.data_ptr())
    err = float((w16 - w32).norm() / w32.norm())
    assert err < 2e-2, err
    assert int(f.mg.status.item()) == 0


def _train_small(net, seeds, steps, res=24, lr=2e-3):
    from warp_gb300 import learned, problems

    tr = learned.SmootherTrainer(net, lr=lr)
    rng = np.random.default_rng(0)
    fields = []
    for sd in seeds:
        s = learned.training_problem(res, seed=sd)
        f = tr.field(s)
        fields.append([f, learned.cg_pairs(f, 1, rng) + learned.slow_pairs(f, 2, rng, smoother=None)])
    for k in range(steps):
        f, pairs = fields[k % len(fields)]
        idx = rng.choice(len(pairs), size=min(6, len(pairs)), replace=False)
        tr.step(f, [pairs[i] for i in idx])
        if k % 100 == 99:  # refresh the slow modes with the current network
            for item in fields:
                item[1] = item[1][:8] + learned.slow_pairs(item[0], 2, rng)
    return tr


def test_trained_network_gains_over_jacobi_smoothing(cuda):
    """Training on a few seeded fields lowers the held-out V-cycle error and the number of flexible-CG
    iterations against the same V-cycle with Jacobi pre-smoothing."""
    from warp_gb300 import learned, multigrid
    from warp_gb300.optim import linear

    net = learned.ConvNet(seed=0)
    tr = _train_small(net, seeds=range(100, 108), steps=400)
    test = learned.training_problem(24, seed=999)
    f = tr.field(test)
    rng = np.random.default_rng(11)
    pairs = learned.slow_pairs(f, 2, rng, smoother=None)
    base = np.mean([tr.eval_loss(f, r, e, None) for r, e in pairs])
    inf = learned.LearnedSmoother(net, f.mg, test.coef)
    got = np.mean([tr.eval_loss(f, r, e, inf) for r, e in pairs])
    assert got < 0.6 * base, (got, base)
    # flexible CG with the plain and the learned V-cycle on the held-out right-hand side, both in the
    # hierarchy and damping the network was trained in
    iters = {}
    for name, sm in (("jacobi", None), ("learned", inf)):
        mg = multigrid.MultigridPreconditioner(test.A, test.geo, test.coef, coarsest_nodes=400, omega=net.cycle_omega)
        mg.smoother = sm if sm is None else learned.LearnedSmoother(net, mg, test.coef)
        x = torch.zeros_like(test.b)
        it, err, atol = linear.fcg(test.A, test.b, x, tol=1e-7, atol=0.0, maxiter=100, M=mg, check_every=1)
        iters[name] = it
    assert iters["learned"] < iters["jacobi"], iters


def test_vec3_features_combine_and_last_layer_match_oracle(cuda):
    """Vec3 (elasticity) pieces of the smoother: features (fp32 and the planar bf16 layout), the combine
    step, and the tcgen05 last layer with three outputs fused with the per-dof Jacobi step."""
    import warp_gb300._native as N
    from warp_gb300 import learned

    L = N.lib()
    dims = (9, 7, 11)
    n = int(np.prod(dims))
    rng = np.random.default_rng(14)
    coef = np.exp(rng.standard_normal(8 * 6 * 10)).astype(np.float32)
    chat = torch.empty(n * 8, device="cuda")
    N.check(L.gb_net_cell_features(*dims, _dev(coef).data_ptr(), 0.1, 0.5, chat.data_ptr(), STREAM()))
    chat_h = chat.cpu().numpy().reshape(n, 8)
    r = rng.standard_normal(3 * n).astype(np.float32)
    dinv = rng.uniform(0.5, 2, 3 * n).astype(np.float32)
    mask = (rng.uniform(size=n) < 0.2).astype(np.float32)
    rd, dd, md = _dev(r), _dev(dinv), _dev(mask)
    f = torch.empty(n * 16, device="cuda")
    N.check(L.gb_net_features(N.GB_F32, 3, n, rd.data_ptr(), dd.data_ptr(), chat.data_ptr(), md.data_ptr(),
                              f.data_ptr(), STREAM()))
    ref_f = C.features_vec3(r, dinv, chat_h, mask)
    np.testing.assert_allclose(f.cpu().numpy().reshape(n, 16), ref_f, rtol=1e-5, atol=1e-6)
    planar = torch.zeros(2 * learned.planar_rows(dims) * 8, dtype=torch.bfloat16, device="cuda")
    N.check(L.gb_net_features_planar(3, *dims, rd.data_ptr(), dd.data_ptr(), chat.data_ptr(), md.data_ptr(),
                                     planar.data_ptr(), STREAM()))
    got = learned.from_planar(planar.view(2, -1, 8), dims).float().cpu().numpy()
    np.testing.assert_allclose(got, ref_f, rtol=8e-3, atol=1e-6)
    act = rng.standard_normal((n, 3)).astype(np.float32)
    out = torch.empty(3 * n, device="cuda")
    N.check(L.gb_net_combine(N.GB_F32, 3, n, 3, _dev(act).data_ptr(), md.data_ptr(), 0.4, dd.data_ptr(), rd.data_ptr(),
                             out.data_ptr(), STREAM()))
    np.testing.assert_allclose(out.cpu().numpy(), C.combine_vec3(act, mask, 0.4, dinv, r), rtol=1e-5, atol=1e-6)
    # last layer, three outputs
    x = _bf16_round(rng.standard_normal((n, 16)))
    W = np.zeros((27, 16, 16), np.float32)
    W[:, :, :3] = _bf16_round(rng.standard_normal((27, 16, 3)) * 0.2)
    src = learned.to_planar(_dev(x), dims)
    Wt = _dev(W.transpose(0, 2, 1), torch.bfloat16)
    w = torch.full((3 * n,), float("nan"), device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(L.gb_conv3_fwd_tc(*dims, 3, src.data_ptr(), Wt.data_ptr(), None, w.data_ptr(), rd.data_ptr(),
                              dd.data_ptr(), md.data_ptr(), 0.4, status.data_ptr(), STREAM()))
    out3 = C.conv3_fwd(dims, x, W)[:, :3]
    ref = C.combine_vec3(out3, mask, 0.4, dinv, r)
    np.testing.assert_allclose(w.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
    assert int(status.item()) == 0


def test_vec3_training_gradient_matches_a_directional_difference(cuda):
    """The vec3 trainer's dLoss/dW through the elasticity V-cycle agrees with a central difference of the
    loss along a random weight direction, and the bf16 tcgen05 smoother equals the fp32 training forward up
    to bf16 rounding."""
    from warp_gb300 import learned, problems

    s = problems.elasticity((12, 12, 12), sigma=1.0, corr_length=0.3, seed=3)
    net = learned.ConvNet(seed=2, ncomp=3)
    gen = torch.Generator().manual_seed(5)
    net.W[3] = (torch.randn(net.W[3].numel(), generator=gen) * 0.05).cuda()
    tr = learned.SmootherTrainer(net)
    f = tr.field(s)
    assert f.bdim == 3 and f.n == 3 * 13 ** 3
    rng = np.random.default_rng(0)
    e = torch.from_numpy(rng.standard_normal(f.n).astype(np.float32)).cuda() * (1 - f.mask_dof)
    r = torch.zeros_like(e)
    learned._spmv(s.A, e, r, 1.0, 0.0, STREAM(), f.mg.status)
    net.zero_grad()
    tr.loss_and_grad(f, r, e)
    torch.cuda.synchronize()
    dirs = [torch.randn(w.numel(), generator=gen).cuda() for w in net.W]
    analytic = sum(float((g * d).sum()) for g, d in zip(net.gW, dirs))
    eps = 5e-4
    W0 = [w.clone() for w in net.W]

    def loss_at(t):
        for w, w0, d in zip(net.W, W0, dirs):
            w.copy_(w0 + t * d)
        return tr.eval_loss(f, r, e, f.sm)

    fd = (loss_at(eps) - loss_at(-eps)) / (2 * eps)
    for w, w0 in zip(net.W, W0):
        w.copy_(w0)
    assert abs(fd - analytic) <= 0.05 * abs(analytic) + 1e-6, (fd, analytic)
    # inference smoother (bf16 tcgen05 layers, 3 outputs) against the fp32 training forward
    rr = torch.randn(f.n, device="cuda") * (1 - f.mask_dof)
    w32 = torch.empty_like(rr)
    f.sm.launch(STREAM(), rr.data_ptr(), w32.data_ptr())
    inf = learned.LearnedSmoother(net, f.mg, s.coef)
    w16 = torch.empty_like(rr)
    inf.launch(STREAM(), rr.data_ptr(), w16.data_ptr())
    err = float((w16 - w32).norm() / w32.norm())
    assert err < 2e-2, err
    assert int(f.mg.status.item()) == 0


@pytest.mark.parametrize("cells,vec3", [((8, 8, 8), False), ((40, 40, 40), False), ((31, 18, 47), False),
                                        ((96, 96, 96), False), ((16, 16, 16), True)])
def test_whole_network_launch_matches_layer_launches(cuda, cells, vec3):
    """One cooperative launch of the features and the four layers writes, bit for bit, what the features
    kernel and four layer launches write: over several launches sharing the counters (a new residual
    each time) and inside a CUDA graph replayed twice."""
    from warp_gb300 import learned, multigrid, problems

    if vec3:
        s = problems.elasticity(cells, sigma=1.0, corr_length=0.3, seed=4)
    else:
        s = problems.diffusion(cells, sigma=1.5, corr_length=0.2, seed=6)
    net = learned.ConvNet(seed=3, ncomp=3 if vec3 else 1)
    net.W[3] = (torch.randn(net.W[3].numel(), generator=torch.Generator().manual_seed(4)) * 0.05).cuda()
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef, **({"faces": ("x-",)} if vec3 else {}))
    layered = learned.LearnedSmoother(net, mg, s.coef, launches=5)
    whole = learned.LearnedSmoother(net, mg, s.coef, launches=1)
    two = learned.LearnedSmoother(net, mg, s.coef, launches=2)
    assert whole.whole_network and whole.kernels_per_apply == 1 and layered.kernels_per_apply == 5
    assert two.whole_network and two.kernels_per_apply == 2
    n = layered.n * (3 if vec3 else 1)
    gen = torch.Generator(device="cuda").manual_seed(1)
    for trial in range(3):
        r = torch.randn(n, device="cuda", generator=gen)
        w_ref = torch.full_like(r, float("nan"))
        w = torch.full_like(r, float("nan"))
        w2 = torch.full_like(r, float("nan"))
        layered.launch(STREAM(), r.data_ptr(), w_ref.data_ptr())
        whole.launch(STREAM(), r.data_ptr(), w.data_ptr())
        two.launch(STREAM(), r.data_ptr(), w2.data_ptr())
        torch.cuda.synchronize()
        assert int(mg.status.item()) == 0
        assert torch.isfinite(w_ref).all()
        assert torch.equal(w, w_ref), f"launch {trial}: max diff {float((w - w_ref).abs().max())}"
        assert torch.equal(w2, w_ref), f"launch {trial}: max diff {float((w2 - w_ref).abs().max())}"
    assert int(whole.epoch[0].item()) == 3 and int(whole.epoch[1].item()) == 0
    assert int(two.epoch[0].item()) == 3
    # graph capture: the counters live on the device, so replays keep advancing the epoch
    r = torch.randn(n, device="cuda", generator=gen)
    w_ref = torch.empty_like(r)
    layered.launch(STREAM(), r.data_ptr(), w_ref.data_ptr())
    w = torch.full_like(r, float("nan"))
    s_cap = torch.cuda.Stream()
    s_cap.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s_cap):
        with torch.cuda.graph(g, stream=s_cap):
            whole.launch(s_cap.cuda_stream, r.data_ptr(), w.data_ptr())
    torch.cuda.current_stream().wait_stream(s_cap)
    for _ in range(2):
        w.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(w, w_ref)
    assert int(whole.epoch[0].item()) == 5
    assert int(mg.status.item()) == 0


def test_whole_network_launch_times_out_when_counters_never_reach(cuda):
    """A dependency that is never met ends the whole-network launch through its bounded waits: the status
    word gets DEV_WAIT_TIMEOUT and the call returns; the next launch with fresh counters is right again."""
    import warp_gb300._native as N
    from warp_gb300 import learned, multigrid, problems

    s = problems.diffusion((16, 16, 16), sigma=1.5, corr_length=0.2, seed=6)
    net = learned.ConvNet(seed=3)
    net.W[3] = (torch.randn(net.W[3].numel(), generator=torch.Generator().manual_seed(4)) * 0.05).cuda()
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    layered = learned.LearnedSmoother(net, mg, s.coef, launches=5)
    two = learned.LearnedSmoother(net, mg, s.coef, launches=2)
    r = torch.randn(layered.n, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    w_ref, w = torch.empty_like(r), torch.empty_like(r)
    layered.launch(STREAM(), r.data_ptr(), w_ref.data_ptr())
    torch.cuda.synchronize()
    assert int(mg.status.item()) == 0
    two.flags.fill_(-4096)  # far below every stage's expected count: layer 1 can never be staged
    two.launch(STREAM(), r.data_ptr(), w.data_ptr())
    torch.cuda.synchronize()
    assert int(mg.status.item()) & N.DEV_WAIT_TIMEOUT
    mg.status.zero_()
    two.flags.zero_()
    two.epoch.zero_()
    two.launch(STREAM(), r.data_ptr(), w.data_ptr())
    torch.cuda.synchronize()
    assert int(mg.status.item()) == 0
    assert torch.equal(w, w_ref)
