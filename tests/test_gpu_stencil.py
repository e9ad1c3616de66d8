"""GPU tests of the 27-point stencil form of the multigrid level operators (gb_st27_build /
gb_st27_apply): every mode against a float64 product of the same CSR matrix, the out-of-stencil
flag, and the V-cycle / flexible-CG solve against the CSR kernels."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _system(dims_cells, seed):
    from warp_gb300 import problems

    return problems.diffusion(dims_cells, sigma=1.5, corr_length=0.2, seed=seed)


def _csr(Am):
    n = Am.nrow
    nnz = Am.nnz_sync()
    off = Am.offsets.cpu().numpy().astype(np.int64)
    col = Am.columns[:nnz].cpu().numpy().astype(np.int64)
    val = Am.values[:nnz].cpu().numpy().astype(np.float64)
    return n, off, col, val


def _matvec(off, col, val, x):
    y = np.zeros(len(off) - 1)
    rows = np.repeat(np.arange(len(off) - 1), np.diff(off))
    np.add.at(y, rows, val * x[col])
    return y


@pytest.mark.parametrize("cells", [(6, 5, 4), (9, 7, 12), (1, 3, 2)])
def test_st27_modes_match_csr_product(cuda, cells):
    from warp_gb300 import _native as N

    s = _system(cells, seed=3)
    dims = tuple(c + 1 for c in cells)
    n, off, col, val = _csr(s.A)
    assert n == int(np.prod(dims))
    L = N.lib()
    S = torch.empty(int(L.gb_st27_bytes(*dims)) // 4, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(L.gb_st27_build(*dims, s.A.offsets.data_ptr(), s.A.columns.data_ptr(), s.A.values.data_ptr(),
                            S.data_ptr(), status.data_ptr(), 0))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    rng = np.random.default_rng(1)
    r = rng.standard_normal(n).astype(np.float32)
    w = rng.standard_normal(n).astype(np.float32)
    d = np.zeros(n)
    rows = np.repeat(np.arange(n), np.diff(off))
    d[rows[col == rows]] = val[col == rows]
    dinv = (1.0 / d).astype(np.float32)
    omega = 0.6
    rt, wt, dt = (torch.from_numpy(a).cuda() for a in (r, w, dinv))
    out = torch.empty_like(rt)
    w_out = torch.empty_like(rt)
    scale = np.abs(val).max() * np.abs(w).max() * 27
    # mode 0: r - A w
    st = status.data_ptr()
    N.check(L.gb_st27_apply(0, *dims, S.data_ptr(), wt.data_ptr(), rt.data_ptr(), None, omega, None, out.data_ptr(), st,
                            0))
    ref = r - _matvec(off, col, val, w.astype(np.float64))
    np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-5 * scale, rtol=1e-5)
    # mode 1: w = omega D^-1 r, r - A w
    N.check(L.gb_st27_apply(1, *dims, S.data_ptr(), None, rt.data_ptr(), dt.data_ptr(), omega, w_out.data_ptr(),
                            out.data_ptr(), st, 0))
    w1 = omega * dinv.astype(np.float64) * r
    np.testing.assert_allclose(w_out.cpu().numpy(), w1, rtol=1e-6, atol=1e-7)
    ref = r - _matvec(off, col, val, w1)
    np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-5 * scale, rtol=1e-5)
    # mode 2: w + omega D^-1 (r - A w)
    N.check(L.gb_st27_apply(2, *dims, S.data_ptr(), wt.data_ptr(), rt.data_ptr(), dt.data_ptr(), omega, None,
                            out.data_ptr(), st, 0))
    ref = w + omega * dinv * (r - _matvec(off, col, val, w.astype(np.float64)))
    np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-5 * scale * np.abs(dinv).max(), rtol=1e-5)
    assert int(status.item()) == 0


def test_st27_build_flags_entries_outside_the_stencil(cuda):
    from warp_gb300 import _native as N
    from warp_gb300 import sparse

    dims = (4, 4, 4)
    n = 64
    rows = np.concatenate([np.arange(n), [5]]).astype(np.int32)
    cols = np.concatenate([np.arange(n), [5 + 2 * 16]]).astype(np.int32)  # two x-slabs away
    vals = np.ones(n + 1, np.float32)
    Am = sparse.bsr_zeros(n, n, torch.float32)
    sparse.bsr_set_from_triplets(Am, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(),
                                 torch.from_numpy(vals).cuda())
    L = N.lib()
    S = torch.empty(int(L.gb_st27_bytes(*dims)) // 4, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(L.gb_st27_build(*dims, Am.offsets.data_ptr(), Am.columns.data_ptr(), Am.values.data_ptr(), S.data_ptr(),
                            status.data_ptr(), 0))
    torch.cuda.synchronize()
    assert int(status.item()) == 1


def test_st27_rejects_aliasing_and_bad_mode(cuda):
    from warp_gb300 import _native as N

    L = N.lib()
    x = torch.zeros(27 * 8, device="cuda")
    v = torch.zeros(8, device="cuda")
    o = torch.zeros(8, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.gb_st27_apply(0, 2, 2, 2, x.data_ptr(), v.data_ptr(), v.data_ptr(), None, 0.6, None, v.data_ptr(),
                           st.data_ptr(), 0) != 0
    assert L.gb_st27_apply(7, 2, 2, 2, x.data_ptr(), v.data_ptr(), v.data_ptr(), v.data_ptr(), 0.6, None, o.data_ptr(),
                           st.data_ptr(), 0) != 0


@pytest.mark.parametrize("learned_smoother", [False, True])
def test_vcycle_and_fcg_stencil_match_csr(cuda, learned_smoother):
    """The stencil V-cycle equals the CSR one up to fp32 summation order, and the flexible-CG solve
    converges in the same number of iterations (within one)."""
    import os

    from warp_gb300 import learned, multigrid
    from warp_gb300.optim import linear

    s = _system((16, 16, 16), seed=7)
    mgs = {}
    for st in (False, True):
        mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef, stencil=st, coarsest_nodes=400)  # 3 levels
        if learned_smoother:
            w = os.path.join(os.path.dirname(__file__), "..", "warp_gb300", "data", "smoother_q1_diffusion.npz")
            mg.smoother = learned.LearnedSmoother(learned.ConvNet.load(w), mg, s.coef)
        mgs[st] = mg
    assert all(lv.S is not None for lv in mgs[True].levels[:-1])
    assert mgs[True].kernels_per_apply < mgs[False].kernels_per_apply
    r = torch.randn(s.A.nrow, device="cuda", generator=torch.Generator("cuda").manual_seed(2))
    r = r * (1 - mgs[True].levels[0].mask)
    z_csr = mgs[False].apply(r)
    z_st = mgs[True].apply(r)
    torch.cuda.synchronize()
    assert int(mgs[True].status.item()) == 0
    err = float((z_st - z_csr).abs().max()) / float(z_csr.abs().max())
    assert err < 1e-4, err
    its = {}
    for st, mg in mgs.items():
        x = torch.zeros_like(s.b)
        it, res, atol = linear.fcg(s.A, s.b, x, tol=1e-6, atol=0.0, maxiter=200, M=mg, check_every=1)
        assert res <= atol
        its[st] = it
    assert abs(its[True] - its[False]) <= 1, its


def _bf16_round(a):
    """Round-to-nearest-even to bf16, returned as float64 (the coefficients the bf16 kernels read)."""
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float64).numpy()


@pytest.mark.parametrize("cells", [(6, 5, 4), (9, 7, 12), (1, 3, 2)])
def test_st27_bf16_modes_match_rounded_product(cuda, cells):
    """The bf16 coefficient copy: every mode against a float64 product with the bf16-rounded CSR values
    (accumulation in fp32, so within fp32 summation error)."""
    from warp_gb300 import _native as N

    s = _system(cells, seed=5)
    dims = tuple(c + 1 for c in cells)
    n, off, col, val = _csr(s.A)
    L = N.lib()
    S = torch.empty(int(L.gb_st27_bytes(*dims)) // 4, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(L.gb_st27_build(*dims, s.A.offsets.data_ptr(), s.A.columns.data_ptr(), s.A.values.data_ptr(),
                            S.data_ptr(), status.data_ptr(), 0))
    Sb = torch.empty(int(L.gb_st27_bytes_bf16(*dims)) // 2, dtype=torch.bfloat16, device="cuda")
    assert Sb.numel() % 8 == 0
    N.check(L.gb_st27_to_bf16(*dims, S.data_ptr(), Sb.data_ptr(), 0))
    torch.cuda.synchronize()
    # layout: 28 values per node, the 27 taps of S rounded to bf16 and one zero
    Sh = S.cpu().numpy()[: n * 27].reshape(n, 27)
    Sbh = Sb.float().cpu().numpy()[: n * 28].reshape(n, 28)
    np.testing.assert_array_equal(Sbh[:, :27], _bf16_round(Sh).astype(np.float32))
    assert not Sbh[:, 27].any()
    valb = _bf16_round(val)
    rng = np.random.default_rng(4)
    r = rng.standard_normal(n).astype(np.float32)
    w = rng.standard_normal(n).astype(np.float32)
    d = np.zeros(n)
    rows = np.repeat(np.arange(n), np.diff(off))
    d[rows[col == rows]] = val[col == rows]
    dinv = (1.0 / d).astype(np.float32)
    omega = 0.6
    rt, wt, dt = (torch.from_numpy(a).cuda() for a in (r, w, dinv))
    out = torch.empty_like(rt)
    w_out = torch.empty_like(rt)
    scale = np.abs(val).max() * np.abs(w).max() * 27
    st = status.data_ptr()
    N.check(L.gb_st27_apply_bf16(0, *dims, Sb.data_ptr(), wt.data_ptr(), rt.data_ptr(), None, omega, None,
                                 out.data_ptr(), st, 0))
    ref = r - _matvec(off, col, valb, w.astype(np.float64))
    np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-5 * scale, rtol=1e-5)
    N.check(L.gb_st27_apply_bf16(1, *dims, Sb.data_ptr(), None, rt.data_ptr(), dt.data_ptr(), omega,
                                 w_out.data_ptr(), out.data_ptr(), st, 0))
    w1 = omega * dinv.astype(np.float64) * r
    np.testing.assert_allclose(w_out.cpu().numpy(), w1, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(out.cpu().numpy(), r - _matvec(off, col, valb, w1), atol=1e-5 * scale, rtol=1e-5)
    N.check(L.gb_st27_apply_bf16(2, *dims, Sb.data_ptr(), wt.data_ptr(), rt.data_ptr(), dt.data_ptr(), omega, None,
                                 out.data_ptr(), st, 0))
    ref = w + omega * dinv * (r - _matvec(off, col, valb, w.astype(np.float64)))
    np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-5 * scale * np.abs(dinv).max(), rtol=1e-5)
    assert int(status.item()) == 0


@pytest.mark.parametrize("learned_smoother", [False, True])
def test_bf16_fine_stencil_fcg_converges(cuda, learned_smoother):
    """Flexible CG with the bf16 fine-level stencil in the V-cycle reaches the same tolerance in at most
    one more iteration than with fp32 coefficients (the cycle is only an approximate inverse)."""
    import os

    from warp_gb300 import learned, multigrid
    from warp_gb300.optim import linear

    s = _system((24, 24, 24), seed=11)
    its = {}
    for fv in (torch.float32, torch.bfloat16):
        mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef, fine_values=fv)
        assert (mg.levels[0].Sb is not None) == (fv == torch.bfloat16)
        if learned_smoother:
            w = os.path.join(os.path.dirname(__file__), "..", "warp_gb300", "data", "smoother_q1_diffusion.npz")
            mg.smoother = learned.LearnedSmoother(learned.ConvNet.load(w), mg, s.coef)
        x = torch.zeros_like(s.b)
        it, res, atol = linear.fcg(s.A, s.b, x, tol=1e-7, atol=0.0, maxiter=300, M=mg, check_every=1)
        assert res <= atol
        assert int(mg.status.item()) == 0
        its[fv] = it
    assert its[torch.bfloat16] <= its[torch.float32] + 1, its


@pytest.mark.parametrize("learned_smoother", [False, True])
def test_fcg_stencil_product_matches_csr_product(cuda, learned_smoother):
    """The flexible solver's two-kernel step on the fine level's stencil form (k_fcg_st27_az: A z with
    z.r, z.Ap_old and z.Az; k_fcg_update: p, Ap, x, r) against the four-kernel step on the CSR product:
    same iteration count within one, and the refined solve reaches 1e-8 with the FP64 residual recomputed
    on the host."""
    import os

    from warp_gb300 import learned, multigrid
    from warp_gb300.optim import linear

    s = _system((20, 18, 22), seed=13)
    n, off, col, val = _csr(s.A)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef)
    if learned_smoother:
        w = os.path.join(os.path.dirname(__file__), "..", "warp_gb300", "data", "smoother_q1_diffusion.npz")
        mg.smoother = learned.LearnedSmoother(learned.ConvNet.load(w), mg, s.coef)
    its = {}
    for st in (False, True):
        x = torch.zeros_like(s.b)
        solver = linear.FCG(s.A, s.b, x, tol=1e-6, atol=0.0, maxiter=300, M=mg, check_every=1,
                            stencil="auto" if st else None)
        assert solver.stencil_product == st
        it, res, atol = solver()
        assert res <= atol
        its[st] = it
        r = s.b.cpu().numpy().astype(np.float64) - _matvec(off, col, val, x.cpu().numpy().astype(np.float64))
        assert np.linalg.norm(r) <= 32e-6 * np.linalg.norm(s.b.cpu().numpy()), st
    assert abs(its[True] - its[False]) <= 1, its
    for sp in (False, True):
        rs = linear.RefinedSolver(s.A, M=mg, method="fcg", inner_tol=1e-5, stencil_product=sp)
        assert rs.inner.stencil_product == sp
        x64, info = rs.solve(s.b, tol=1e-8)
        assert info["converged"] and rs.fallbacks == 0
        bh = s.b.cpu().numpy().astype(np.float64)
        r = bh - _matvec(off, col, val, x64.cpu().numpy())
        assert np.linalg.norm(r) <= 2e-8 * np.linalg.norm(bh)


def test_fcg_stencil_rejects_mismatched_grid(cuda):
    from warp_gb300 import _native as N
    from warp_gb300 import multigrid
    from warp_gb300.optim import linear

    s = _system((8, 8, 8), seed=2)
    mg = multigrid.MultigridPreconditioner(s.A, s.geo, s.coef, coarsest_nodes=400)
    S = mg.levels[0].S
    assert S is not None and len(mg.levels) > 1
    x = torch.zeros_like(s.b)
    solver = linear.FCG(s.A, s.b, x, tol=1e-6, maxiter=50, M=mg)
    assert N.lib().gb_krylov_set_stencil(solver._native, 9, 9, 10, S.data_ptr()) != 0  # 810 nodes, not 729
    assert N.lib().gb_krylov_set_stencil(solver._native, 9, 9, 9, S.data_ptr()) == 0
    assert N.lib().gb_krylov_set_stencil(solver._native, 0, 0, 0, None) == 0


def test_residual_df_on_stencil_matches_fp64(cuda):
    """gb_residual_df_st27 against the FP64 oracle product on the same fp32 values (the double-float
    tolerance of gb_residual_df) and against gb_residual_df on the CSR form."""
    from warp_gb300 import _native as N

    s = _system((14, 12, 16), seed=21)
    dims = (15, 13, 17)
    n, off, col, val = _csr(s.A)
    L = N.lib()
    S = torch.empty(int(L.gb_st27_bytes(*dims)) // 4, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(L.gb_st27_build(*dims, s.A.offsets.data_ptr(), s.A.columns.data_ptr(), s.A.values.data_ptr(),
                            S.data_ptr(), status.data_ptr(), 0))
    rng = np.random.default_rng(8)
    x64 = rng.standard_normal(n)
    b = rng.standard_normal(n).astype(np.float32)
    hi = x64.astype(np.float32)
    lo = (x64 - hi.astype(np.float64)).astype(np.float32)
    x2 = torch.from_numpy(np.stack([hi, lo], 1).reshape(-1).copy()).cuda()
    bd = torch.from_numpy(b).cuda()
    ws = torch.zeros(int(L.gb_residual_f64_workspace_bytes(1, n, len(val), N.GB_F32)), dtype=torch.uint8, device="cuda")
    out = {}
    for kind in ("st27", "csr"):
        r64 = torch.zeros(n, dtype=torch.float64, device="cuda")
        r32 = torch.zeros(n, dtype=torch.float32, device="cuda")
        norms = torch.zeros(2, dtype=torch.float64, device="cuda")
        if kind == "st27":
            N.check(L.gb_residual_df_st27(*dims, S.data_ptr(), x2.data_ptr(), bd.data_ptr(), r64.data_ptr(),
                                          r32.data_ptr(), norms.data_ptr(), ws.data_ptr(), ws.numel(),
                                          status.data_ptr(), 0))
        else:
            N.check(L.gb_residual_df(1, n, len(val), s.A.capacity, s.A.offsets.data_ptr(), None,
                                     s.A.columns.data_ptr(), s.A.values.data_ptr(), N.GB_F32, x2.data_ptr(),
                                     bd.data_ptr(), r64.data_ptr(), r32.data_ptr(), norms.data_ptr(), ws.data_ptr(),
                                     ws.numel(), status.data_ptr(), 0))
        torch.cuda.synchronize()
        out[kind] = (r64.cpu().numpy(), r32.cpu().numpy(), norms.cpu().numpy())
    assert int(status.item()) == 0
    exact = b.astype(np.float64) - _matvec(off, col, val, x64)
    scale = _matvec(off, col, np.abs(val), np.abs(x64)) + np.abs(b)
    for kind, (r64, r32, norms) in out.items():
        assert np.all(np.abs(r64 - exact) <= 1e-11 * scale), kind
        np.testing.assert_allclose(r32, exact.astype(np.float32), rtol=2e-7, atol=1e-12 * scale.max())
        np.testing.assert_allclose(norms[0], np.dot(r32.astype(np.float64), r32), rtol=1e-5)
        np.testing.assert_allclose(norms[1], np.dot(b.astype(np.float64), b), rtol=1e-5)
    np.testing.assert_allclose(out["st27"][2], out["csr"][2], rtol=1e-6)
