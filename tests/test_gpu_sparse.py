"""GPU parity: triplet assembly (bit-exact structure) and SpMV against the CPU oracle."""

import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "triplets_ref.npz")


def _t(a, dtype=None):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda" if dtype is None else "cuda").to(
        dtype if dtype is not None else torch.from_numpy(np.ascontiguousarray(a)).dtype)


def _native_from_triplets(nrow, ncol, rows, cols, vals, bs, prune=True):
    """Raw C-ABI call; returns numpy (offsets, columns, run_ends, sorted ids, nnz, values)."""
    import warp_gb300._arrays as A
    import warp_gb300._native as N

    n = len(rows)
    rows_d = torch.from_numpy(np.ascontiguousarray(rows, np.int32)).cuda()
    cols_d = torch.from_numpy(np.ascontiguousarray(cols, np.int32)).cuda()
    vals_d = None if vals is None else torch.from_numpy(np.ascontiguousarray(vals, np.float32).reshape(n, bs)).cuda()
    tbo = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    tbi = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    offsets = torch.full((nrow + 1,), -7, dtype=torch.int32, device="cuda")
    columns = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    L = N.lib()
    ws = A.workspace(L.gb_bsr_from_triplets_workspace_bytes(n, nrow, ncol))
    nnz_host = torch.zeros(1, dtype=torch.int32, pin_memory=True)
    mask = 0x7FFFFFFF if (prune and vals is not None) else 0
    N.check(L.gb_bsr_matrix_from_triplets_device(
        bs, 4 if vals is not None else 0, nrow, ncol, n, None, rows_d.data_ptr(), cols_d.data_ptr(),
        None if vals_d is None else vals_d.data_ptr(), mask, 0, tbo.data_ptr(), tbi.data_ptr(), offsets.data_ptr(),
        None, columns.data_ptr(), nnz_host.data_ptr(), None, ws.data_ptr(), ws.numel(), A.stream()))
    torch.cuda.synchronize()
    nnz = int(nnz_host[0])
    out = dict(offsets=offsets.cpu().numpy(), columns=columns.cpu().numpy()[:nnz], runends=tbo.cpu().numpy()[:nnz],
               ids=tbi.cpu().numpy()[:n], nnz=nnz)
    if vals is not None:
        bv = torch.zeros((max(nnz, 1), bs), dtype=torch.float32, device="cuda")
        N.check(L.gb_bsr_accumulate_triplet_values(N.GB_F32, bs, nrow, offsets.data_ptr(), tbo.data_ptr(),
                                                   tbi.data_ptr(), vals_d.data_ptr(), bv.data_ptr(), n, A.stream()))
        out["values"] = bv.cpu().numpy()[:nnz]
    return out


@pytest.mark.parametrize("prune", [0, 1])
def test_from_triplets_matches_reference_golden(cuda, prune):
    g = np.load(GOLDEN)
    names = sorted({k.split("_")[0] for k in g.files if k.startswith("case")})
    for name in names:
        key = f"{name}_p{prune}"
        nrow, ncol, bs, _, nnz = (int(v) for v in g[key + "_meta"])
        rows, cols, vals = g[name + "_rows"], g[name + "_cols"], g[name + "_vals"]
        got = _native_from_triplets(nrow, ncol, rows, cols, vals, bs, prune=bool(prune))
        assert got["nnz"] == nnz, name
        np.testing.assert_array_equal(got["offsets"], g[key + "_offsets"])
        np.testing.assert_array_equal(got["columns"], g[key + "_columns"])
        np.testing.assert_array_equal(got["runends"], g[key + "_runends"])
        np.testing.assert_array_equal(got["ids"][: len(g[key + "_runidx"])], g[key + "_runidx"])


@pytest.mark.parametrize("case", [
    (1, 1, 0, 1), (3, 3, 7, 1), (100, 80, 5000, 1), (4000, 4000, 200000, 1), (3000, 2000, 100000, 9),
    (70000, 70000, 300000, 1),   # 17+17 bits -> 64-bit key path
    (1 << 20, 3, 50000, 1),      # tall
])
def test_from_triplets_vs_oracle(cuda, case):
    nrow, ncol, n, bs = case
    rng = np.random.default_rng(nrow * 7 + n)
    rows = rng.integers(-1, nrow + 1, n)
    cols = rng.integers(-1, ncol + 1, n)
    vals = rng.standard_normal((n, bs)).astype(np.float32)
    vals[rng.random(n) < 0.05] = 0.0
    exp = oracle.bsr_from_triplets(nrow, ncol, rows, cols, vals, block_shape=(bs, 1))
    got = _native_from_triplets(nrow, ncol, rows, cols, vals, bs)
    assert got["nnz"] == exp["nnz"]
    np.testing.assert_array_equal(got["offsets"], exp["offsets"])
    np.testing.assert_array_equal(got["columns"], exp["columns"])
    np.testing.assert_array_equal(got["runends"], exp["tpl_block_offsets"])
    np.testing.assert_array_equal(got["ids"], exp["tpl_block_indices"])
    if exp["nnz"]:
        # same summation order as the oracle -> bit-exact fp32 sums
        np.testing.assert_array_equal(got["values"].reshape(-1), exp["values"].reshape(-1))


def test_from_triplets_topology_only_and_empty(cuda):
    got = _native_from_triplets(2, 3, [1, 0, 1], [2, 1, 2], None, 1)
    assert got["nnz"] == 2
    np.testing.assert_array_equal(got["offsets"], [0, 1, 2])
    np.testing.assert_array_equal(got["columns"], [1, 2])
    got = _native_from_triplets(5, 5, [], [], None, 1)
    assert got["nnz"] == 0
    np.testing.assert_array_equal(got["offsets"], np.zeros(6))
    # all triplets pruned
    got = _native_from_triplets(12, 12, [1, 0, 2, 3], [0, 1, 2, 3], np.zeros(4, np.float32), 1, prune=True)
    assert got["nnz"] == 0
    got = _native_from_triplets(12, 12, [1, 0, 2, 3], [0, 1, 2, 3], np.zeros(4, np.float32), 1, prune=False)
    assert got["nnz"] == 4


def test_bsr_api_from_triplets_count_and_dense(cuda):
    from warp_gb300 import sparse

    rng = np.random.default_rng(123)
    nrow, ncol, n = 4, 9, 50
    rows = rng.integers(0, nrow, n).astype(np.int32)
    cols = rng.integers(0, ncol, n).astype(np.int32)
    vals = rng.random((n, 3, 3)).astype(np.float32)
    A = sparse.bsr_zeros(nrow, ncol, ((3, 3), torch.float32))
    sparse.bsr_set_from_triplets(A, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(),
                                 torch.from_numpy(vals).cuda())
    ref = oracle.triplets_to_dense(nrow, ncol, rows, cols, vals, (3, 3))
    np.testing.assert_allclose(A.numpy_dense(), ref, atol=1e-4)
    # device-side triplet count: only the first 20 triplets are used
    count = torch.tensor([20], dtype=torch.int32, device="cuda")
    B = sparse.bsr_zeros(nrow, ncol, ((3, 3), torch.float32))
    sparse.bsr_set_from_triplets(B, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(),
                                 torch.from_numpy(vals).cuda(), count=count)
    ref20 = oracle.triplets_to_dense(nrow, ncol, rows[:20], cols[:20], vals[:20], (3, 3))
    np.testing.assert_allclose(B.numpy_dense(), ref20, atol=1e-4)
    with pytest.raises(TypeError):
        sparse.bsr_set_from_triplets(A, torch.from_numpy(rows).float().cuda(), torch.from_numpy(cols).cuda())


def _random_bsr(nrow, ncol, n, bs, seed):
    from warp_gb300 import sparse

    rng = np.random.default_rng(seed)
    rows = rng.integers(0, nrow, n).astype(np.int32)
    cols = rng.integers(0, ncol, n).astype(np.int32)
    vals = rng.standard_normal((n, *bs)).astype(np.float32)
    blk = torch.float32 if bs == (1, 1) else (bs, torch.float32)
    A = sparse.bsr_zeros(nrow, ncol, blk)
    v = vals.reshape(n) if bs == (1, 1) else vals
    sparse.bsr_set_from_triplets(A, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(),
                                 torch.from_numpy(v).cuda())
    A.nnz_sync()
    o = oracle.bsr_from_triplets(nrow, ncol, rows, cols, vals.reshape(n, -1), block_shape=bs)
    return A, o


@pytest.mark.parametrize("bs", [(1, 1), (3, 3), (2, 2), (1, 3), (3, 1)])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (-0.5, 1.0), (2.0, 0.25), (0.0, 3.0)])
def test_bsr_mv_vs_oracle(cuda, bs, alpha, beta):
    from warp_gb300 import sparse

    nrow, ncol = 3001, 2999
    A, o = _random_bsr(nrow, ncol, 60000, bs, seed=bs[0] * 10 + bs[1])
    rng = np.random.default_rng(5)
    x = rng.standard_normal(ncol * bs[1]).astype(np.float32)
    y0 = rng.standard_normal(nrow * bs[0]).astype(np.float32)
    y = torch.from_numpy(y0.copy()).cuda()
    sparse.bsr_mv(A, torch.from_numpy(x).cuda(), y, alpha=alpha, beta=beta)
    exp = alpha * oracle.bsr_mv_f64(o["offsets"], o["columns"], o["values"], x, block_shape=bs) + beta * y0
    scale = abs(alpha) * oracle.bsr_abs_mv_f64(o["offsets"], o["columns"], o["values"], x, block_shape=bs) + \
        abs(beta * y0)
    # fp32 products and sums of <= ~40 terms: |err| <= 1e-5 * sum |a_ij x_j| (+ tiny absolute)
    err = np.abs(y.cpu().numpy() - exp)
    assert np.all(err <= 1e-5 * scale + 1e-30), float((err / (scale + 1e-30)).max())


def test_bsr_mv_regular_fem_structure_and_tiles(cuda):
    """27-point Q1 structure exercised with every lanes-per-row choice and staging on/off."""
    import warp_gb300._native as N
    from warp_gb300 import fem, sparse

    geo = fem.Grid3D(res=(20, 17, 13))
    space = fem.make_polynomial_space(geo, degree=1)
    nu = np.random.default_rng(1).lognormal(size=geo.cell_count()).astype(np.float32)
    A = fem.integrate(fem.diffusion_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)},
                      values={"nu": nu})
    nnz = A.nnz_sync()
    off = A.offsets.cpu().numpy()
    cols = A.columns[:nnz].cpu().numpy()
    vals = A.values[:nnz].cpu().numpy()
    n = A.nrow
    x = np.random.default_rng(2).standard_normal(n).astype(np.float32)
    exp = oracle.bsr_mv_f64(off, cols, vals, x)
    scale = oracle.bsr_abs_mv_f64(off, cols, vals, x)
    xd = torch.from_numpy(x).cuda()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    for G in (1, 2, 4, 8, 16, 32):
        for rows, cap in ((64, 0), (128, 4096), (256, 8192), (32, 16)):
            y = torch.empty(n, dtype=torch.float32, device="cuda")
            N.check(N.lib().gb_bsr_mv(1, 1, n, n, nnz, A.capacity, A.offsets.data_ptr(), None, A.columns.data_ptr(),
                                      A.values.data_ptr(), N.GB_F32, xd.data_ptr(), y.data_ptr(), y.data_ptr(),
                                      N.GB_F32, 1.0, 0.0, 0, rows, G, cap, status.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream))
            err = np.abs(y.cpu().numpy() - exp)
            assert np.all(err <= 1e-5 * scale + 1e-30), (G, rows, cap)
    assert int(status.item()) == 0


def test_bsr_mv_bf16_values_and_f64_vectors(cuda):
    from warp_gb300 import sparse

    for bs in [(1, 1), (3, 3)]:
        A, o = _random_bsr(2000, 2000, 40000, bs, seed=11)
        x = np.random.default_rng(0).standard_normal(2000 * bs[1])
        # fp64 vectors with fp32 values: fp64 accumulation -> ~1e-15 relative
        y = torch.zeros(2000 * bs[0], dtype=torch.float64, device="cuda")
        sparse.bsr_mv(A, torch.from_numpy(x).cuda(), y)
        exp = oracle.bsr_mv_f64(o["offsets"], o["columns"], o["values"], x, block_shape=bs)
        scale = oracle.bsr_abs_mv_f64(o["offsets"], o["columns"], o["values"], x, block_shape=bs)
        assert np.all(np.abs(y.cpu().numpy() - exp) <= 1e-13 * scale + 1e-300)
        # bf16 values: error bounded by bf16 rounding of the values (2^-8 relative)
        Ab = sparse.bsr_copy(A)
        Ab.values = A.values[: A.nnz].to(torch.bfloat16)
        yb = sparse.bsr_mv(Ab, torch.from_numpy(x.astype(np.float32)).cuda())
        assert np.all(np.abs(yb.cpu().numpy().reshape(-1) - exp) <= 4e-3 * scale + 1e-6)


def test_bsr_mv_aliasing_and_transpose(cuda):
    from warp_gb300 import sparse

    A, o = _random_bsr(500, 500, 5000, (1, 1), seed=21)
    x = np.random.default_rng(1).standard_normal(500).astype(np.float32)
    xd = torch.from_numpy(x.copy()).cuda()
    sparse.bsr_mv(A, xd, xd, alpha=1.0, beta=0.5)  # x and y alias
    exp = oracle.bsr_mv_f64(o["offsets"], o["columns"], o["values"], x) + 0.5 * x
    np.testing.assert_allclose(xd.cpu().numpy(), exp, rtol=1e-4, atol=1e-4)
    D = oracle.bsr_to_dense(o["offsets"], o["columns"], o["values"], 500)
    yt = sparse.bsr_mv(A, torch.from_numpy(x).cuda(), transpose=True)
    np.testing.assert_allclose(yt.cpu().numpy(), D.T @ x, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("shapes", [((1, 1), (1, 1)), ((3, 3), (3, 3)), ((2, 3), (3, 1))])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (0.5, 2.0)])
def test_bsr_mm_vs_dense(cuda, shapes, alpha, beta):
    from warp_gb300 import sparse

    (a, k), (k2, c) = shapes
    X, ox = _random_bsr(60, 50, 400, (a, k), seed=1)
    Y, oy = _random_bsr(50, 70, 500, (k2, c), seed=2)
    Z, oz = _random_bsr(60, 70, 300, (a, c), seed=3)
    Dx = oracle.bsr_to_dense(ox["offsets"], ox["columns"], ox["values"], 50, (a, k))
    Dy = oracle.bsr_to_dense(oy["offsets"], oy["columns"], oy["values"], 70, (k2, c))
    Dz = oracle.bsr_to_dense(oz["offsets"], oz["columns"], oz["values"], 70, (a, c))
    out = sparse.bsr_mm(X, Y, Z, alpha=alpha, beta=beta)
    exp = alpha * Dx @ Dy + beta * Dz
    np.testing.assert_allclose(out.numpy_dense(), exp, rtol=1e-4, atol=1e-4 * np.abs(exp).max())
    # topology = union of product pattern and z pattern when beta != 0
    nnz = out.nnz_sync()
    pat = (np.abs(Dx) > 0).astype(int) @ (np.abs(Dy) > 0).astype(int)
    if beta != 0:
        pat = pat + (np.abs(Dz) > 0)
    blocks = (pat.reshape(60, a, 70, c).sum(axis=(1, 3)) > 0).sum()
    assert nnz == blocks


def test_bsr_mm_diagonal_projector_keeps_structure(cuda):
    from warp_gb300 import fem, sparse

    geo = fem.Grid3D(res=(5, 4, 3))
    space = fem.make_polynomial_space(geo, degree=1)
    A = fem.integrate(fem.diffusion_form, fields={"u": fem.make_trial(space), "v": fem.make_test(space)})
    bd = fem.BoundarySides(geo)
    P = fem.integrate(fem.boundary_projector_form, fields={"u": fem.make_trial(space, bd),
                                                           "v": fem.make_test(space, bd)}, assembly="nodal")
    D = A.numpy_dense()
    PA = sparse.bsr_mm(P, A)
    np.testing.assert_allclose(PA.numpy_dense(), P.numpy_dense() @ D, atol=1e-5)


@pytest.mark.parametrize("shapes", [((1, 1), (1, 1)), ((3, 3), (3, 3)), ((2, 3), (3, 1))])
@pytest.mark.parametrize("beta", [0.0, 0.5])
def test_bsr_mm_masked_keeps_z_topology(cuda, shapes, beta):
    """topology="masked" (reference sparse.py:4200-4260): z keeps its blocks; on them
    z = alpha x y + beta z, and product terms outside z's pattern are dropped."""
    from warp_gb300 import sparse

    (a, k), (k2, c) = shapes
    X, ox = _random_bsr(60, 50, 400, (a, k), seed=11)
    Y, oy = _random_bsr(50, 70, 500, (k2, c), seed=12)
    Z, oz = _random_bsr(60, 70, 900, (a, c), seed=13)
    Dx = oracle.bsr_to_dense(ox["offsets"], ox["columns"], ox["values"], 50, (a, k))
    Dy = oracle.bsr_to_dense(oy["offsets"], oy["columns"], oy["values"], 70, (k2, c))
    Dz = oracle.bsr_to_dense(oz["offsets"], oz["columns"], oz["values"], 70, (a, c))
    off0, cols0 = Z.offsets.clone(), Z.columns[: Z.nnz_sync()].clone()
    out = sparse.bsr_mm(X, Y, Z, alpha=1.5, beta=beta, topology="masked")
    assert out is Z
    np.testing.assert_array_equal(Z.offsets.cpu().numpy(), off0.cpu().numpy())
    np.testing.assert_array_equal(Z.columns[: Z.nnz_sync()].cpu().numpy(), cols0.cpu().numpy())
    mask = np.kron((oracle.bsr_to_dense(oz["offsets"], oz["columns"], np.ones_like(oz["values"]), 70, (a, c))
                    .reshape(60, a, 70, c)[:, 0, :, 0] != 0).astype(float), np.ones((a, c)))
    exp = (1.5 * Dx @ Dy + beta * Dz) * mask
    np.testing.assert_allclose(Z.numpy_dense(), exp, rtol=1e-4, atol=1e-4 * np.abs(exp).max())
    # the deprecated masked=True spelling is the same operation
    Z2, _ = _random_bsr(60, 70, 900, (a, c), seed=13)
    sparse.bsr_mm(X, Y, Z2, alpha=1.5, beta=beta, masked=True)
    nz = Z.nnz_sync()
    np.testing.assert_array_equal(Z2.values[:nz].cpu().numpy(), Z.values[:nz].cpu().numpy())
