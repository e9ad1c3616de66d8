"""CPU tests of the oracle: pinned against the reference's known-answer tests and against the
reference's own compiled host routine (frozen in tests/golden/triplets_ref.npz)."""

import os

import numpy as np
import pytest

import oracle
from oracle import fem_q1

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "triplets_ref.npz")


def test_structure_kat():
    # warp/tests/test_sparse.py:151-161 -- rows [1,0,1], cols [2,1,2] on a 2x3 matrix
    o = oracle.bsr_from_triplets(2, 3, [1, 0, 1], [2, 1, 2])
    assert o["nnz"] == 2
    np.testing.assert_array_equal(o["offsets"], [0, 1, 2])
    np.testing.assert_array_equal(o["columns"], [1, 2])


def test_probe_kat():
    # rows [1,0,1,1], cols [2,1,2,0] -> offsets [0,1,3], columns [1,0,2]
    o = oracle.bsr_from_triplets(2, 3, [1, 0, 1, 1], [2, 1, 2, 0])
    np.testing.assert_array_equal(o["offsets"], [0, 1, 3])
    np.testing.assert_array_equal(o["columns"], [1, 0, 2])


def test_prune_kat():
    # warp/tests/test_sparse.py:199-222
    rows, cols = [1, 0, 2, 3], [0, 1, 2, 3]
    vals = np.zeros(4, np.float32)
    assert oracle.bsr_from_triplets(12, 12, rows, cols, vals, prune_numerical_zeros=False)["nnz"] == 4
    assert oracle.bsr_from_triplets(12, 12, rows, cols, vals, prune_numerical_zeros=True)["nnz"] == 0


def test_dense_reconstruction():
    # warp/tests/test_sparse.py:109-196 (dense reconstruction, atol 1e-4)
    rng = np.random.default_rng(123)
    for (nrow, ncol, bs, n) in [(8, 6, (1, 1), 100), (4, 9, (3, 2), 50)]:
        rows = rng.integers(0, nrow, n)
        cols = rng.integers(0, ncol, n)
        vals = rng.random((n, bs[0] * bs[1])).astype(np.float32)
        o = oracle.bsr_from_triplets(nrow, ncol, rows, cols, vals, block_shape=bs)
        ref = oracle.triplets_to_dense(nrow, ncol, rows, cols, vals, bs)
        got = oracle.bsr_to_dense(o["offsets"], o["columns"], o["values"], ncol, bs)
        np.testing.assert_allclose(got, ref, atol=1e-4)


def _golden_cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("_")[0] for k in g.files if k.startswith("case")})
    return g, names


@pytest.mark.parametrize("prune", [0, 1])
def test_oracle_matches_reference_golden(prune):
    g, names = _golden_cases()
    for name in names:
        key = f"{name}_p{prune}"
        nrow, ncol, bs, _, nnz = (int(v) for v in g[key + "_meta"])
        rows, cols, vals = g[name + "_rows"], g[name + "_cols"], g[name + "_vals"]
        o = oracle.bsr_from_triplets(nrow, ncol, rows, cols, vals, block_shape=(bs, 1),
                                     prune_numerical_zeros=bool(prune))
        assert o["nnz"] == nnz, name
        np.testing.assert_array_equal(o["offsets"], g[key + "_offsets"])
        np.testing.assert_array_equal(o["columns"], g[key + "_columns"])
        np.testing.assert_array_equal(o["tpl_block_offsets"], g[key + "_runends"])
        # stable order inside each run: the oracle's ids are already ascending
        idx = o["tpl_block_indices"][: len(g[key + "_runidx"])]
        np.testing.assert_array_equal(idx, g[key + "_runidx"])


def test_oracle_matches_compiled_reference_live():
    if oracle.ref_lib() is None:
        pytest.skip("reference routine not compiled here (no Warp sources)")
    rng = np.random.default_rng(7)
    for _ in range(20):
        nrow, ncol = (int(v) for v in rng.integers(1, 200, 2))
        n = int(rng.integers(0, 3000))
        rows = rng.integers(-1, nrow + 1, n)
        cols = rng.integers(-1, ncol + 1, n)
        vals = rng.random(n).astype(np.float32)
        vals[rng.random(n) < 0.1] = 0
        o = oracle.bsr_from_triplets(nrow, ncol, rows, cols, vals)
        r = oracle.ref_bsr_from_triplets(nrow, ncol, rows, cols, vals)
        assert o["nnz"] == r["nnz"]
        np.testing.assert_array_equal(o["offsets"], r["offsets"])
        np.testing.assert_array_equal(o["columns"], r["columns"])
        np.testing.assert_array_equal(o["tpl_block_offsets"], r["tpl_block_offsets"])


def _spd(n, seed):
    # warp/tests/test_linear_solvers.py:64-81
    rng = np.random.default_rng(seed)
    C = rng.uniform(-100, 100, (n, n))
    f = rng.uniform(-100, 100, n)
    return C @ C.T, C @ f


def _dense_to_csr(Ad):
    n = Ad.shape[0]
    offsets = np.arange(0, n * n + 1, n, dtype=np.int32)
    cols = np.tile(np.arange(n, dtype=np.int32), n)
    return offsets, cols, Ad.astype(np.float32).reshape(-1)


def test_oracle_pcg_bicgstab_small_spd():
    Ad, b = _spd(16, 321)
    off, cols, vals = _dense_to_csr(Ad)
    dinv = oracle.inverse_diagonal_f32(off, cols, vals)
    np.testing.assert_allclose(dinv, 1.0 / np.diag(Ad).astype(np.float32), rtol=1e-6)
    for solver in (oracle.pcg_f32, oracle.bicgstab_f32):
        x, it, err, atol = solver(off, cols, vals, b.astype(np.float32), inv_diag=dinv, maxiter=1000)
        assert err <= atol
        # reference bound on the true residual for fp32 (test_linear_solvers.py:56-61)
        assert np.linalg.norm(Ad @ x - b) <= 32 * atol


def test_oracle_spmv_bounds():
    rng = np.random.default_rng(3)
    nrow = 200
    rows = rng.integers(0, nrow, 3000)
    cols = rng.integers(0, nrow, 3000)
    vals = rng.standard_normal(3000).astype(np.float32)
    o = oracle.bsr_from_triplets(nrow, nrow, rows, cols, vals)
    x = rng.standard_normal(nrow).astype(np.float32)
    y32 = oracle.bsr_mv_f32(o["offsets"], o["columns"], o["values"], x)
    y64 = oracle.bsr_mv_f64(o["offsets"], o["columns"], o["values"], x)
    scale = oracle.bsr_abs_mv_f64(o["offsets"], o["columns"], o["values"], x)
    assert np.all(np.abs(y32 - y64) <= 1e-6 * scale + 1e-30)


def test_fem_oracle_properties():
    # scalar stiffness: constants in the kernel; elasticity: rigid translations in the kernel
    for dim, res in [(2, (5, 4)), (3, (3, 2, 4))]:
        r, c, v = fem_q1.assemble_triplets(res)
        nn = int(np.prod([k + 1 for k in res]))
        D = oracle.triplets_to_dense(nn, nn, r, c, v)
        np.testing.assert_allclose(D @ np.ones(nn), 0.0, atol=1e-5)
        np.testing.assert_allclose(D, D.T, atol=1e-6)
    res = (2, 3, 2)
    r, c, v = fem_q1.assemble_triplets(res, ncomp=3, lame=(1.5, 0.7))
    nn = 3 * 4 * 3
    D = oracle.triplets_to_dense(nn, nn, r, c, v, (3, 3))
    for d in range(3):
        t = np.zeros((nn, 3))
        t[:, d] = 1
        np.testing.assert_allclose(D @ t.reshape(-1), 0.0, atol=1e-5)
    # consistent mass rhs of f = 1 integrates to the domain volume
    b = fem_q1.assemble_rhs((4, 5, 6), f_const=[1.0])
    assert abs(b.sum() - 1.0) < 1e-12


def test_fem_oracle_triplet_order():
    # node-major, then ascending element, then trial node (virtual.py:1084-1115)
    r, c, _ = fem_q1.assemble_triplets((2, 2))
    assert np.all(np.diff(r) >= 0)
    assert len(r) == 4 * 16
    # node 4 (centre of a 2x2 grid) touches all four cells: its first trial block is cell 0
    first = np.where(r == 4)[0][0]
    np.testing.assert_array_equal(c[first:first + 4], [0, 1, 3, 4])


COMPRESS_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "compress_ref.npz")


@pytest.mark.parametrize("prune", [0, 1])
def test_compress_restatement_matches_reference_golden(prune):
    """The row-compress restatement equals the reference's compiled in-place compression bit for bit
    (frozen by tests/golden/make_golden_compress.py)."""
    g = np.load(COMPRESS_GOLDEN)
    names = sorted({k.split("_")[0] for k in g.files})
    for n in names:
        bs = int(g[n + "_bs"][0])
        off, col, val = oracle.bsr_compress_rows(g[n + "_offsets"], g[n + "_counts"], g[n + "_cols"], g[n + "_vals"],
                                                 bs, bool(prune))
        np.testing.assert_array_equal(off, g[f"{n}_p{prune}_offsets"])
        np.testing.assert_array_equal(col, g[f"{n}_p{prune}_columns"])
        np.testing.assert_array_equal(val.reshape(-1).view(np.uint32),
                                      g[f"{n}_p{prune}_values"].reshape(-1).view(np.uint32))


def test_compress_restatement_matches_live_reference():
    if oracle.ref_lib() is None:
        pytest.skip("reference library not built here")
    rng = np.random.default_rng(5)
    counts = rng.integers(0, 40, 25).astype(np.int32)
    offsets = np.concatenate([[0], np.cumsum(counts + 1)]).astype(np.int32)
    cols = rng.integers(-1, 15, int(offsets[-1])).astype(np.int32)
    vals = rng.standard_normal(int(offsets[-1])).astype(np.float32)
    vals[rng.random(vals.size) < 0.2] = 0.0
    r = oracle.ref_bsr_compress(offsets, counts, cols, vals)
    off, col, val = oracle.bsr_compress_rows(offsets, counts, cols, vals)
    np.testing.assert_array_equal(off, r["offsets"])
    np.testing.assert_array_equal(col, r["columns"])
    np.testing.assert_array_equal(val.reshape(-1), r["values"].reshape(-1))


def test_krylov_restatements_converge_to_direct_solutions():
    """The CR / GMRES restatements (oracle.krylov) reach their tolerance and the direct solution."""
    from oracle import krylov

    rng = np.random.default_rng(4)
    Q = rng.standard_normal((40, 40))
    S = Q @ Q.T + 40 * np.eye(40)
    b = rng.standard_normal(40)
    xs = np.linalg.solve(S, b)
    for dinv in (None, 1.0 / np.diag(S)):
        x, it, res = krylov.cr(S, b, dinv=dinv, tol=1e-10, atol=0.0)
        assert res <= 1e-10 * np.linalg.norm(b) and np.allclose(x, xs, rtol=1e-7, atol=1e-9) and 0 < it < 40
    N_ = 4 * np.eye(50) + 0.3 * rng.standard_normal((50, 50))
    b = rng.standard_normal(50)
    xs = np.linalg.solve(N_, b)
    for dinv, left in ((None, False), (1.0 / np.diag(N_), False), (1.0 / np.diag(N_), True)):
        x, it, res = krylov.gmres(N_, b, dinv=dinv, tol=1e-10, atol=0.0, restart=8, left=left)
        assert np.linalg.norm(N_ @ x - b) <= 1e-10 * np.linalg.norm(b) and it % 8 == 0
        assert np.allclose(x, xs, rtol=1e-7, atol=1e-9)


def test_oracle_structure_matches_reference_routine_at_configs():
    """The oracle's triplet->BSR of the configuration systems equals the reference's compiled routine
    (tests/golden/config_structure_ref.npz), offsets, columns and run ends."""
    import os

    from oracle import fem_q1

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config_structure_ref.npz"))
    for name in ("cfg1", "q1_2d_irregular", "elasticity_6x5x4"):
        meta = g[name + "_meta"]
        dim = int(meta[0])
        res = tuple(int(k) for k in meta[1:1 + dim])
        ncomp = int(meta[4])
        if name == "cfg1":
            r, c, v = fem_q1.assemble_triplets(res, coef=1.0)
        elif ncomp == 1:
            r, c, v = fem_q1.assemble_triplets(res, coef=g[name + "_coef"])
        else:
            E = g[name + "_young"]
            lam = E * 0.3 / (1.3 * 0.4)
            mu = E / 2.6
            r, c, v = fem_q1.assemble_triplets(res, ncomp=3, lame=(lam.astype(np.float32), mu.astype(np.float32)))
        nn = int(np.prod([k + 1 for k in res]))
        o = oracle.bsr_from_triplets(nn, nn, r, c, v.reshape(len(r), ncomp * ncomp), block_shape=(ncomp, ncomp))
        assert o["nnz"] == int(meta[5]) == len(g[name + "_columns"])
        np.testing.assert_array_equal(o["offsets"], g[name + "_offsets"])
        np.testing.assert_array_equal(o["columns"], g[name + "_columns"])
        np.testing.assert_array_equal(o["tpl_block_offsets"], g[name + "_runends"])


def test_oracle_stencil_assembly_equals_triplet_assembly():
    """The CPU baseline's stencil-form assembly (every node's 27-neighbourhood) gives the triplet
    route's unpruned matrix: same structure, values equal up to FP64 summation order."""
    from oracle import fem_q1

    res = (6, 5, 4)
    coef = np.exp(np.random.default_rng(0).standard_normal(120)).astype(np.float32)
    off, cols, vals = fem_q1.assemble_csr_stencil(res, coef)
    r, c, v = fem_q1.assemble_triplets(res, coef=coef)
    nn = 7 * 6 * 5
    o = oracle.bsr_from_triplets(nn, nn, r, c, v, prune_numerical_zeros=False)
    np.testing.assert_array_equal(o["offsets"], off)
    np.testing.assert_array_equal(o["columns"], cols)
    assert np.abs(o["values"] - vals).max() <= 1e-6 * np.abs(vals).max()


def test_oracle_random_field_equals_product_field_generator():
    from oracle import fem_q1
    from warp_gb300 import fem

    np.testing.assert_array_equal(fem.gaussian_random_field((8, 9, 10), 0.1, 1.5, 3),
                                  fem_q1.gaussian_random_field((8, 9, 10), 0.1, 1.5, 3))
