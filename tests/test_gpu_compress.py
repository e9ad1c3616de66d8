"""GPU tests of the row-local compression (bsr_compress, fem.integrate row_compress construction)
against the reference's compiled routine (golden fixture) and against the triplet construction."""

import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "compress_ref.npz")


@pytest.mark.parametrize("prune", [False, True])
def test_bsr_compress_matches_reference_golden(cuda, prune):
    """Padded rows with slack, duplicates, negative columns, zero and -0 blocks, rows up to 200
    candidates (the serial long-row path): bit-exact offsets, columns and values."""
    from warp_gb300 import sparse

    g = np.load(GOLDEN)
    names = sorted({k.split("_")[0] for k in g.files})
    for n in names:
        bs = int(g[n + "_bs"][0])
        offsets, counts = g[n + "_offsets"], g[n + "_counts"]
        nrow = len(offsets) - 1
        shape = (1, 1) if bs == 1 else {4: (2, 2), 9: (3, 3)}[bs]
        M = sparse.bsr_zeros(nrow, 1 << 20, torch.float32 if bs == 1 else (shape, torch.float32))
        M.offsets = torch.from_numpy(offsets).cuda()
        M.row_counts = torch.from_numpy(counts).cuda()
        M.columns = torch.from_numpy(g[n + "_cols"]).cuda()
        vals = torch.from_numpy(g[n + "_vals"]).cuda()
        M.values = vals.reshape(-1) if bs == 1 else vals.reshape(-1, *shape)
        M.nnz = int(offsets[-1])
        sparse.bsr_compress(M, prune_numerical_zeros=prune)
        nnz = M.nnz_sync()
        p = int(prune)
        np.testing.assert_array_equal(M.offsets.cpu().numpy(), g[f"{n}_p{p}_offsets"])
        np.testing.assert_array_equal(M.columns[:nnz].cpu().numpy(), g[f"{n}_p{p}_columns"])
        got = M.values[:nnz].reshape(-1).cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(got, g[f"{n}_p{p}_values"].reshape(-1).view(np.uint32))
        assert M.row_counts is None


@pytest.mark.parametrize("case", ["diffusion3d", "diffusion2d", "elasticity"])
def test_row_compress_construction_equals_triplets(cuda, case):
    """fem.integrate with bsr_options={"construction": "row_compress"} gives the triplet construction's
    matrix bit for bit (structure and values): same candidates, same summation order."""
    from warp_gb300 import fem

    rng = np.random.default_rng(3)
    if case == "elasticity":
        geo = fem.Grid3D(res=(6, 5, 7))
        space = fem.make_polynomial_space(geo, degree=1, dtype="vec3")
        lam = rng.uniform(1, 3, geo.cell_count()).astype(np.float32)
        mu = rng.uniform(1, 3, geo.cell_count()).astype(np.float32)
        form, values = fem.linear_elasticity_form, {"lame": (lam, mu)}
    else:
        geo = fem.Grid3D(res=(16, 12, 9)) if case == "diffusion3d" else fem.Grid2D(res=(33, 20))
        space = fem.make_polynomial_space(geo, degree=1)
        form, values = fem.diffusion_form, {"nu": np.exp(rng.standard_normal(geo.cell_count())).astype(np.float32)}
    fields = {"u": fem.make_trial(space), "v": fem.make_test(space)}
    A1 = fem.integrate(form, fields=fields, values=values)
    A2 = fem.integrate(form, fields=fields, values=values, bsr_options={"construction": "row_compress"})
    n1, n2 = A1.nnz_sync(), A2.nnz_sync()
    assert n1 == n2
    assert torch.equal(A1.offsets, A2.offsets)
    assert torch.equal(A1.columns[:n1], A2.columns[:n2])
    v1 = A1.values[:n1].reshape(-1).cpu().numpy().view(np.uint32)
    v2 = A2.values[:n2].reshape(-1).cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(v1, v2)


def test_compress_padded_topology_keeps_row_capacity(cuda):
    from warp_gb300 import sparse

    offsets = torch.tensor([0, 4, 4, 9], dtype=torch.int32, device="cuda")
    cols = torch.tensor([3, 1, 3, -1, 2, 2, 0, 7, 0], dtype=torch.int32, device="cuda")
    vals = torch.tensor([1.0, 2.0, 3.0, 9.0, 4.0, 5.0, 6.0, 0.0, 7.0], device="cuda")
    M = sparse.bsr_zeros(3, 8, torch.float32)
    M.offsets, M.columns, M.values, M.nnz = offsets, cols, vals, 9
    sparse.bsr_compress(M, topology="padded")
    assert torch.equal(M.offsets, offsets)
    assert M.row_counts.tolist() == [2, 0, 2]
    assert M.columns[:2].tolist() == [1, 3] and M.values[:2].tolist() == [2.0, 4.0]
    assert M.columns[4:6].tolist() == [0, 2] and M.values[4:6].tolist() == [13.0, 9.0]
