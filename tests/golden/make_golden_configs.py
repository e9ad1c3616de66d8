"""Generates tests/golden/config_structure_ref.npz: BSR structure of assembled FEM systems at the
benchmark configurations' small sizes, produced by the reference's OWN compiled host routine
wp_bsr_matrix_from_triplets_host (warp/native/sparse.cpp:267-413, built into oracle/_ref by
oracle/Makefile from the unmodified Warp source file).

Cases (the triplets are the Q1 dispatch-order triplets of the oracle's FP64 restatement,
oracle/fem_q1.py, with numerical-zero pruning on as fem.integrate does by default,
warp/_src/fem/integrate.py:1855):
  * cfg1: Grid2D 64 x 64 Q1 Poisson (nu = 1), 4225 nodes;
  * q1_2d_irregular: Grid2D 13 x 7, lognormal per-cell coefficient;
  * elasticity_6x5x4: Grid3D 6 x 5 x 4 Q1 vec3 elasticity (3x3 blocks), lognormal Young's modulus.
No block of these systems is zero in exact arithmetic (2-D Q1 stiffness couples every node with its
3 x 3 neighbourhood; every 3x3 elasticity block has a nonzero entry), so their pruned structure
does not depend on rounding and the fixture pins the structure the GPU assembly must reproduce.

Run from the repository root where the Warp sources are available:
    make -C oracle && python tests/golden/make_golden_configs.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from oracle import fem_q1  # noqa: E402


def cases():
    rng = np.random.default_rng(7)
    out = [("cfg1", (64, 64), 1, fem_q1.assemble_triplets((64, 64), coef=1.0))]
    nu = np.exp(rng.standard_normal(13 * 7)).astype(np.float32)
    out.append(("q1_2d_irregular", (13, 7), 1, fem_q1.assemble_triplets((13, 7), coef=nu)))
    E = 1e3 * np.exp(rng.standard_normal(6 * 5 * 4))
    nu_p = 0.3
    lam = E * nu_p / ((1 + nu_p) * (1 - 2 * nu_p))
    mu = E / (2 * (1 + nu_p))
    out.append(("elasticity_6x5x4", (6, 5, 4), 3,
                fem_q1.assemble_triplets((6, 5, 4), ncomp=3, lame=(lam.astype(np.float32), mu.astype(np.float32)))))
    return out, nu, E


def main():
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libref_sparse.so not built (needs the Warp sources)")
    data = {}
    all_cases, nu, E = cases()
    for name, res, ncomp, (r, c, v) in all_cases:
        nn = int(np.prod([k + 1 for k in res]))
        ref = oracle.ref_bsr_from_triplets(nn, nn, r, c, v.reshape(len(r), ncomp * ncomp), block_size=ncomp * ncomp,
                                           prune_numerical_zeros=True)
        data[name + "_meta"] = np.array([len(res), *res, *([0] * (3 - len(res))), ncomp, ref["nnz"]], np.int64)
        data[name + "_offsets"] = ref["offsets"]
        data[name + "_columns"] = ref["columns"]
        data[name + "_runends"] = ref["tpl_block_offsets"]
    data["q1_2d_irregular_coef"] = nu
    data["elasticity_6x5x4_young"] = E
    np.savez_compressed(os.path.join(HERE, "config_structure_ref.npz"), **data)
    print("wrote", os.path.join(HERE, "config_structure_ref.npz"), {k: v.shape for k, v in data.items()})


if __name__ == "__main__":
    main()
