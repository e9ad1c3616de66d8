"""Generates tests/golden/triplets_ref.npz from the reference's OWN compiled host routine
wp_bsr_matrix_from_triplets_host (warp/native/sparse.cpp:267-413, built into oracle/_ref by
oracle/Makefile from the unmodified Warp source file).

Run from the repository root in a checkout where the Warp sources are available:
    make -C oracle && python tests/golden/make_golden.py
The fixture freezes, for seeded random triplet sets (with invalid indices, zero blocks and
duplicates), the reference's BSR offsets, columns and run ends, plus the sorted set of triplet
ids of each run (the host routine's std::sort is unstable, so only the set is defined).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def cases():
    rng = np.random.default_rng(20261204)
    out = []
    shapes = [(2, 3, 3, 1), (8, 6, 100, 1), (4, 9, 50, 6), (50, 40, 600, 1), (300, 300, 4000, 9), (1, 1, 5, 1),
              (1000, 7, 3000, 1), (7, 1000, 3000, 4)]
    for k, (nrow, ncol, n, bs) in enumerate(shapes):
        rows = rng.integers(-2, nrow + 2, n).astype(np.int32)
        cols = rng.integers(-2, ncol + 2, n).astype(np.int32)
        vals = rng.random((n, bs)).astype(np.float32)
        zero = rng.random(n) < 0.15
        vals[zero] = 0.0
        if bs > 1:
            neg0 = rng.random(n) < 0.05
            vals[neg0] = -0.0
        out.append((f"case{k}", nrow, ncol, rows, cols, vals, bs))
    return out


def main():
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libref_sparse.so not built (needs the Warp sources)")
    data = {}
    for name, nrow, ncol, rows, cols, vals, bs in cases():
        for prune in (0, 1):
            r = oracle.ref_bsr_from_triplets(nrow, ncol, rows, cols, vals, block_size=bs,
                                             prune_numerical_zeros=bool(prune))
            key = f"{name}_p{prune}"
            data[key + "_meta"] = np.array([nrow, ncol, bs, prune, r["nnz"]], np.int64)
            data[key + "_offsets"] = r["offsets"]
            data[key + "_columns"] = r["columns"]
            data[key + "_runends"] = r["tpl_block_offsets"]
            # canonical (sorted) run membership
            idx = r["tpl_block_indices"].copy()
            beg = 0
            for b, end in enumerate(r["tpl_block_offsets"]):
                idx[beg:end] = np.sort(idx[beg:end])
                beg = end
            data[key + "_runidx"] = idx[: (r["tpl_block_offsets"][-1] if r["nnz"] else 0)]
        data[name + "_rows"] = rows
        data[name + "_cols"] = cols
        data[name + "_vals"] = vals
    np.savez_compressed(os.path.join(HERE, "triplets_ref.npz"), **data)
    print("wrote", os.path.join(HERE, "triplets_ref.npz"), len(data), "arrays")


if __name__ == "__main__":
    main()
