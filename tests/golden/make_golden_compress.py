"""Generates tests/golden/compress_ref.npz from the reference's OWN compiled host routine
wp_bsr_compress_inplace_host (warp/native/sparse.cpp:521-610 -> sparse_util.h:82-139, built into
oracle/_ref by oracle/Makefile from the unmodified Warp sources).

Run from the repository root in a checkout where the Warp sources are available:
    make -C oracle && python tests/golden/make_golden_compress.py
Each case is a padded BSR (offsets + row_counts with slack, duplicate columns, negative columns,
zero and -0 blocks) compressed with and without numerical-zero pruning into compact storage.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def cases():
    rng = np.random.default_rng(20261205)
    out = []
    # (rows, columns, max candidates per row, block size); row lengths up to 200 exercise the long-row path
    for k, (nrow, ncol, cap, bs) in enumerate([(1, 4, 5, 1), (10, 8, 12, 1), (60, 30, 64, 1), (40, 25, 64, 9),
                                               (20, 500, 200, 1), (30, 12, 40, 4)]):
        counts = rng.integers(0, cap + 1, nrow)
        slack = rng.integers(0, 3, nrow)
        offsets = np.concatenate([[0], np.cumsum(counts + slack)]).astype(np.int32)
        n = int(offsets[-1])
        cols = rng.integers(-1, ncol, n).astype(np.int32)
        vals = rng.standard_normal((n, bs)).astype(np.float32)
        zero = rng.random(n) < 0.1
        vals[zero] = 0.0
        negz = rng.random(n) < 0.05
        vals[negz] = -0.0
        out.append((f"case{k}", offsets, counts.astype(np.int32), cols, vals, bs))
    return out


def main():
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libref_sparse.so not built (needs the Warp sources)")
    data = {}
    for name, offsets, counts, cols, vals, bs in cases():
        data[name + "_offsets"] = offsets
        data[name + "_counts"] = counts
        data[name + "_cols"] = cols
        data[name + "_vals"] = vals
        data[name + "_bs"] = np.array([bs], np.int32)
        for prune in (0, 1):
            r = oracle.ref_bsr_compress(offsets, counts, cols, vals, block_size=bs, prune_numerical_zeros=bool(prune))
            data[f"{name}_p{prune}_offsets"] = r["offsets"]
            data[f"{name}_p{prune}_columns"] = r["columns"]
            data[f"{name}_p{prune}_values"] = r["values"]
    np.savez_compressed(os.path.join(HERE, "compress_ref.npz"), **data)
    print("wrote", os.path.join(HERE, "compress_ref.npz"), len(data), "arrays")


if __name__ == "__main__":
    main()
