"""CPU ORACLE for the FEM linear-solve path -- test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg (and its
``--impl reference`` arm) import this package; the product package ``warp_gb300`` never does.

Contents:
  * ``liboracle.so`` (``gbfem_oracle.c``): C restatements of the reference's triplet->BSR
    topology build, value accumulation, BSR SpMV, Jacobi inverse diagonal, PCG and BiCGSTAB,
    each citing the reference file:line it follows.
  * ``_ref/libref_sparse.so``: the reference's own host routine
    ``wp_bsr_matrix_from_triplets_host`` (warp/native/sparse.cpp:267-413) compiled from the
    unmodified Warp source file; only present where the Warp source tree was available at build
    time.  It pins the C restatement (``tests/golden/`` freezes its outputs).
  * ``fem_q1.py``: NumPy FP64 restatement of Q1 bilinear-form assembly on Grid2D/Grid3D, the
    triplet ordering of the reference's dispatch kernel, right-hand sides and the Dirichlet
    projection.
"""

from .oracle import *  # noqa: F401,F403
