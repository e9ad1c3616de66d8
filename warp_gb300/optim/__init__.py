"""Solvers of the FEM linear-solve path (drop-in for ``warp.optim.linear``)."""

from . import linear  # noqa: F401
