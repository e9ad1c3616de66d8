"""warp_gb300 -- GB300-native (sm_103a) implementation of Warp's finite-element linear-solve path.

Drop-in modules:
  * ``warp_gb300.sparse``        for ``warp.sparse`` (BSR assembly from triplets, SpMV, SpGEMM)
  * ``warp_gb300.optim.linear``  for ``warp.optim.linear`` (CG, BiCGSTAB, Jacobi, LinearOperator)
  * ``warp_gb300.fem``           for the ``warp.fem`` calls of the path (Q1 grids, integrate,
                                 Dirichlet projection)
All numerical work runs in ``libwarp_gb300.so`` (hand-written CUDA for sm_103a) called through a
C ABI (``include/warp_gb300.h``); PyTorch provides device memory and streams only.
"""

from . import _native  # noqa: F401
from ._arrays import ScopedStream  # noqa: F401
from . import sparse  # noqa: F401
from . import optim  # noqa: F401
from . import fem  # noqa: F401
from . import spgemm  # noqa: F401

__version__ = "1.0.0"


def build(verbose: bool = False) -> str:
    """Compile libwarp_gb300.so in-tree for sm_103a."""
    from ._build import build as _b

    return _b(verbose=verbose)
