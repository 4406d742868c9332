"""CPU oracle for the block-sparse symmetric tensor path of Xped.

TEST INFRASTRUCTURE ONLY.  This package is a plain-Python/numpy restatement of
the reference algorithms (sector bookkeeping, fusion trees, permute, block
GEMM, truncated SVD/QR, the CTM moves).  It exists to check the GPU backend
in ``xped_gb300``; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import it.  The product never routes through
it: the GPU path raises when its CUDA library is missing.

Each function cites the reference file:line it follows (paths relative to the
Xped source tree).  The reference itself cannot be built here (Eigen, Boost,
GSL, stan-math ... are absent), so parity is pinned by the reference's own
test properties (permute == dense shuffle, fusion-tree round trips, norm
identities) and by exact SU(2) 6j values from sympy; see tests/test_oracle_*.
"""

from .sym import U1, ZN, SU2, make_symmetry  # noqa: F401
from .basis import FusionTree, Qbasis, build_fusion_tree  # noqa: F401
from .tensor import Tensor  # noqa: F401
