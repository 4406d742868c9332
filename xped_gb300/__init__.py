"""GB300-native backend for Xped's block-sparse symmetric tensor hot path.

Native pieces (xped_gb300/csrc, built in-tree to xped_gb300/_lib/libxgb.so):
  * meta.cpp    - symmetry algebra, fusion trees, leg bases (host C++)
  * tensor.cpp  - device tensors, cached permute/GEMM/SVD plans, CTM moves
  * kernels.cu  - sm_103a kernels: grouped GEMM, permute, batched QR,
                  truncation, normalisation
  * svd.cu      - batched cluster Jacobi SVD (mixed FP32 / FP64)
  * rsvd.cu/.cpp - randomized blockwise tSVD (sketch, subspace iterations)
  * mlp.cu/.cpp - rank-predictor MLP (forward, backward, Adam) and its
                  sketch-width policy
  * capi.cpp    - the C-ABI (include/xgb.h, include/xgb_tensor.h)
This package only binds that library; it has no CPU implementation of the
hot path and raises if the library has not been built.
"""
from ._lib import XgbError, ensure_device, lib  # noqa: F401
from .tensor import CTM, Basis, SimpleUpdate, Tensor, bond_expectation, contract_perms, decompose  # noqa: F401
from .learn import RankModel  # noqa: F401

__all__ = ["Basis", "Tensor", "CTM", "SimpleUpdate", "RankModel", "bond_expectation", "decompose", "contract_perms", "XgbError",
           "ensure_device", "lib"]
