"""permgpu — GB300 (sm_103a) exact-permanent engines behind a C ABI.

Public API (mirrors rivin-perm):
  matrix_permanent(A, ..., method="generic")   perm.matrix_permanent
  permanent(n) / schur_permanent_of_size(n)    perm.permanent
  binary_permanent(A), binary_permanent_mod_p  perm_binary.*
  GpuExt, BinaryGpuExt                         drop-ins for perm_c_ext /
                                               perm_binary_ext
  affine_permanent, rook_polynomial, ...       perm_polynomial.* (permgpu.poly)
  permanent_gpu, permanent_float,              perm_cuda / perm_float, and the
  glynn_permanent                              FP64 autograd permanent
                                               (permgpu.f64; imports torch)
"""

from ._lib import PermGpuError, cuda_available, load
from .binary import (binary_permanent, binary_permanent_bound,
                     binary_permanent_mod_p)
from .crt import (graham_lehmer_congruence, matrix_permanent_bound,
                  schur_permanent_bound)
from .ext import BinaryGpuExt, GpuExt
from .generic import matrix_permanent, permanent, schur_permanent_of_size
from .poly import (affine_permanent, affine_permanent_bounds, affine_permanent_mod,
                   principal_permanent_polynomial, principal_permanent_polynomial_mod,
                   rook_polynomial, weighted_rook_polynomial)

_F64_NAMES = ("permanent_gpu", "permanent_float", "glynn_permanent", "permanent_f64",
              "permanent_c64")


def __getattr__(name):
    # the FP64 engine needs torch; import it only when asked for
    if name in _F64_NAMES:
        from . import f64
        return getattr(f64, name)
    raise AttributeError(f"module 'permgpu' has no attribute {name!r}")


__all__ = [
    "BinaryGpuExt", "GpuExt", "PermGpuError", "affine_permanent",
    "affine_permanent_bounds", "affine_permanent_mod", "binary_permanent",
    "binary_permanent_bound", "binary_permanent_mod_p", "cuda_available",
    "graham_lehmer_congruence", "load", "matrix_permanent",
    "matrix_permanent_bound", "permanent", "principal_permanent_polynomial",
    "principal_permanent_polynomial_mod", "rook_polynomial",
    "schur_permanent_bound", "schur_permanent_of_size", "weighted_rook_polynomial",
    *_F64_NAMES,
]
