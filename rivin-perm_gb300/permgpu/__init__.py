"""permgpu — GB300 (sm_103a) exact-permanent engines behind a C ABI.

Public API (mirrors rivin-perm):
  matrix_permanent(A, ..., method="generic")   perm.matrix_permanent
  permanent(n) / schur_permanent_of_size(n)    perm.permanent
  binary_permanent(A), binary_permanent_mod_p  perm_binary.*
  GpuExt, BinaryGpuExt                         drop-ins for perm_c_ext /
                                               perm_binary_ext
"""

from ._lib import PermGpuError, cuda_available, load
from .binary import (binary_permanent, binary_permanent_bound,
                     binary_permanent_mod_p)
from .crt import (graham_lehmer_congruence, matrix_permanent_bound,
                  schur_permanent_bound)
from .ext import BinaryGpuExt, GpuExt
from .generic import matrix_permanent, permanent, schur_permanent_of_size

__all__ = [
    "BinaryGpuExt", "GpuExt", "PermGpuError", "binary_permanent",
    "binary_permanent_bound", "binary_permanent_mod_p", "cuda_available",
    "graham_lehmer_congruence", "load", "matrix_permanent",
    "matrix_permanent_bound", "permanent", "schur_permanent_bound",
    "schur_permanent_of_size",
]
