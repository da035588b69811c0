"""Permanents modulo 3 on the GPU.

Mirrors rivin-perm's ``perm_mod3.py`` public entry points with the same
validation and results:

  permanent_mod3_fast(matrix, num_threads=None)   perm_mod3.py:355-383
  encode_matrix_f3(matrix) / decode_f3_element    perm_mod3.py:62-115

The evaluation is ``pg_permanent_mod3`` (Ryser over F_3 with bit-sliced row
sums, one launch); there is no CPU path.
"""

from __future__ import annotations

from numbers import Integral
from typing import Tuple

import numpy as np

from . import _lib


def _validate_num_threads(num_threads):
    if num_threads is None:
        return None
    if isinstance(num_threads, bool) or not isinstance(num_threads, Integral):
        raise TypeError("num_threads must be a positive integer or None")
    num_threads = int(num_threads)
    if num_threads <= 0:
        raise ValueError("num_threads must be positive")
    return num_threads


def _as_square_integer_matrix(matrix) -> np.ndarray:
    try:
        matrix = np.asarray(matrix)
    except ValueError as exc:
        raise ValueError("Matrix must be a rectangular two-dimensional array") from exc
    if matrix.ndim == 1 and matrix.size == 0:
        matrix = np.empty((0, 0), dtype=np.int64)
    if matrix.ndim != 2:
        raise ValueError("Matrix must be two-dimensional")
    if matrix.shape[0] != matrix.shape[1]:
        raise ValueError("Matrix must be square")
    if not np.issubdtype(matrix.dtype, np.integer):
        raise TypeError("Matrix entries must be integers")
    return matrix


def encode_f3_element(x: int) -> Tuple[int, int]:
    """(magnitude, sign) bits of x mod 3: 0 -> (0,0), 1 -> (1,0), 2 -> (1,1)."""
    v = int(x) % 3
    return (0, 0) if v == 0 else ((1, 0) if v == 1 else (1, 1))


def decode_f3_element(mag: int, sgn: int) -> int:
    """Element of {0, 1, 2} from its (magnitude, sign) bits."""
    if not mag:
        return 0
    return 2 if sgn else 1


def encode_matrix_f3(matrix) -> Tuple[np.ndarray, np.ndarray]:
    """Column encodings: bit i of mags[j] set when a_ij != 0 (mod 3), bit i
    of sgns[j] set when a_ij == 2 (mod 3)."""
    a = _as_square_integer_matrix(matrix)
    n = a.shape[0]
    if n >= 64:
        raise ValueError("Matrix size must be less than 64 for bipedal encoding")
    r = np.mod(a, 3).astype(np.int64) if n else a
    mags = np.zeros(n, dtype=np.uint64)
    sgns = np.zeros(n, dtype=np.uint64)
    for j in range(n):
        m = s = 0
        for i in range(n):
            if r[i, j]:
                m |= 1 << i
                if r[i, j] == 2:
                    s |= 1 << i
        mags[j], sgns[j] = m, s
    return mags, sgns


def permanent_mod3_fast(matrix, num_threads=None) -> int:
    """per(matrix) mod 3 in {0, 1, 2}; order < 64, integer entries of any
    size (reduced mod 3 on the host)."""
    a = _as_square_integer_matrix(matrix)
    _validate_num_threads(num_threads)
    n = a.shape[0]
    if n >= 64:
        raise ValueError("Matrix size must be less than 64")
    if n == 0:
        return 1
    if n == 1:
        return int(a[0, 0]) % 3
    return _lib.permanent_mod3(np.mod(a, 3).astype(np.int64))
