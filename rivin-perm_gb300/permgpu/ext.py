"""Drop-in extension objects for rivin-perm's native seams.

``GpuExt`` exposes the method names of the ``perm_c_ext`` module that
perm.py calls (perm.py:917-923 ``permanent_mod_p`` / ``ryser_permanent_mod_p``,
perm.py:752-753 ``schur_permanent_mod_p``, perm.py:855,1141
``get_max_threads``); ``BinaryGpuExt`` exposes ``binary_permanent_mod_p``
of ``perm_binary_ext`` (perm_binary.py:822-824).  Argument validation and
error types follow the C extensions (perm_c_omp.c:858-929, 942-970;
perm_binary_omp.c:386-460) so a module swap is transparent:

    import perm, permgpu
    perm.perm_c_ext = permgpu.GpuExt(); perm.HAS_C_EXT = True
    import perm_binary
    perm_binary._binary_ext = permgpu.BinaryGpuExt(); perm_binary.HAS_BINARY_EXT = True
"""

from __future__ import annotations

import operator
from numbers import Integral

import numpy as np

from . import _lib

_INT64_MIN = -(1 << 63)
_INT64_MAX = (1 << 63) - 1
_INT_MAX = (1 << 31) - 1


def _parse_long_long(value, name: str) -> int:
    # PyArg_ParseTuple "L": integers only (floats are a TypeError), range
    # checked into an OverflowError.
    if isinstance(value, float) or not hasattr(value, "__index__"):
        raise TypeError(f"{name} must be an integer")
    v = operator.index(value)
    if not _INT64_MIN <= v <= _INT64_MAX:
        raise OverflowError(f"{name} does not fit in a signed 64-bit integer")
    return int(v)


def _parse_int(value, name: str) -> int:
    if isinstance(value, float) or not hasattr(value, "__index__"):
        raise TypeError(f"{name} must be an integer")
    v = operator.index(value)
    if not -(1 << 31) <= v <= _INT_MAX:
        raise OverflowError(f"{name} does not fit in a C int")
    return int(v)


def _matrix_from_lists(matrix_obj, p: int) -> np.ndarray:
    if not isinstance(matrix_obj, list):
        raise TypeError("matrix must be a list of lists")
    n = len(matrix_obj)
    if p <= 0:
        raise ValueError("p must be a positive signed 64-bit integer")
    if n >= 64:
        raise ValueError("matrix dimension must be less than 64")
    out = np.zeros((n, n), dtype=np.int64)
    for i, row in enumerate(matrix_obj):
        if not isinstance(row, list) or len(row) != n:
            raise ValueError("matrix must be square")
        for j, item in enumerate(row):
            out[i, j] = _parse_long_long(item, "matrix entry")
    return out


class GpuExt:
    """GPU stand-in for the ``perm_c_ext`` CPython extension module."""

    def __init__(self):
        self._threads = 1

    def permanent_mod_p(self, matrix, p, num_threads=0):
        p = _parse_long_long(p, "p")
        _parse_int(num_threads, "num_threads")
        a = _matrix_from_lists(matrix, p)
        if a.shape[0] == 0:
            return 1 % p
        return _lib.residues(a, [p])[0]

    # The explicit Ryser entry point computes the same residue.
    ryser_permanent_mod_p = permanent_mod_p

    def schur_permanent_mod_p(self, n, omega, p, num_threads=0):
        n = _parse_int(n, "n")
        omega = _parse_long_long(omega, "omega")
        p = _parse_long_long(p, "p")
        _parse_int(num_threads, "num_threads")
        if n < 0 or n >= 64:
            raise ValueError("n must satisfy 0 <= n < 64")
        if p <= 0:
            raise ValueError("p must be a positive signed 64-bit integer")
        if n <= 1:
            return 1 % p
        if p == 1:
            return 0
        return _lib.schur_residues(n, [p], [omega % p])[0]

    def schur_necklace_orbit_stats(self, n):
        """(representatives, covered sign words) of the necklace quotient;
        perm_c_omp.c:1062-1082 semantics (ValueError unless n is an odd
        prime with 3 <= n < 64).  Host only."""
        return _lib.necklace_orbit_stats(_parse_int(n, "n"))

    def get_max_threads(self):
        return self._threads

    def set_num_threads(self, num_threads):
        num_threads = _parse_int(num_threads, "num_threads")
        if num_threads <= 0:
            raise ValueError("num_threads must be positive")
        self._threads = num_threads


class BinaryGpuExt:
    """GPU stand-in for the ``perm_binary_ext`` CPython extension module."""

    def binary_permanent_mod_p(self, matrix, p, num_threads=0):
        try:
            p = operator.index(p)
        except TypeError as exc:
            raise TypeError("p must be an integer") from exc
        try:
            num_threads = operator.index(num_threads)
        except TypeError as exc:
            raise TypeError("num_threads must be an integer") from exc
        if num_threads > _INT_MAX:
            raise ValueError("num_threads is too large")
        if num_threads < 0:
            raise ValueError("num_threads must be non-negative")
        try:
            rows = list(matrix)
        except TypeError as exc:
            raise TypeError("matrix must be a sequence of rows") from exc
        n = len(rows)
        if n > 63:
            raise ValueError("native binary backend supports order at most 63")
        if p <= 1:
            raise ValueError("p must be greater than 1")
        if p == 2:
            raise ValueError("p must be odd")
        if p <= n:
            raise ValueError("p must be greater than the matrix order")
        if p > _INT64_MAX:
            raise OverflowError("p does not fit in a signed 64-bit integer")
        a = np.zeros((n, n), dtype=np.uint8)
        for i, row in enumerate(rows):
            row = list(row)
            if len(row) != n:
                raise ValueError("matrix must be square")
            for j, v in enumerate(row):
                v = operator.index(v)
                if v not in (0, 1):
                    raise ValueError("binary matrix entries must be 0 or 1")
                a[i, j] = v
        try:
            return _lib.binary_residues(a, [p])[0]
        except _lib.PermGpuError as exc:
            if exc.status == _lib.PG_ERANGE:
                raise ValueError(str(exc)) from exc
            raise
