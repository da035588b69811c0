"""Exact integer and Schur permanents on the GPU.

``matrix_permanent`` keeps the signature and results of rivin-perm
``perm.matrix_permanent`` (perm.py:1076-1212); ``permanent`` /
``schur_permanent_of_size`` those of perm.py:1219-1244.

Engine choice for integer matrices:
  * exact engine (pg_exact_permanent) whenever every row-sum bound
    sum_j |a_ij| < 2^30 and the order is <= 48: one traversal, exact integer
    row sums, exact multi-word Glynn terms, no CRT;
  * otherwise residues modulo descending primes below 2^31 (one launch for
    all primes) and the signed CRT lift of perm.py:1207-1210.
"""

from __future__ import annotations

from numbers import Integral
from typing import List, Optional

import numpy as np

from . import _lib
from .crt import (descending_primes, matrix_permanent_bound, nth_root_of_unity,
                  plan_schur, signed_lift, crt)


def _validate_integer_matrix(matrix) -> int:
    shape = getattr(matrix, "shape", None)
    if shape is not None:
        if len(shape) != 2:
            raise ValueError("Matrix must be two-dimensional")
        if shape[0] != shape[1]:
            raise ValueError("Matrix must be square")
    try:
        n = len(matrix)
    except TypeError as exc:
        raise TypeError("Matrix must be a sequence of rows") from exc
    for row in matrix:
        try:
            width = len(row)
        except TypeError as exc:
            raise TypeError("Matrix rows must be sequences") from exc
        if width != n:
            raise ValueError("Matrix must be square")
        for entry in row:
            if not isinstance(entry, Integral):
                raise TypeError("Matrix entries must be integers")
    return n


def _validate_threads(num_threads) -> int:
    if isinstance(num_threads, bool) or not isinstance(num_threads, Integral):
        raise TypeError("num_threads must be an integer")
    if num_threads < 0:
        raise ValueError("num_threads must be non-negative")
    return int(num_threads)


def residue_plan(bound: int) -> List[int]:
    """Primes (< 2^31, descending) whose product is >= 2*bound + 1."""
    return descending_primes(2 * bound + 1)


def matrix_permanent(matrix, verbose: bool = False, parallel: bool = True,
                     num_threads: int = 0, *, method: str = "auto",
                     engine: str = "auto") -> int:
    """Exact permanent of an integer matrix (perm.matrix_permanent API).

    ``method`` accepts 'auto' and 'generic' (both run the GPU generic path;
    the CPU low-rank specialisation of perm.py:956-1073 is not part of this
    engine, so 'low_rank' raises).  ``engine`` selects 'auto', 'exact' or
    'residue' for testing either GPU path directly.
    """
    n = _validate_integer_matrix(matrix)
    _validate_threads(num_threads)
    if not isinstance(method, str):
        raise TypeError("method must be a string")
    method = method.lower()
    if method not in ("auto", "generic", "low_rank"):
        raise ValueError("method must be one of: 'auto', 'generic', 'low_rank'")
    if method == "low_rank":
        raise ValueError("the GPU engine implements method='generic' only")
    if engine not in ("auto", "exact", "residue"):
        raise ValueError("engine must be one of: 'auto', 'exact', 'residue'")
    if n == 0:
        return 1
    if n == 1:
        return int(matrix[0][0])
    rows = [[int(x) for x in row] for row in matrix]
    fits_int64 = all(-(1 << 63) <= x < (1 << 63) for row in rows for x in row)
    arr = np.array(rows, dtype=np.int64) if fits_int64 else None
    if engine != "residue" and arr is not None and _lib.exact_supported(arr):
        if verbose:
            print(f"exact GPU engine, order {n}")
        return _lib.exact_permanent(arr, _lib.exact_limbs(arr))
    if engine == "exact":
        raise ValueError("matrix is outside the exact engine's range")
    bound = matrix_permanent_bound(rows)
    primes = residue_plan(bound)
    if verbose:
        print(f"residue GPU engine, {len(primes)} primes")
    if arr is None:
        # entries beyond int64: reduce on the host per prime (exact), then
        # hand each reduced matrix to the residue kernel
        res = [_lib.residues(np.array([[x % p for x in r] for r in rows], dtype=np.int64), [p])[0]
               for p in primes]
    else:
        res = _lib.residues(arr, primes)
    return signed_lift(res, primes, bound)


def schur_residues(n: int, primes: List[int]) -> List[int]:
    omegas = [nth_root_of_unity(n, p) for p in primes]
    return _lib.schur_residues(n, primes, omegas)


def schur_permanent_of_size(n: int, verbose: bool = False, parallel: bool = True,
                            num_threads: int = 0) -> int:
    """Exact perm(S_n) (perm.schur_permanent_of_size / perm.permanent API)."""
    if isinstance(n, bool) or not isinstance(n, Integral):
        raise TypeError("n must be an integer")
    n = int(n)
    if n < 0:
        raise ValueError("n must be non-negative")
    _validate_threads(num_threads)
    if n <= 1:
        return 1
    if n % 2 == 0:
        return 0
    primes, congruence, bound = plan_schur(n)
    res = schur_residues(n, primes) if primes else []
    moduli = list(primes)
    if congruence is not None:
        res.append(congruence[0])
        moduli.append(congruence[1])
    if verbose:
        print(f"perm(S_{n}): {len(primes)} GPU primes, congruence {congruence}")
    value = crt(res, moduli)
    product = 1
    for m in moduli:
        product *= m
    if value > bound:
        value -= product
    return value


permanent = schur_permanent_of_size
