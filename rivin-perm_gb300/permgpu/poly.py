"""Polynomial permanents on the GPU.

The public functions of rivin-perm's ``perm_polynomial.py`` with the same
signatures, validation, results and errors:

  affine_permanent_bounds(C, L)               perm_polynomial.py:883-895
  affine_permanent_mod(C, L, m)               perm_polynomial.py:1086-1115
  affine_permanent(C, L)                      perm_polynomial.py:1183-1214
  principal_permanent_polynomial_mod(A, m)    perm_polynomial.py:1217-1250
  principal_permanent_polynomial(A)           perm_polynomial.py:1253-1285
  rook_polynomial(A)                          perm_polynomial.py:1288-1411
  weighted_rook_polynomial(A)                 perm_polynomial.py:1512-1606

Every residue comes from ``pg_affine_residues`` (coefficients of
per(C + x L) modulo odd moduli below 2^30, all moduli in one launch).
Exact coefficient vectors are reconstructed by CRT over descending primes
below 2^30 covering the certified coefficientwise bound (the reference's
bound, restated), and the reconstruction is checked against that bound.
Rook polynomials are per(J + x A) divided coefficientwise by (n - k)!.
There is no CPU path: without a GPU the calls raise.
"""

from __future__ import annotations

import math
import operator
from typing import List, Sequence, Tuple

import numpy as np

from . import _lib
from .crt import is_prime

_INT64_MAX = (1 << 63) - 1
_INT32_MAX = (1 << 31) - 1
# largest odd modulus the affine kernel takes (lazy sums stay below p * 2^32)
GPU_MODULUS_LIMIT = 1 << 30
GPU_MAX_ORDER = 63

Matrix = Tuple[Tuple[int, ...], ...]


# ---- validation (perm_polynomial.py:98-232 contracts) ---------------------

def _validate_modulus(modulus) -> int:
    try:
        value = operator.index(modulus)
    except TypeError as exc:
        raise TypeError("modulus must be an integer") from exc
    if isinstance(modulus, bool):
        raise TypeError("modulus must be an integer")
    value = int(value)
    if value <= 1 or value % 2 == 0:
        raise ValueError("modulus must be an odd integer greater than 1")
    if value > _INT64_MAX:
        raise ValueError("modulus must fit in a positive signed 64-bit integer")
    return value


def _validate_num_threads(num_threads) -> int:
    try:
        value = operator.index(num_threads)
    except TypeError as exc:
        raise TypeError("num_threads must be an integer") from exc
    if isinstance(num_threads, bool):
        raise TypeError("num_threads must be an integer")
    value = int(value)
    if value < 0:
        raise ValueError("num_threads must be non-negative")
    if value > _INT32_MAX:
        raise ValueError("num_threads is too large")
    return value


def _validate_backend(backend) -> None:
    # "auto" and "native" both mean the GPU engine; there is no Python
    # fallback path to select
    if backend not in ("auto", "native"):
        raise ValueError("backend must be 'auto' or 'native' (GPU engine)")


def _validate_parallel(parallel) -> None:
    if not isinstance(parallel, bool):
        raise TypeError("parallel must be a boolean")


def _snapshot_integer_matrix(matrix, name: str) -> Matrix:
    declared_shape = getattr(matrix, "shape", None)
    if declared_shape is not None:
        try:
            declared_shape = tuple(declared_shape)
        except TypeError as exc:
            raise ValueError(f"{name} must have a two-dimensional square shape") from exc
        if len(declared_shape) != 2:
            raise ValueError(f"{name} must be two-dimensional")
        if declared_shape[0] != declared_shape[1]:
            raise ValueError(f"{name} must be square")
    try:
        order = len(matrix)
    except TypeError as exc:
        raise TypeError(f"{name} must be a sequence of rows") from exc
    if order >= 64:
        raise ValueError("matrix order must be less than 64")
    rows = []
    for i, row in enumerate(matrix):
        try:
            width = len(row)
        except TypeError as exc:
            raise TypeError(f"{name} rows must be sequences") from exc
        if width != order:
            raise ValueError(f"{name} must be square")
        out = []
        for j, entry in enumerate(row):
            try:
                out.append(int(operator.index(entry)))
            except TypeError as exc:
                raise TypeError(f"{name} entries must be integers; entry ({i}, {j}) is "
                                f"{type(entry).__name__}") from exc
        rows.append(tuple(out))
    return tuple(rows)


def _snapshot_binary_matrix(matrix) -> Matrix:
    m = _snapshot_integer_matrix(matrix, "matrix")
    for i, row in enumerate(m):
        for j, v in enumerate(row):
            if v not in (0, 1):
                raise ValueError(f"matrix entries must be 0 or 1; entry ({i}, {j}) is {v}")
    return m


def _snapshot_nonnegative_matrix(matrix) -> Matrix:
    m = _snapshot_integer_matrix(matrix, "matrix")
    for i, row in enumerate(m):
        for j, v in enumerate(row):
            if v < 0:
                raise ValueError(f"matrix entries must be nonnegative; entry ({i}, {j}) is {v}")
    return m


def _validate_affine(constant, linear) -> Tuple[Matrix, Matrix]:
    c = _snapshot_integer_matrix(constant, "constant_matrix")
    l = _snapshot_integer_matrix(linear, "linear_matrix")
    if len(c) != len(l):
        raise ValueError("constant_matrix and linear_matrix must have the same shape")
    return c, l


def _check_order(n: int) -> None:
    if n > GPU_MAX_ORDER:
        raise ValueError(f"order {n} exceeds the GPU polynomial engine's maximum "
                         f"{GPU_MAX_ORDER}")


# ---- bounds (perm_polynomial.py:573-586, 782-861) --------------------------

def _affine_product(constants: Sequence[int], linears: Sequence[int]) -> List[int]:
    """Coefficients of prod_i (a_i + x b_i), ascending."""
    poly = [1]
    for a, b in zip(constants, linears):
        nxt = [0] * (len(poly) + 1)
        for k, v in enumerate(poly):
            nxt[k] += v * a
            nxt[k + 1] += v * b
        poly = nxt
    return poly


def _bounds(c: Matrix, l: Matrix) -> Tuple[int, ...]:
    """Coefficientwise minimum of four relaxations of per(|C| + x|L|): row
    sums, column sums, and n! times the row / column maxima."""
    n = len(c)
    if n == 0:
        return (1,)
    cols = range(n)
    rc = [sum(abs(v) for v in row) for row in c]
    rl = [sum(abs(v) for v in row) for row in l]
    cc = [sum(abs(c[i][j]) for i in cols) for j in cols]
    cl = [sum(abs(l[i][j]) for i in cols) for j in cols]
    mc = [max(abs(v) for v in row) for row in c]
    ml = [max(abs(v) for v in row) for row in l]
    kc = [max(abs(c[i][j]) for i in cols) for j in cols]
    kl = [max(abs(l[i][j]) for i in cols) for j in cols]
    f = math.factorial(n)
    cands = (_affine_product(rc, rl), _affine_product(cc, cl),
             [f * v for v in _affine_product(mc, ml)], [f * v for v in _affine_product(kc, kl)])
    return tuple(min(vals) for vals in zip(*cands))


def affine_permanent_bounds(constant_matrix, linear_matrix) -> Tuple[int, ...]:
    """Certified absolute bounds for the coefficients of per(C + x L),
    ascending degree, order + 1 entries."""
    c, l = _validate_affine(constant_matrix, linear_matrix)
    return _bounds(c, l)


# ---- residues and CRT ----------------------------------------------------

def _gpu_primes(target: int) -> List[int]:
    """Descending primes below 2^30 whose product exceeds target."""
    primes, prod, q = [], 1, GPU_MODULUS_LIMIT - 1
    while prod <= target:
        if q < 3:
            raise RuntimeError("exhausted the CRT prime range")
        if is_prime(q):
            primes.append(q)
            prod *= q
        q -= 2
    return primes


def _fits_int64(m: Matrix) -> bool:
    return all(-(1 << 63) <= v <= _INT64_MAX for row in m for v in row)


def _residues(c: Matrix, l: Matrix, moduli: Sequence[int]) -> List[List[int]]:
    """Coefficient residues for every modulus (odd, < 2^30)."""
    n = len(c)
    if _fits_int64(c) and _fits_int64(l):
        return _lib.affine_residues(np.array(c, dtype=np.int64).reshape(n, n),
                                    np.array(l, dtype=np.int64).reshape(n, n), moduli)
    out = []
    for m in moduli:   # entries beyond int64: reduce per modulus first
        cr = np.array([[v % m for v in row] for row in c], dtype=np.int64).reshape(n, n)
        lr = np.array([[v % m for v in row] for row in l], dtype=np.int64).reshape(n, n)
        out.extend(_lib.affine_residues(cr, lr, [m]))
    return out


def _exact(c: Matrix, l: Matrix) -> Tuple[int, ...]:
    n = len(c)
    if n == 0:
        return (1,)
    if n == 1:
        return (c[0][0], l[0][0])
    _check_order(n)
    bounds = _bounds(c, l)
    top = max(bounds)
    if top == 0:
        return (0,) * (n + 1)
    nonneg = all(v >= 0 for m in (c, l) for row in m for v in row)
    primes = _gpu_primes(top if nonneg else 2 * top)
    res = _residues(c, l, primes)
    vals, mod = list(res[0]), primes[0]
    for r, q in zip(res[1:], primes[1:]):
        inv = pow(mod % q, -1, q)
        for d in range(n + 1):
            vals[d] += mod * ((r[d] - vals[d]) * inv % q)
        mod *= q
    if nonneg:
        exact = tuple(vals)
        ok = all(0 <= v <= b for v, b in zip(exact, bounds))
    else:
        exact = tuple(v - mod if v > mod // 2 else v for v in vals)
        ok = all(abs(v) <= b for v, b in zip(exact, bounds))
    if not ok:
        raise RuntimeError("CRT reconstruction lies outside its certified coefficient bound")
    return exact


def _mod(c: Matrix, l: Matrix, modulus: int) -> Tuple[int, ...]:
    n = len(c)
    cr = tuple(tuple(v % modulus for v in row) for row in c)
    lr = tuple(tuple(v % modulus for v in row) for row in l)
    if n == 0:
        return (1 % modulus,)
    if n == 1:
        return (cr[0][0], lr[0][0])
    _check_order(n)
    if modulus < GPU_MODULUS_LIMIT:
        return tuple(_residues(cr, lr, [modulus])[0])
    # wide modulus: the exact polynomial of the reduced matrices, reduced
    return tuple(v % modulus for v in _exact(cr, lr))


# ---- public API ------------------------------------------------------------

def affine_permanent_mod(constant_matrix, linear_matrix, modulus: int, *,
                         backend: str = "auto", parallel: bool = True,
                         num_threads: int = 0) -> Tuple[int, ...]:
    """Coefficients of per(C + x L) modulo an odd modulus (need not be
    prime), canonical residues in ascending degree, order + 1 entries."""
    modulus = _validate_modulus(modulus)
    _validate_parallel(parallel)
    _validate_num_threads(num_threads)
    _validate_backend(backend)
    c, l = _validate_affine(constant_matrix, linear_matrix)
    return _mod(c, l, modulus)


def affine_permanent(constant_matrix, linear_matrix, *, backend: str = "auto",
                     parallel: bool = True, num_threads: int = 0) -> Tuple[int, ...]:
    """Exact integer coefficients of per(C + x L), ascending degree, order + 1
    entries; the empty permanent is (1,)."""
    _validate_parallel(parallel)
    _validate_num_threads(num_threads)
    _validate_backend(backend)
    c, l = _validate_affine(constant_matrix, linear_matrix)
    return _exact(c, l)


def _identity(n: int) -> Matrix:
    return tuple(tuple(int(i == j) for j in range(n)) for i in range(n))


def principal_permanent_polynomial_mod(matrix, modulus: int, *, backend: str = "auto",
                                       parallel: bool = True,
                                       num_threads: int = 0) -> Tuple[int, ...]:
    """Coefficients of per(I + x A) mod an odd modulus: entry k is the sum
    of per(A[S, S]) over index sets of size k."""
    modulus = _validate_modulus(modulus)
    _validate_parallel(parallel)
    _validate_num_threads(num_threads)
    _validate_backend(backend)
    a = _snapshot_integer_matrix(matrix, "matrix")
    return _mod(_identity(len(a)), a, modulus)


def principal_permanent_polynomial(matrix, *, backend: str = "auto", parallel: bool = True,
                                   num_threads: int = 0) -> Tuple[int, ...]:
    """Exact coefficients of per(I + x A)."""
    _validate_parallel(parallel)
    _validate_num_threads(num_threads)
    _validate_backend(backend)
    a = _snapshot_integer_matrix(matrix, "matrix")
    return _exact(_identity(len(a)), a)


def _rook_from_affine(a: Matrix) -> Tuple[int, ...]:
    """Weighted matching sums: coefficient k of per(J + x A) is (n-k)! times
    the sum over k-matchings of the products of their entries."""
    n = len(a)
    ones = tuple((1,) * n for _ in range(n))
    coeffs = _exact(ones, a)
    out = []
    for k, v in enumerate(coeffs):
        f = math.factorial(n - k)
        q, r = divmod(v, f)
        if r:
            raise RuntimeError("per(J + xA) coefficient not divisible by (n-k)!")
        out.append(q)
    return tuple(out)


def rook_polynomial(matrix, *, backend: str = "auto", parallel: bool = True,
                    num_threads: int = 0) -> Tuple[int, ...]:
    """Matching counts of a square 0/1 matrix: entry k is the number of ways
    to choose k one-entries with no shared row or column (order + 1 entries,
    ascending; the empty matrix gives (1,))."""
    _validate_parallel(parallel)
    _validate_num_threads(num_threads)
    _validate_backend(backend)
    a = _snapshot_binary_matrix(matrix)
    n = len(a)
    if n == 0:
        return (1,)
    if n == 1:
        return (1, a[0][0])
    if not any(any(row) for row in a):
        return (1,) + (0,) * n
    return _rook_from_affine(a)


def weighted_rook_polynomial(matrix, *, backend: str = "auto", parallel: bool = True,
                             num_threads: int = 0) -> Tuple[int, ...]:
    """Weighted matching sums of a square nonnegative integer matrix: entry
    k sums, over all k-matchings, the product of the chosen entries."""
    _validate_parallel(parallel)
    _validate_num_threads(num_threads)
    _validate_backend(backend)
    a = _snapshot_nonnegative_matrix(matrix)
    n = len(a)
    if n == 0:
        return (1,)
    if n == 1:
        return (1, a[0][0])
    if not any(any(row) for row in a):
        return (1,) + (0,) * n
    return _rook_from_affine(a)
