"""CPU oracle — TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the plain-C restatement in oracle_perm.c, each
function citing the rivin-perm lines it follows) and, when present, the
reference's own extensions compiled into ``oracle/_ref/`` by
``oracle/build_ref.sh``.  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use this module; the GPU product path never
imports it.

Parity of the restatement is pinned in tests/test_oracle_pins.py against
the golden vectors under tests/golden/ (generated from the reference by
tests/golden/make_golden.py) and, when oracle/_ref exists, against the
reference extensions directly.
"""

from __future__ import annotations

import ctypes
import importlib
import math
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "oracle_perm.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=gnu99",
               str(src), "-o", str(LIB), "-lm"]
        tmp = HERE / ".tmp"           # the compiler's temporary files stay here
        tmp.mkdir(exist_ok=True)
        subprocess.run(cmd, check=True, env=dict(os.environ, TMPDIR=str(tmp)))
    return LIB


def load():
    global _lib
    if _lib is None:
        build()      # no-op unless the library is missing or older than its source
        lib = ctypes.CDLL(str(LIB))
        i64p = ctypes.POINTER(ctypes.c_int64)
        f64p = ctypes.POINTER(ctypes.c_double)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        lib.or_permanent_mod_p.argtypes = [i64p, ctypes.c_int, ctypes.c_int64, ctypes.c_int]
        lib.or_permanent_mod_p.restype = ctypes.c_int64
        lib.or_glynn_mod_p.argtypes = [i64p, ctypes.c_int, ctypes.c_int64, ctypes.c_int]
        lib.or_glynn_mod_p.restype = ctypes.c_int64
        lib.or_ryser_mod_p.argtypes = [i64p, ctypes.c_int, ctypes.c_int64, ctypes.c_int]
        lib.or_ryser_mod_p.restype = ctypes.c_int64
        lib.or_schur_mod_p.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
        lib.or_schur_mod_p.restype = ctypes.c_int64
        lib.or_binary_mod_p.argtypes = [u8p, ctypes.c_int, ctypes.c_int64, ctypes.c_int]
        lib.or_binary_mod_p.restype = ctypes.c_int64
        lib.or_glynn_f64.argtypes = [f64p, ctypes.c_int, ctypes.c_int, f64p]
        lib.or_glynn_f64.restype = ctypes.c_double
        lib.or_glynn_f64_grad.argtypes = [f64p, ctypes.c_int, ctypes.c_int, f64p]
        lib.or_glynn_f64_grad.restype = None
        lib.or_glynn_range_mod_p.argtypes = [i64p, ctypes.c_int, ctypes.c_int64,
                                             ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        lib.or_glynn_range_mod_p.restype = ctypes.c_int64
        lib.or_glynn_c64.argtypes = [f64p, f64p, ctypes.c_int, f64p, f64p, f64p]
        lib.or_glynn_c64.restype = None
        lib.or_max_threads.argtypes = []
        lib.or_max_threads.restype = ctypes.c_int
        lib.or_mod3_range.argtypes = [i64p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                      ctypes.c_int]
        lib.or_mod3_range.restype = ctypes.c_int
        lib.or_permanent_mod3.argtypes = [i64p, ctypes.c_int, ctypes.c_int]
        lib.or_permanent_mod3.restype = ctypes.c_int
        lib.or_affine_mod_p.argtypes = [i64p, i64p, ctypes.c_int, ctypes.c_int64, ctypes.c_int, i64p]
        lib.or_affine_mod_p.restype = ctypes.c_int
        lib.or_affine_range_mod_p.argtypes = [i64p, i64p, ctypes.c_int, ctypes.c_int64,
                                              ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, i64p]
        lib.or_affine_range_mod_p.restype = ctypes.c_int
        _lib = lib
    return _lib


def max_threads() -> int:
    return int(load().or_max_threads())


def _i64(matrix) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(matrix, dtype=np.int64).reshape(len(matrix), len(matrix)) if len(matrix) else np.zeros((0, 0), np.int64))


def permanent_mod_p(matrix, p: int, threads: int = 1) -> int:
    """perm_c_ext.permanent_mod_p semantics for int64 entries and 1 <= p < 2^63."""
    a = _i64(matrix)
    r = load().or_permanent_mod_p(a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                  a.shape[0], int(p), int(threads))
    if r < 0:
        raise RuntimeError("oracle failed")
    return int(r)


def glynn_range_mod_p(matrix, p: int, lo: int, hi: int, threads: int = 0) -> int:
    """Unscaled Glynn partial sum over Gray states [lo, hi) mod odd p."""
    a = _i64(matrix)
    r = load().or_glynn_range_mod_p(a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                    a.shape[0], int(p), int(lo), int(hi),
                                    int(threads or max_threads()))
    if r < 0:
        raise RuntimeError("oracle failed")
    return int(r)


def reference_prime_count(matrix) -> int:
    """Number of CRT primes the reference plan (ascending from 2^30,
    perm.py:1116-1128) uses for this matrix."""
    bound = 1
    for r in matrix:
        bound *= max(1, sum(abs(int(x)) for x in r))
    target, count, prod, c = 2 * bound + 1, 0, 1, 1 << 30
    while prod < target:
        if _is_prime(c):
            count += 1
            prod *= c
        c += 1
    return count


def schur_mod_p(n: int, omega: int, p: int, threads: int = 1) -> int:
    r = load().or_schur_mod_p(int(n), int(omega), int(p), int(threads))
    if r < 0:
        raise RuntimeError("oracle failed")
    return int(r)


def binary_mod_p(matrix, p: int, threads: int = 1) -> int:
    a = np.ascontiguousarray(np.asarray(matrix, dtype=np.uint8))
    n = a.shape[0] if a.ndim == 2 else 0
    r = load().or_binary_mod_p(a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), n,
                               int(p), int(threads))
    if r < 0:
        raise RuntimeError("oracle failed")
    return int(r)


def _is_prime(n: int) -> bool:
    if n < 2:
        return False
    for q in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        if n % q == 0:
            return n == q
    d, r = n - 1, 0
    while d % 2 == 0:
        d //= 2
        r += 1
    for a in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(r - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def exact_permanent(matrix, threads: int = 0) -> int:
    """Exact integer permanent by CRT over oracle residues (perm.py:1076-1212:
    bound, ascending primes from 2^30, Garner, sign rule)."""
    rows = [[int(x) for x in r] for r in matrix]
    n = len(rows)
    if n == 0:
        return 1
    if n == 1:
        return rows[0][0]
    threads = threads or max_threads()
    bound = 1
    for r in rows:
        bound *= max(1, sum(abs(x) for x in r))
    target, primes, prod, c = 2 * bound + 1, [], 1, 1 << 30
    while prod < target:
        if _is_prime(c):
            primes.append(c)
            prod *= c
        c += 1
    res = [permanent_mod_p(rows, p, threads) for p in primes]
    x, m = res[0], primes[0]
    for r, p in zip(res[1:], primes[1:]):
        x += m * ((r - x) * pow(m, -1, p) % p)
        m *= p
    return x - prod if x > bound else x


def glynn_f64(matrix, threads: int = 0):
    """(per, 2^(1-n) * sum |terms|) in FP64 with Kahan summation."""
    a = np.ascontiguousarray(np.asarray(matrix, dtype=np.float64))
    n = a.shape[0] if a.ndim == 2 else 0
    s = ctypes.c_double()
    v = load().or_glynn_f64(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n,
                            int(threads or max_threads()), ctypes.byref(s))
    return float(v), float(s.value)


def glynn_c64(matrix):
    """(per, 2^(1-n) * sum |terms|) of a complex matrix, FP64 Kahan."""
    a = np.asarray(matrix, dtype=np.complex128)
    re = np.ascontiguousarray(a.real)
    im = np.ascontiguousarray(a.imag)
    n = a.shape[0] if a.ndim == 2 else 0
    pr, pi, s = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    p = lambda x: x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    load().or_glynn_c64(p(re), p(im), n, ctypes.byref(pr), ctypes.byref(pi), ctypes.byref(s))
    return complex(pr.value, pi.value), s.value


def glynn_f64_grad(matrix, threads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(matrix, dtype=np.float64))
    n = a.shape[0]
    g = np.zeros((n, n), dtype=np.float64)
    load().or_glynn_f64_grad(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n,
                             int(threads or max_threads()),
                             g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return g


def affine_mod_p(constant, linear, p: int, threads: int = 0) -> list[int]:
    """Coefficients of per(C + x L) mod odd p, ascending degree (n + 1 of
    them) — the fixed-sign Glynn of perm_polynomial.py:268-329."""
    c = _i64(constant)
    l = _i64(linear)
    n = c.shape[0] if c.ndim == 2 else 0
    out = np.zeros(n + 1, dtype=np.int64)
    p64 = ctypes.POINTER(ctypes.c_int64)
    st = load().or_affine_mod_p(c.ctypes.data_as(p64), l.ctypes.data_as(p64), n, int(p),
                                int(threads or max_threads()), out.ctypes.data_as(p64))
    if st != 0:
        raise RuntimeError("oracle failed")
    return [int(x) for x in out]


def permanent_mod3(matrix, threads: int = 0) -> int:
    """per(A) mod 3 by the bit-sliced F_3 Ryser walk (perm_mod3_omp.c)."""
    a = _i64(matrix)
    n = a.shape[0] if a.ndim == 2 else 0
    return int(load().or_permanent_mod3(a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n,
                                        int(threads or max_threads())))


def mod3_range(matrix, lo: int, hi: int, threads: int = 0) -> int:
    """Partial bit-sliced Ryser sum over subsets [lo, hi), as a count mod 3."""
    a = _i64(matrix)
    return int(load().or_mod3_range(a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                    a.shape[0], int(lo), int(hi), int(threads or max_threads())))


def affine_range_mod_p(constant, linear, p: int, lo: int, hi: int, threads: int = 0) -> list[int]:
    """Unscaled partial coefficient sums over Gray states [lo, hi) mod odd p."""
    c = _i64(constant)
    l = _i64(linear)
    n = c.shape[0]
    out = np.zeros(n + 1, dtype=np.int64)
    p64 = ctypes.POINTER(ctypes.c_int64)
    st = load().or_affine_range_mod_p(c.ctypes.data_as(p64), l.ctypes.data_as(p64), n, int(p),
                                      int(lo), int(hi), int(threads or max_threads()),
                                      out.ctypes.data_as(p64))
    if st != 0:
        raise RuntimeError("oracle failed")
    return [int(x) for x in out]


def affine_exact(constant, linear, threads: int = 0) -> list[int]:
    """Exact coefficients of per(C + x L) by CRT over oracle residues
    (bound: coefficients of prod_i (sum_j |c_ij| + x sum_j |l_ij|))."""
    c = [[int(x) for x in r] for r in constant]
    l = [[int(x) for x in r] for r in linear]
    n = len(c)
    if n == 0:
        return [1]
    bound = [1]
    for i in range(n):
        a, b = sum(abs(x) for x in c[i]), sum(abs(x) for x in l[i])
        bound = [(bound[k] if k < len(bound) else 0) * a + (bound[k - 1] * b if k else 0)
                 for k in range(len(bound) + 1)]
    target, primes, prod, q = 2 * max(bound) + 1, [], 1, (1 << 31) - 1
    while prod < target:
        if _is_prime(q):
            primes.append(q)
            prod *= q
        q -= 2
    res = [affine_mod_p(c, l, q, threads) for q in primes]
    out = []
    for k in range(n + 1):
        x, m = res[0][k], primes[0]
        for r, q in zip(res[1:], primes[1:]):
            x += m * ((r[k] - x) * pow(m, -1, q) % q)
            m *= q
        out.append(x - prod if x > prod // 2 else x)
    return out


def reference_modules():
    """(perm_c_ext, perm_binary_ext) compiled from the reference sources, or
    (None, None) when oracle/_ref was not built (e.g. on a machine without
    the reference checkout)."""
    if not REF_DIR.exists():
        return None, None
    sys.path.insert(0, str(REF_DIR))
    try:
        c = importlib.import_module("perm_c_ext")
        b = importlib.import_module("perm_binary_ext")
        return c, b
    except ImportError:
        return None, None
    finally:
        sys.path.remove(str(REF_DIR))
