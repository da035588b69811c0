"""GPU parity of the affine-polynomial engine (pg_affine_residues) and the
polynomial API built on it: coefficient residues bit-exact against the
oracle, exact vectors against the reference's perm_polynomial results, and
full-size identities."""

import math

import numpy as np
import pytest

import oracle
from conftest import golden

pytestmark = pytest.mark.gpu

MODULI = [3, 9, 15, 1_000_003, 536_870_909, 1_073_741_789]   # odd, some composite


@pytest.mark.parametrize("n", list(range(2, 21)))
def test_residues_match_oracle(lib, n):
    rng = np.random.default_rng(900 + n)
    c = rng.integers(-(1 << 40), 1 << 40, (n, n))
    l = rng.integers(-9, 10, (n, n))
    got = lib.affine_residues(c, l, MODULI)
    for m, row in zip(MODULI, got):
        assert row == oracle.affine_mod_p(c, l, m), (n, m)


@pytest.mark.parametrize("n", [2, 3, 5, 8, 13, 19, 20, 22])
def test_equal_row_kernel_matches_oracle(lib, n):
    # C with equal rows (all ones, or one random row repeated) takes the
    # uniform kernel: elementary symmetric sums of the L row sums weighted
    # by powers of the common C row sum
    rng = np.random.default_rng(950 + n)
    l = rng.integers(-9, 10, (n, n))
    for c in (np.ones((n, n), dtype=np.int64),
              np.tile(rng.integers(-(1 << 40), 1 << 40, n), (n, 1))):
        got = lib.affine_residues(c, l, MODULI)
        for m, row in zip(MODULI, got):
            assert row == oracle.affine_mod_p(c, l, m), (n, m)
    # one differing entry sends the matrix back to the general kernel
    c = np.ones((n, n), dtype=np.int64)
    c[n - 1, 0] = 2
    got = lib.affine_residues(c, l, MODULI)
    for m, row in zip(MODULI, got):
        assert row == oracle.affine_mod_p(c, l, m), (n, m)


def test_exact_vectors_match_reference():
    import permgpu
    data = golden("poly.json")
    for c in data["affine"]:
        assert permgpu.affine_permanent(c["constant"], c["linear"]) == \
            tuple(int(v) for v in c["exact"])
        for m, want in zip(c["moduli"], c["residues"]):
            assert permgpu.affine_permanent_mod(c["constant"], c["linear"], m) == tuple(want)
    for c in data["principal"]:
        assert permgpu.principal_permanent_polynomial(c["matrix"]) == \
            tuple(int(v) for v in c["exact"])
        assert permgpu.principal_permanent_polynomial_mod(c["matrix"], 1_000_003) == \
            tuple(c["mod_1000003"])
    for c in data["rook"]:
        assert permgpu.rook_polynomial(c["matrix"]) == tuple(int(v) for v in c["rook"])
    for c in data["weighted_rook"]:
        assert permgpu.weighted_rook_polynomial(c["matrix"]) == tuple(int(v) for v in c["rook"])


@pytest.mark.parametrize("n", [6, 17, 24])
def test_rook_polynomial_of_all_ones(n):
    import permgpu
    want = tuple(math.comb(n, k) ** 2 * math.factorial(k) for k in range(n + 1))
    assert permgpu.rook_polynomial([[1] * n for _ in range(n)]) == want


def test_full_size_rook_identities():
    # 28x28 Bernoulli(0.5): r_1 = number of ones, r_n = per(A) from the
    # exact engine, sum_k r_k (n-k)! = per(J + A) ... checked through the
    # top and bottom coefficients
    import permgpu
    a = (np.random.default_rng(28).random((28, 28)) < 0.5).astype(int)
    r = permgpu.rook_polynomial(a.tolist())
    assert r[0] == 1 and r[1] == int(a.sum())
    assert r[28] == permgpu.binary_permanent(a.tolist())


def test_principal_polynomial_identities():
    import permgpu
    n = 22
    # per(I + x I) = (1 + x)^n
    eye = [[int(i == j) for j in range(n)] for i in range(n)]
    assert permgpu.principal_permanent_polynomial(eye) == \
        tuple(math.comb(n, k) for k in range(n + 1))
    # top coefficient of per(I + x A) is per(A)
    a = np.random.default_rng(22).integers(-3, 4, (n, n))
    top = permgpu.principal_permanent_polynomial(a.tolist())[-1]
    assert top == permgpu.matrix_permanent(a.tolist())


def test_wide_modulus_goes_through_the_exact_vector():
    import permgpu
    rng = np.random.default_rng(17)
    c = rng.integers(-5, 6, (12, 12)).tolist()
    l = rng.integers(-5, 6, (12, 12)).tolist()
    exact = permgpu.affine_permanent(c, l)
    for m in (3_037_000_501, (1 << 63) - 1):
        assert permgpu.affine_permanent_mod(c, l, m) == tuple(v % m for v in exact)


@pytest.mark.parametrize("n", [3, 9, 20, 33])
def test_window_kernel_whole_walks_vs_oracle(lib, n):
    # the shared-memory kernel (orders above 32 and every window) over whole
    # walks at small orders, and over a window at 33, against the oracle
    rng = np.random.default_rng(970 + n)
    c = rng.integers(-(1 << 40), 1 << 40, (n, n))
    l = rng.integers(-9, 10, (n, n))
    states = 1 << (n - 1)
    lo, hi = (0, states) if n <= 20 else (states // 3 & ~63, (states // 3 & ~63) + (1 << 16))
    got = lib.affine_residues_partial(c, l, lo, hi, MODULI)
    for m, row in zip(MODULI, got):
        assert row == oracle.affine_range_mod_p(c, l, m, lo, hi), (n, m)


@pytest.mark.parametrize("n", [34, 40, 63])
def test_windows_at_large_orders(lib, n):
    # the reference accepts orders below 64 (perm_polynomial.py:151); whole
    # walks at these orders take hours per modulus, so windows of 2^16
    # states at the start, the middle and the end are checked against the
    # oracle's window sums, for a general C and for C = J (rook form)
    rng = np.random.default_rng(990 + n)
    l = (rng.random((n, n)) < 0.5).astype(np.int64)
    states, w = 1 << (n - 1), 1 << 16
    for c in (rng.integers(-5, 6, (n, n)), np.ones((n, n), dtype=np.int64)):
        for lo in (0, states // 2 + (1 << 20), states - w):
            got = lib.affine_residues_partial(c, l, lo, lo + w, MODULI[3:])
            for m, row in zip(MODULI[3:], got):
                assert row == oracle.affine_range_mod_p(c, l, m, lo, lo + w), (n, lo, m)


def test_rook_polynomial_order_34_whole_walk(lib):
    # one whole 2^33-state evaluation above the register kernels' range: the
    # exact rook polynomial of a sparse 34 x 34 0/1 matrix (the reference's
    # rook_polynomial, perm_polynomial.py:1288-1411, accepts any order below
    # 64), checked by identities that need no polynomial oracle: r_0 = 1,
    # r_1 = number of ones, r_34 = per(A) from the exact engine, and
    # sum_k r_k (34-k)! t^k = per(J + tA) for t = 1, 2 from the exact engine
    import permgpu
    rng = np.random.default_rng(3434)
    n = 34
    a = (rng.random((n, n)) < 0.15).astype(np.int64)
    np.fill_diagonal(a, 1)
    r = permgpu.rook_polynomial(a.tolist())
    assert len(r) == n + 1
    assert r[0] == 1 and r[1] == int(a.sum())
    assert r[n] == lib.exact_permanent(a, lib.exact_limbs(a))
    for t in (1, 2):
        m = np.ones((n, n), dtype=np.int64) + t * a
        want = lib.exact_permanent(m, lib.exact_limbs(m))
        assert sum(rk * math.factorial(n - k) * t ** k for k, rk in enumerate(r)) == want
