"""GPU parity of the bit-sliced 0/1 kernel (binary_glynn.cuh) that the exact
engine runs for 0/1 matrices of order 24..48.

Doubling one row of a 0/1 matrix doubles its permanent and sends it to the
general exact kernel (entries no longer 0/1), which is pinned to the
reference's exact values; the 0/1 kernel's result must equal half of it for
every order, density, bit-plane count (maximum degree 7, 15, 31, 63) and
row-group size the host can pick.  Zero rows, permutation matrices and
all-ones blocks check the zero-row test at its edges.
"""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _exact(lib, a):
    return lib.exact_permanent(a, lib.exact_limbs(a))


def _via_general_kernel(lib, a):
    b = a.copy()
    b[0] *= 2
    return _exact(lib, b) // 2


@pytest.mark.parametrize("n,density", [(24, 0.5), (25, 0.3), (28, 0.5), (30, 0.15), (31, 0.7),
                                       (32, 0.5), (33, 0.5), (36, 0.2), (37, 0.5)])
def test_binary_kernel_matches_general_kernel(lib, n, density):
    rng = np.random.default_rng(int(1000 * density) + n)
    a = (rng.random((n, n)) < density).astype(np.int64)
    plan = lib.ExactPlan(a)
    assert plan.bit_planes >= 3
    plan.close()
    assert _exact(lib, a) == _via_general_kernel(lib, a)


@pytest.mark.parametrize("maxdeg", [7, 15, 31])
def test_every_bit_plane_count(lib, maxdeg):
    # rows of degree up to maxdeg (3, 4, 5 planes) at order 30
    n = 30
    rng = np.random.default_rng(maxdeg)
    a = np.zeros((n, n), dtype=np.int64)
    for i in range(n):
        d = int(rng.integers(1, maxdeg + 1)) if i else maxdeg
        a[i, rng.choice(n, size=min(d, n), replace=False)] = 1
    plan = lib.ExactPlan(a)
    want_planes = max(3, int(a.sum(1).max()).bit_length())
    assert plan.bit_planes == want_planes
    plan.close()
    assert _exact(lib, a) == _via_general_kernel(lib, a)


def test_six_planes_dense_order_40(lib):
    # degrees near 36 need 6 planes; a 2^22-state window keeps it short,
    # against the general kernel's window on the row-doubled matrix
    from permgpu import shard
    n = 40
    a = (np.random.default_rng(40).random((n, n)) < 0.9).astype(np.int64)
    plan = lib.ExactPlan(a)
    assert plan.bit_planes == 6
    plan.close()
    b = a.copy()
    b[0] *= 2
    for lo in (0, 1 << 30, (1 << 39) - (1 << 22)):
        v = shard.words_value(shard.exact_partial_words(a, lo, lo + (1 << 22)))
        w = shard.words_value(shard.exact_partial_words(b, lo, lo + (1 << 22)))
        assert 2 * v == w


def test_zero_rows_permutations_and_ones(lib):
    n = 26
    rng = np.random.default_rng(26)
    a = (rng.random((n, n)) < 0.5).astype(np.int64)
    a[5] = 0                                             # a zero row
    assert _exact(lib, a) == 0
    p = np.eye(n, dtype=np.int64)[rng.permutation(n)]    # a permutation matrix
    assert _exact(lib, p) == 1
    j = np.ones((n, n), dtype=np.int64)                  # every row even: n!
    assert _exact(lib, j) == math.factorial(n)
    j25 = np.ones((25, 25), dtype=np.int64)              # odd degrees: no zero row
    assert _exact(lib, j25) == math.factorial(25)
    blocks = np.kron(np.eye(2, dtype=np.int64), np.ones((13, 13), dtype=np.int64))
    assert _exact(lib, blocks) == math.factorial(13) ** 2
