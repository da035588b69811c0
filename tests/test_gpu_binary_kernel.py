"""GPU parity of the bit-sliced 0/1 kernel (binary_glynn.cuh) that the exact
engine runs for 0/1 matrices of order 24..48 with few surviving states.

Doubling one row of a 0/1 matrix doubles its permanent and sends it to the
general exact kernel (entries no longer 0/1), which is pinned to the
reference's exact values; the 0/1 kernel's result must equal half of it for
every order, density, number of offset planes K (half-degrees up to 3, 7,
15, 31), tracking width (up to 32 and up to 64 even-degree rows) and
row-group size the host can pick.  Zero rows, permutation matrices and
all-ones blocks check the edges of the zero-row test and the host's choice
between the two kernels.
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


def _planes(lib, a):
    plan = lib.ExactPlan(a)
    k = plan.bit_planes
    plan.close()
    return k


def _even_rows(n, degree, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros((n, n), dtype=np.int64)
    for i in range(n):
        a[i, rng.choice(n, size=degree, replace=False)] = 1
    return a


@pytest.mark.parametrize("n,density", [(24, 0.5), (25, 0.3), (28, 0.5), (30, 0.15), (31, 0.7),
                                       (32, 0.5), (33, 0.5), (36, 0.2), (37, 0.5)])
def test_binary_kernel_matches_general_kernel(lib, n, density):
    rng = np.random.default_rng(int(1000 * density) + n)
    a = (rng.random((n, n)) < density).astype(np.int64)
    if density == 0.5:
        assert _planes(lib, a) >= 2          # dense random 0/1: the 0/1 kernel runs
    assert _exact(lib, a) == _via_general_kernel(lib, a)


@pytest.mark.parametrize("degree,planes", [(6, 2), (14, 3), (22, 4)])
def test_every_offset_plane_count(lib, degree, planes):
    # all rows of one even degree at order 30: K = smallest with 2^K > degree/2
    a = _even_rows(30, degree, degree)
    assert _planes(lib, a) == planes
    assert _exact(lib, a) == _via_general_kernel(lib, a)


def test_five_planes_and_two_tracking_words_order_48(lib):
    # 48 even rows of degree 32 (K = 5, more than 32 tracked rows: two
    # words; about 1/8 of the states survive); 2^22-state windows keep it
    # short, against the general kernel's windows on the row-doubled matrix
    from permgpu import shard
    a = _even_rows(48, 32, 48)
    assert _planes(lib, a) == 5
    b = a.copy()
    b[0] *= 2
    for lo in (0, 1 << 30, (1 << 47) - (1 << 22)):
        v = shard.words_value(shard.exact_partial_words(a, lo, lo + (1 << 22)))
        w = shard.words_value(shard.exact_partial_words(b, lo, lo + (1 << 22)))
        assert 2 * v == w


def test_windows_on_and_off_the_group_grid(lib):
    # a window whose first chunk is a multiple of 32 runs the split
    # evaluation with chunk groups taken from a counter; one that starts
    # three chunks later runs without the split, dealt round-robin; both
    # against the general kernel's windows on the row-doubled matrix
    from permgpu import shard
    a = (np.random.default_rng(411).random((40, 40)) < 0.5).astype(np.int64)
    assert _planes(lib, a) >= 2
    b = a.copy()
    b[0] *= 2
    for lo in (1 << 30, (1 << 30) + 3 * (1 << 10), (1 << 38) + 5 * (1 << 10)):
        hi = lo + (1 << 22) + 7 * (1 << 10)
        v = shard.words_value(shard.exact_partial_words(a, lo, hi))
        w = shard.words_value(shard.exact_partial_words(b, lo, hi))
        assert 2 * v == w


def test_zero_rows_permutations_and_ones(lib):
    n = 26
    rng = np.random.default_rng(26)
    a = (rng.random((n, n)) < 0.5).astype(np.int64)
    a[5] = 0                                             # a zero row
    assert _exact(lib, a) == 0
    p = np.eye(n, dtype=np.int64)[rng.permutation(n)]    # odd degrees: general kernel
    assert _planes(lib, p) == 0
    assert _exact(lib, p) == 1
    j = np.ones((n, n), dtype=np.int64)                  # equal rows: most states survive
    assert _planes(lib, j) == 0
    assert _exact(lib, j) == math.factorial(n)
    blocks = np.kron(np.eye(2, dtype=np.int64), np.ones((14, 14), dtype=np.int64))
    assert _exact(lib, blocks) == math.factorial(14) ** 2
    sparse = _even_rows(40, 4, 4)                        # K = 2, nearly every state zero
    assert _planes(lib, sparse) == 2
    assert _exact(lib, sparse) == _via_general_kernel(lib, sparse)
